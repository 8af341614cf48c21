"""Receiver fixtures of whole workloads computed by the reference itself.

The reference (built from its sources by oracle/build_ref.sh) solves a workload of
demo_matrixfree_csem_gb300.synthetic - layered_120 (100^3 core cells of 100 m, nb=10
padding to 120^3, airbc=1, one Ex dipole at (0,0,950), 101 seafloor receivers),
vti_block_120 (the same grid, rho33 = 2 rho11, a 50 ohm-m 2 x 2 x 0.1 km block at
2050 m) or bathymetry_125 (125 x 125 x 100 cells of 100 m under a seafloor of three
Gaussian hills, nb=10, its first source) - with BiCGStab + LU-SGS to tol=1e-8/f, one
frequency per process, and this script stores for each frequency:
  * the receivers in complex128 (the value extract_emf computes before its complex64
    store; the oracle's extraction is bit-identical to it), channels Ex, Ey, Ez;
  * the complex64 values the reference stores in dcal_fd;
  * the relative-residual history the reference prints (iterate_fbicgstab.txt) and the
    iteration count.
Output: tests/golden/<workload>/reference_receivers.npz (a few tens of KB).

FFTW is replaced by the self-written DFT of oracle/fft2d.c (see oracle/ref_stubs), so
the airwave part of these numbers carries that transform's rounding.

With CSEM_REF_VARIANT=fma the reference is built with multiply-add contraction (what its
Makefile's -O3 gives with GCC on aarch64, oracle/build_ref.sh) and the output is
reference_receivers_fma.npz: the same solves from a second, equally valid build of the
reference, which measures how far the reference's receivers move with rounding alone.

    python tests/golden/make_reference_receivers.py [layered_120|vti_block_120|bathymetry_125|marlim_like_96]
    CSEM_REF_VARIANT=fma python tests/golden/make_reference_receivers.py vti_block_120
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
def out_path(workload: str) -> str:
    suffix = "_fma" if os.environ.get("CSEM_REF_VARIANT") == "fma" else ""
    return os.path.join(HERE, workload, f"reference_receivers{suffix}.npz")


def one(workload: str, ifreq: int, work: str) -> None:
    from demo_matrixfree_csem_gb300 import synthetic
    from oracle import Ref
    from oracle.pyoracle import Oracle
    cfg = synthetic.workload(workload)
    synthetic.write_config(cfg, work)
    os.chdir(work)
    R = Ref(cfg.args(work) + ["preco=1", "algopt=1"])  # BiCGStab + LU-SGS, whatever the workload's default
    x, b, t = R.solve(ifreq, verb=1)
    hist = []
    with open("iterate_fbicgstab.txt") as f:
        next(f)
        for line in f:
            hist.append(float(line.split()[1]))
    dcal = R.extract(x, ifreq)[:, ifreq, :]
    O = Oracle(R.grid_arrays())
    rec = O.extract([0, 1, 2], cfg.acq.rec, x)
    np.savez(os.path.join(work, f"f{ifreq}.npz"), rec=rec, dcal=dcal, hist=np.array(hist), seconds=t,
             freq=R.freqs[ifreq])


def main() -> None:
    if len(sys.argv) == 4:
        one(sys.argv[1], int(sys.argv[2]), sys.argv[3])
        return
    workload = sys.argv[1] if len(sys.argv) > 1 else "layered_120"
    OUT = out_path(workload)
    from oracle import build_ref, ref_available
    if not ref_available():
        sys.exit("reference sources not found")
    build_ref()
    os.makedirs(os.path.join(HERE, workload), exist_ok=True)
    from demo_matrixfree_csem_gb300 import synthetic
    nf = len(synthetic.workload(workload).params["freqs"].split(","))  # one process per frequency
    tmp = tempfile.mkdtemp(prefix="_work_", dir=os.path.join(HERE, workload))  # removed at the end
    works = [os.path.join(tmp, f"w{i}") for i in range(nf)]
    for w in works:
        os.makedirs(w)
    with cf.ThreadPoolExecutor(nf) as ex:
        list(ex.map(lambda i: subprocess.run([sys.executable, __file__, workload, str(i), works[i]], check=True,
                                             stdout=subprocess.DEVNULL), range(nf)))
    parts = [np.load(os.path.join(works[i], f"f{i}.npz")) for i in range(nf)]
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    np.savez_compressed(OUT, rec=np.stack([p["rec"] for p in parts]), dcal=np.stack([p["dcal"] for p in parts]),
                        freqs=np.array([float(p["freq"]) for p in parts], np.float32),
                        seconds=np.array([float(p["seconds"]) for p in parts]),
                        **{f"hist{i}": parts[i]["hist"] for i in range(nf)})
    shutil.rmtree(tmp)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
