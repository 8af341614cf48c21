"""Receiver fixtures of the layered 120^3 workload computed by the reference itself.

The reference (built from its sources by oracle/build_ref.sh) solves the layered
workload of demo_matrixfree_csem_gb300.synthetic.layered_120 - 100^3 core cells of
100 m, nb=10 padding to 120^3, airbc=1, one Ex dipole at (0,0,950), 101 seafloor
receivers, BiCGStab + LU-SGS to tol=1e-8/f - one frequency per process, and this
script stores for each frequency:
  * the receivers in complex128 (the value extract_emf computes before its complex64
    store; the oracle's extraction is bit-identical to it), channels Ex, Ey, Ez;
  * the complex64 values the reference stores in dcal_fd;
  * the relative-residual history the reference prints (iterate_fbicgstab.txt) and the
    iteration count.
Output: tests/golden/layered_120/reference_receivers.npz (a few tens of KB).

FFTW is replaced by the self-written DFT of oracle/fft2d.c (see oracle/ref_stubs), so
the airwave part of these numbers carries that transform's rounding.

    python tests/golden/make_layered_reference.py          # all frequencies, in parallel
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
OUT = os.path.join(HERE, "layered_120", "reference_receivers.npz")


def one(ifreq: int, work: str) -> None:
    from demo_matrixfree_csem_gb300 import synthetic
    from oracle import Ref
    from oracle.pyoracle import Oracle
    cfg = synthetic.layered_120()
    synthetic.write_config(cfg, work)
    os.chdir(work)
    R = Ref(cfg.args(work))
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
    if len(sys.argv) == 3:
        one(int(sys.argv[1]), sys.argv[2])
        return
    from oracle import build_ref, ref_available
    if not ref_available():
        sys.exit("reference sources not found")
    build_ref()
    tmp = tempfile.mkdtemp()
    works = [os.path.join(tmp, f"w{i}") for i in range(3)]
    for w in works:
        os.makedirs(w)
    with cf.ThreadPoolExecutor(3) as ex:
        list(ex.map(lambda i: subprocess.run([sys.executable, __file__, str(i), works[i]], check=True,
                                             stdout=subprocess.DEVNULL), range(3)))
    parts = [np.load(os.path.join(works[i], f"f{i}.npz")) for i in range(3)]
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    np.savez_compressed(OUT, rec=np.stack([p["rec"] for p in parts]), dcal=np.stack([p["dcal"] for p in parts]),
                        freqs=np.array([float(p["freq"]) for p in parts], np.float32),
                        hist0=parts[0]["hist"], hist1=parts[1]["hist"], hist2=parts[2]["hist"],
                        seconds=np.array([float(p["seconds"]) for p in parts]))
    print("wrote", OUT)


if __name__ == "__main__":
    main()
