"""Generate the golden fixtures in tests/golden/ from the reference itself.

The reference (yangpl/demo_matrixfree_csem) is compiled from its own sources with the
link stubs of oracle/ref_stubs (oracle/build_ref.sh) and driven through its public
functions on tiny seeded models. For each case this writes:
  <case>/fx1..3, frho11..33, sources.txt, receivers.txt   the model and acquisition
  <case>/args.json                                        the key=value flags
  <case>/golden.npz                                       the reference's outputs:
      grid arrays (x*, d*, sigma*, airwave filters), a probe vector x (exact dyadic
      values), A x, M^-1 x (LU-SGS or A-phi per case), the injected source b,
      x after `niter` solver iterations, the relative-residual history of that run
      (the value the reference prints), and the receivers it extracts (complex64).

Run where the reference sources exist (CSEM_REFERENCE_DIR, else a sibling directory
"reference" of this repository):
    python tests/golden/make_golden.py
The fixtures are committed; the tests only read them.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from demo_matrixfree_csem_gb300 import synthetic  # noqa: E402

# name -> (seed, random_small kwargs)
CASES = {
    "lusgs_air0": (11, dict(airbc=0, nb=2, preco=1, algopt=1, fvm=0, niter=8)),
    "lusgs_air1": (12, dict(airbc=1, nb=2, preco=1, algopt=1, fvm=0, niter=8, n1fft=16, n2fft=16)),
    "aphi_air0_fvm": (13, dict(airbc=0, nb=2, preco=3, algopt=2, fvm=1, niter=20, nrestart=5)),
    "aphi_air1": (14, dict(airbc=1, nb=2, preco=3, algopt=1, fvm=0, niter=8, n1fft=16, n2fft=16)),
    "plain_gmres_air0": (15, dict(airbc=0, nb=2, preco=0, algopt=2, fvm=0, niter=30, nrestart=6)),
    "plain_bicg_air0": (16, dict(airbc=0, nb=2, preco=0, algopt=1, fvm=0, niter=10)),
    "gmrespre_air0": (17, dict(airbc=0, nb=2, preco=2, algopt=1, fvm=0, niter=4, mp=5)),
}


def probe_vector(n: int, seed: int) -> np.ndarray:
    """Exactly representable pseudo-random complex vector (dyadic rationals)."""
    rng = np.random.default_rng(seed)
    re = rng.integers(-2 ** 20, 2 ** 20, n).astype(np.float64) / 2 ** 20
    im = rng.integers(-2 ** 20, 2 ** 20, n).astype(np.float64) / 2 ** 20
    return re + 1j * im


def run_case(name: str) -> None:
    """Run one case in a fresh process (the reference keeps global state)."""
    from oracle import Ref
    seed, kw = CASES[name]
    d = os.path.join(HERE, name)
    cfg = synthetic.random_small(seed, nx=6, ny=5, nz=5, chsrc="Ex,Ey,Ez", **kw)
    synthetic.write_config(cfg, d)
    args = cfg.args(d)
    rel_args = [a.replace(d + "/", "") for a in args]
    with open(os.path.join(d, "args.json"), "w") as f:
        json.dump(rel_args, f, indent=1)
    cwd = os.getcwd()
    os.chdir(d)
    try:
        R = Ref(rel_args)
        g = R.grid_arrays()
        out = {k: getattr(g, k) for k in ("x1", "x2", "x3", "x1s", "x2s", "x3s", "d1", "d2", "d3",
                                          "d1s", "d2s", "d3s", "sigma11", "sigma22", "sigma33")}
        if g.airbc:
            out.update(sH1=g.sH1, sH2=g.sH2)
        x = probe_vector(R.lE, seed)
        R.set_freq(0)
        out["x"] = x
        out["Ax"] = R.apply(0, x)
        if R.preco == 1:
            out["Mx"] = R.apply(1, x)
        elif R.preco == 3:
            out["Mx"] = R.apply(2, x)
        out["b"] = R.inject()
        R.lib().ref_run_main  # noqa: B018 (symbol presence)
        xs, bs, _ = R.solve(0, verb=1)
        out["x_solve"] = xs
        hist_file = "iterate_fbicgstab.txt" if R.algopt == 1 and R.preco else (
            "iterate_bicgstab.txt" if R.algopt == 1 else ("iterate_fgmres.txt" if R.preco else "iterate_gmres.txt"))
        hist = []
        with open(hist_file) as f:
            next(f)
            for line in f:
                hist.append(float(line.split()[1]))
        os.remove(hist_file)
        out["hist_printed"] = np.array(hist)
        out["dcal"] = R.extract(xs, 0)[:, 0, :]
        out["freqs"] = R.freqs
        out["info"] = np.array([R.n1, R.n2, R.n3, R.nb, R.nx, R.ny, R.nz, R.lE, R.airbc, R.fvm, R.preco,
                                R.algopt, R.niter, R.nrestart, R.mp, R.n1fft, R.n2fft])
        out["rho_water"] = np.array(R.rho_water)
        out["tol"] = np.array(R.tol)
        np.savez_compressed(os.path.join(d, "golden.npz"), **out)
    finally:
        os.chdir(cwd)


def main() -> None:
    from oracle import ref_available
    if not ref_available():
        sys.exit("reference sources not found; nothing generated")
    if len(sys.argv) > 1:
        run_case(sys.argv[1])
        return
    for name in CASES:
        subprocess.run([sys.executable, __file__, name], check=True, stdout=subprocess.DEVNULL)
        print("wrote", name)


if __name__ == "__main__":
    main()
