"""Known answers from the reference for two options around the hot path.

For golden cases (tests/golden/<case>/, made by make_golden.py) the reference, compiled
from its sources (oracle/build_ref.sh), writes:
  <case>/extended/{frho11,frho22,frho33,fx1,fx2,fx3}_extended
      the padded model it exports with param_extended=1 (extend_model.c:254-289);
  <case>/acsr.npz  (cases without airwave)
      Ax_csr = Acsr_apply(x) after Acsr_init (Acsr.c:22-716), the operator assembled in
      CSR, and Mx_csr = Acsr_lusgs_apply(x) (Acsr.c:719-748), the LU-SGS sweeps on the
      assembled rows, for the case's probe vector x at its first frequency.

Probing both the assembled matrix and fdfd_apply column by column on these tiny grids
shows how the two relate. The assembled operator is I*omega*mu0 times the matrix-free
one (curl curl - I*omega*mu0*sigma, Acsr.c, against curl curl / (I*omega*mu0) - sigma,
fdfd.c:86-205) and adds the boundary rows; every off-diagonal coupling of an interior
row agrees to rounding; but Acsr_init stores each row's diagonal term in column
row - 1, with a geometric part that differs from fdfd_apply's own diagonal. So the
assembled operator is not the matrix-free one, and Acsr_lusgs_apply is a different
preconditioner. The fixture therefore also holds, per row, what the known-answer test
needs to compare the off-diagonal couplings only:
      interior   rows fdfd_apply writes (it leaves the boundary rows zero);
      fdfd_diag  fdfd_apply's diagonal entry of each row;
      self_term  the assembled row's column row - 1 contribution to Ax_csr beyond
                 I*omega*mu0 times fdfd_apply's entry there;
      iom        I*omega*mu0 as Acsr_init forms it.

A third fixture pins the reference's Hy scratch length (fdfd.c:59 sizes Hy as
n1*(n2+1)*n2, where n3 is meant): on a model with n2 < n3 the Hy and Hz scratch overlap
and fdfd_apply mixes the two. hy_overlap/ holds that model (case.json: its flags) and
  hy_overlap/fdfd.npz   x, Ax = fdfd_apply(x) and the frequency.

Run where the reference sources exist (CSEM_REFERENCE_DIR, else a sibling directory
"reference" of this repository):
    python tests/golden/make_known_answers.py
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

EXTENDED = ["lusgs_air0", "lusgs_air1"]
ACSR = ["lusgs_air0", "plain_bicg_air0"]
NAMES = ["frho11_extended", "frho22_extended", "frho33_extended", "fx1_extended", "fx2_extended", "fx3_extended"]


def run_case(case: str, what: str) -> None:
    from oracle import Ref
    d = os.path.join(HERE, case)
    args = json.load(open(os.path.join(d, "args.json")))
    gold = np.load(os.path.join(d, "golden.npz"))
    with tempfile.TemporaryDirectory() as t:
        for f in os.listdir(d):
            if not os.path.isdir(os.path.join(d, f)):
                shutil.copy(os.path.join(d, f), t)
        cwd = os.getcwd()
        os.chdir(t)
        try:
            if what == "extended":
                Ref(args + ["param_extended=1", "verb=1"])
                out = os.path.join(d, "extended")
                os.makedirs(out, exist_ok=True)
                for n in NAMES:
                    shutil.copy(os.path.join(t, n), os.path.join(out, n))
            else:
                R = Ref(args)
                R.set_freq(0)
                R.lib().ref_acsr_init(0)
                x = gold["x"]
                n = R.lE
                A = np.zeros((n, n), complex)
                F = np.zeros((n, n), complex)
                for j in range(n):  # probe both operators column by column
                    e = np.zeros(n, complex)
                    e[j] = 1.0
                    A[:, j] = R.apply(5, e)
                    F[:, j] = R.apply(0, e)
                iom = 1j * 2.0 * np.pi * float(np.float32(R.freqs[0])) * 4e-7 * np.pi
                interior = np.any(F != 0, axis=1)
                rows = np.arange(n)
                fdfd_diag = F[rows, rows]
                prev = np.maximum(rows - 1, 0)
                self_term = np.where(interior & (rows > 0), (A[rows, prev] - iom * F[rows, prev]) * x[prev], 0)
                np.savez_compressed(os.path.join(d, "acsr.npz"), x=x, Ax_csr=R.apply(5, x), Mx_csr=R.apply(6, x),
                                    freq=R.freqs[0], interior=interior, fdfd_diag=fdfd_diag, self_term=self_term,
                                    iom=iom)
        finally:
            os.chdir(cwd)


HY_OVERLAP = os.path.join(HERE, "hy_overlap")


def run_hy_overlap() -> None:
    from demo_matrixfree_csem_gb300 import synthetic
    from oracle import Ref
    d = HY_OVERLAP
    cfg = synthetic.random_small(18, nx=6, ny=3, nz=7, nb=2, airbc=0, preco=1, fvm=0)  # n2 = 7 < n3 = 11
    synthetic.write_config(cfg, d)
    args = [a.replace(d + "/", "") for a in cfg.args(d)]
    with open(os.path.join(d, "case.json"), "w") as f:
        json.dump(args, f, indent=1)
    cwd = os.getcwd()
    os.chdir(d)
    try:
        R = Ref(args)
        assert R.n2 < R.n3, (R.n2, R.n3)
        R.set_freq(0)
        rng = np.random.default_rng(18)
        x = (rng.integers(-2 ** 20, 2 ** 20, R.lE) + 1j * rng.integers(-2 ** 20, 2 ** 20, R.lE)) / 2 ** 20
        np.savez_compressed(os.path.join(d, "fdfd.npz"), x=x, Ax=R.apply(0, x), freq=R.freqs[0])
    finally:
        os.chdir(cwd)


def main() -> None:
    from oracle import ref_available
    if not ref_available():
        sys.exit("reference sources not found; nothing generated")
    if len(sys.argv) > 2:
        run_case(sys.argv[1], sys.argv[2])
        return
    if sys.argv[1:] == ["hy_overlap"]:
        run_hy_overlap()
        return
    subprocess.run([sys.executable, __file__, "hy_overlap"], check=True, stdout=subprocess.DEVNULL)
    print("wrote hy_overlap")
    for case in EXTENDED:
        subprocess.run([sys.executable, __file__, case, "extended"], check=True, stdout=subprocess.DEVNULL)
        print("wrote", case, "extended")
    for case in ACSR:
        subprocess.run([sys.executable, __file__, case, "acsr"], check=True, stdout=subprocess.DEVNULL)
        print("wrote", case, "acsr")


if __name__ == "__main__":
    main()
