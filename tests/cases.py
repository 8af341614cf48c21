"""Shared test helpers: golden cases, product grids and oracle contexts built from them."""
from __future__ import annotations

import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
# per-operator cases (args.json + golden.npz); layered_120/ holds whole-solve receivers only
GOLDEN_CASES = sorted(d for d in os.listdir(GOLDEN) if os.path.exists(os.path.join(GOLDEN, d, "args.json")))


def parse_args(args: list[str]) -> dict:
    """key=value list -> dict, last occurrence wins (as getpar)."""
    out = {}
    for a in args[1:]:
        if "=" in a:
            k, v = a.split("=", 1)
            out[k] = v
    return out


def load_golden(case: str):
    d = os.path.join(GOLDEN, case)
    with open(os.path.join(d, "args.json")) as f:
        args = json.load(f)
    z = np.load(os.path.join(d, "golden.npz"))
    return d, args, {k: z[k] for k in z.files}


def product_grid(d: str, params: dict):
    """The product's host setup (csem_grid_read/extend/airbc) for a case directory."""
    import demo_matrixfree_csem_gb300 as cs
    G = cs.Grid.from_files(*[os.path.join(d, n) for n in ("fx1", "fx2", "fx3", "frho11", "frho22", "frho33")])
    G.extend(int(params.get("nb", 15)), float(params.get("lextend", -1)), float(params.get("rho_air", 1e6)),
             int(params.get("istretch", 1)))
    if int(params.get("airbc", 0)):
        G.airbc(int(params.get("n1fft", 1024)), int(params.get("n2fft", 1024)))
    return G


def oracle_for(G, params: dict):
    """An oracle context fed with the product grid's arrays."""
    from oracle.pyoracle import GridArrays, Oracle
    A = G.arrays()
    g = G.g
    kw = {}
    if int(params.get("airbc", 0)):
        kw = dict(n1fft=g.n1fft, n2fft=g.n2fft, d1fft=g.d1fft, d2fft=g.d2fft, sH1=A["sH1"], sH2=A["sH2"],
                  jx=A["jx"], jy=A["jy"], wx=A["wx"], wy=A["wy"])
    ga = GridArrays(g.n1, g.n2, g.n3, g.nb, g.nz, int(params.get("airbc", 0)), int(params.get("fvm", 0)),
                    *[A[k] for k in ("x1", "x2", "x3", "x1s", "x2s", "x3s", "d1", "d2", "d3", "d1s", "d2s",
                                     "d3s", "sigma11", "sigma22", "sigma33")], rho_water=float(g.rho_water), **kw)
    return Oracle(ga)


def read_rows(path: str) -> np.ndarray:
    rows = []
    with open(path) as f:
        next(f)
        for line in f:
            p = line.split()
            if len(p) >= 5:
                rows.append([float(v) for v in p[:5]])
    return np.asarray(rows, np.float32)


def channels(params: dict, key: str) -> list[int]:
    m = {"Ex": 0, "Ey": 1, "Ez": 2, "Hx": 3, "Hy": 4, "Hz": 5}
    return [m[c] for c in params.get(key, "Ex").split(",")]


def probe(n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    re = rng.integers(-2 ** 20, 2 ** 20, n).astype(np.float64) / 2 ** 20
    im = rng.integers(-2 ** 20, 2 ** 20, n).astype(np.float64) / 2 ** 20
    return re + 1j * im


def tol_of(params: dict, ifreq: int, freqs) -> float:
    """tol/f computed in float, as main.c:94."""
    return float(np.float32(np.float32(float(params.get("tol", 1e-8))) / np.float32(freqs[ifreq])))


def relerr(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / den) if den > 0 else float(np.abs(a - b).max())
