"""SHA-256 checksums of the reference's own padded model at the bench workload's scale.

The reference (compiled from its sources by oracle/build_ref.sh) reads the Marlim-shaped
model (synthetic.marlim_like(seed=0): 180x120x120 cells, nb=10 stretched padding to
lextend=120 km, airbc=1 with 1024x1024 airwave filters) and runs its set-up
(emf_init_free.c, extend_model.c:24-252 including the bottom-padding quirk at
:169-173, create_nugrid.c, find_index.c, airbc_init_free.c:24-109). The arrays are far
too large to commit (three edge conductivity arrays of about 4M doubles each), so this
writes one checksum per array instead; tests/test_oracle_golden.py recomputes them from
the product's set-up (host/csem_setup.c) and requires equality, i.e. bit-identical
arrays.

Run where the reference sources exist (CSEM_REFERENCE_DIR, else a sibling directory
"reference" of this repository):
    python tests/golden/make_setup_checksums.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

ARRAYS = ("x1", "x2", "x3", "x1s", "x2s", "x3s", "d1", "d2", "d3", "d1s", "d2s", "d3s",
          "sigma11", "sigma22", "sigma33", "sH1", "sH2", "jx", "jy", "wx", "wy")


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def valid_nodes(g) -> dict:
    """Uniform airwave nodes the reference's set-up writes (airbc_init_free.c:90-105):
    x below the last staggered node of the model. The entries past them are left
    unwritten by the reference (its malloc'd jx/jy/wx/wy) and never read."""
    n1 = int(np.sum(g.x1s[0] + np.arange(g.n1fft) * g.d1fft < g.x1s[g.n1 - 1]))
    n2 = int(np.sum(g.x2s[0] + np.arange(g.n2fft) * g.d2fft < g.x2s[g.n2 - 1]))
    return {"jx": n1, "wx": n1, "jy": n2, "wy": n2}


def checksums(g) -> dict:
    nv = valid_nodes(g)
    return {k: digest(getattr(g, k)[:nv[k]] if k in nv else getattr(g, k)) for k in ARRAYS}


def main() -> None:
    from demo_matrixfree_csem_gb300 import synthetic
    from oracle import Ref, ref_available
    if not ref_available():
        sys.exit("reference sources not found; nothing generated")
    cfg = synthetic.workload("marlim_like_96")
    with tempfile.TemporaryDirectory() as d:
        synthetic.write_config(cfg, d)
        cwd = os.getcwd()
        os.chdir(d)
        try:
            R = Ref(cfg.args(d))
            g = R.grid_arrays()
        finally:
            os.chdir(cwd)
    out = {"workload": "marlim_like_96", "n1": g.n1, "n2": g.n2, "n3": g.n3f, "nb": g.nb,
           "n1fft": g.n1fft, "n2fft": g.n2fft, "valid_airwave_nodes": valid_nodes(g), "sha256": checksums(g)}
    path = os.path.join(HERE, "marlim_like_96", "setup_sha256.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
