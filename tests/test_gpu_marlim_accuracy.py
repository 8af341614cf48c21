"""Accuracy of the batch the bench times, against the complex128 solver.

tests/golden/marlim_like_96/fp64_receivers.npz holds the receivers of 18 systems of the
96-system bench workload (all six frequencies 0.125-1.25 Hz x sources 0, 7 and 15),
solved by the plain complex128 path (the reference's BiCGStab + LU-SGS arithmetic,
tolerance 1e-8/f, iteration limit raised to 4000 so that every one converged;
tests/golden/make_fp64_receivers.py). The batched mixed-precision path with the bench's
settings (complex64 inner solves inside complex128 defect correction) solves the same 18
systems in one batch; its receivers must agree to 1e-7 relative (max norm over the
receiver line) per frequency and channel, the accuracy target of the bench. Ey vanishes
by symmetry on the source line up to the model's off-line resistors, so its error is
measured against the Ex maximum.
"""
import os
import tempfile

import numpy as np
import pytest

import demo_matrixfree_csem_gb300 as cs
from demo_matrixfree_csem_gb300 import synthetic

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "marlim_like_96", "fp64_receivers.npz")
TOL = 1e-7


def channel_errors(got, ref):
    """[Ex, Ey, Ez] max-norm relative errors; Ey against the Ex maximum."""
    ex = np.abs(ref[0]).max()
    return [float(np.abs(got[c] - ref[c]).max() / (np.abs(ref[c]).max() if c != 1 else ex)) for c in range(3)]


def test_mixed_batch_matches_complex128_on_all_frequencies(gpu):
    z = np.load(FIXTURE)
    assert list(z["status"]) == ["converged"] * len(z["freqs"])
    cfg = synthetic.workload("marlim_like_96")
    with tempfile.TemporaryDirectory() as d:
        G = synthetic.build_grid(cfg, d)
    ctx = cs.Ctx(G, 1, 0)
    freqs = np.asarray(z["freqs"], np.float32)
    src = cfg.acq.src[np.asarray(z["isrc"]), :3]
    r = cs.solve_batch(ctx, freqs, src, rec=cfg.acq.rec, precision=32, preco=1, niter=1000, tol=1e-8,
                       inner_tol=0.2, check_every=4)
    assert r["status"] == ["converged"] * len(freqs), r["status"]
    worst = {}
    for q in range(len(freqs)):
        err = channel_errors(r["dcal"][q], z["rec"][q])
        f = float(freqs[q])
        worst[f] = [max(a, b) for a, b in zip(worst.get(f, [0.0] * 3), err)]
        print(f"{f} Hz source {int(z['isrc'][q])}: mixed vs complex128 Ex/Ey/Ez {err[0]:.2e} {err[1]:.2e} "
              f"{err[2]:.2e} (inner iterations {int(r['iters'][q])}, complex128 {int(z['iters'][q])})")
    for f, e in sorted(worst.items()):
        assert max(e) <= TOL, (f, e)
