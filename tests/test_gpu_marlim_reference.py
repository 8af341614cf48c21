"""The bench workload against the reference's own receivers.

tests/golden/marlim_like_96/reference_receivers.npz holds the receivers of the
Marlim-shaped model's first source at its six frequencies, computed by the reference
itself (tests/golden/make_reference_receivers.py: BiCGStab + LU-SGS to tol = 1e-8/f,
niter = 1000; it converged at 0.5-1.25 Hz in 641/468/391/317 iterations and stopped at
1000 at 0.125 and 0.25 Hz). At the frequencies where the reference converged, the
batched mixed-precision path (complex64 inner solves inside complex128 defect
correction, the path the bench times) must give the same receivers to 1e-7 relative,
max norm per channel (Ey measured against the Ex maximum, as it is small on the source
line).
"""
import os
import tempfile

import numpy as np
import pytest

import demo_matrixfree_csem_gb300 as cs
from demo_matrixfree_csem_gb300 import synthetic

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "marlim_like_96",
                       "reference_receivers.npz")


@pytest.mark.skipif(not os.path.exists(FIXTURE), reason="no reference receivers of the bench workload")
def test_mixed_batch_matches_reference_on_bench_workload(gpu):
    z = np.load(FIXTURE)
    cfg = synthetic.workload("marlim_like_96")
    niter = int(cfg.params.get("niter", 1000))
    # the reference logs niter residuals when it stops at niter, fewer when it converges
    conv = [f for f in range(len(z["freqs"])) if len(z[f"hist{f}"]) < niter]
    assert conv, "the reference converged at no frequency"
    with tempfile.TemporaryDirectory() as d:
        G = synthetic.build_grid(cfg, d)
    ctx = cs.Ctx(G, 1, 0)
    freqs = np.asarray(z["freqs"], np.float32)[conv]
    src = np.repeat(cfg.acq.src[:1, :3], len(conv), axis=0)
    r = cs.solve_batch(ctx, freqs, src, rec=cfg.acq.rec, precision=32, preco=1, niter=niter, tol=1e-8)
    assert r["status"] == ["converged"] * len(conv), r["status"]
    for q, f in enumerate(conv):
        ref = z["rec"][f]
        ex = np.abs(ref[0]).max()
        err = [float(np.abs(r["dcal"][q][c] - ref[c]).max() / (np.abs(ref[c]).max() if c != 1 else ex))
               for c in range(3)]
        print(f"{float(freqs[q])} Hz: mixed vs reference {err}")
        assert max(err) <= 1e-7, (float(freqs[q]), err)


@pytest.mark.skipif(not os.path.exists(FIXTURE), reason="no reference receivers of the bench workload")
def test_fp64_dropin_matches_reference_on_bench_workload(gpu):
    """The plain complex128 drop-in at the highest frequency: within 1e-9 of the reference."""
    z = np.load(FIXTURE)
    cfg = synthetic.workload("marlim_like_96")
    f = len(z["freqs"]) - 1
    with tempfile.TemporaryDirectory() as d:
        G = synthetic.build_grid(cfg, d)
    ctx = cs.Ctx(G, 1, 0)
    freq = float(z["freqs"][f])
    iom = cs.iom_of(freq)
    b = ctx.inject_source(iom, ["Ex"], cfg.acq.src[0])
    tol = float(np.float32(np.float32(1e-8) / np.float32(freq)))
    x, hist, it, st = ctx.solve_fp64(iom, b, algopt=1, preco=1, niter=1000, tol=tol)
    assert st == "converged"
    ref = z["rec"][f]
    out = ctx.extract_emf(["Ex", "Ey", "Ez"], cfg.acq.rec, x)
    ex = np.abs(ref[0]).max()
    err = [float(np.abs(out[c] - ref[c]).max() / (np.abs(ref[c]).max() if c != 1 else ex)) for c in range(3)]
    print(f"{freq} Hz: complex128 vs reference {err}, iterations {it} (reference {len(z[f'hist{f}']) - 1})")
    assert max(err) <= 1e-9, (freq, err)
