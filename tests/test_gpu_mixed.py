"""Batched mixed-precision solver vs the complex128 solver and the oracle.

A small airwave model with two frequencies x two sources is solved three ways:
  * the CPU oracle (the reference's arithmetic, sequential dots), system by system;
  * the complex128 GPU path (precision 64), system by system;
  * the batched mixed-precision GPU path (precision 32), all four systems at once.
Receivers are compared per frequency and channel in the max norm over receivers.
Tolerances: complex128 GPU vs oracle after convergence to tol/f: the two runs differ
only in the summation order of their dot products, so the bound is the larger of 1e-9
and 100x the change the oracle itself shows when b moves by one ulp, capped at 1e-6
(both stop at the same residual level); mixed vs complex128 GPU <= 1e-6 at tol=1e-8
(the true-residual stopping test of the mixed path is at least as strict as the
reference's recursive-residual test).
"""
import numpy as np
import pytest

import demo_matrixfree_csem_gb300 as cs
from cases import oracle_for, product_grid, relerr
from demo_matrixfree_csem_gb300 import synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_case(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("mixed"))
    cfg = synthetic.random_small(51, nx=24, ny=20, nz=14, nb=4, airbc=1, n1fft=64, n2fft=64, freqs=(0.5, 1.0))
    synthetic.write_config(cfg, d)
    p = {k: str(v) for k, v in cfg.params.items()}
    G = product_grid(d, p)
    ctx = cs.Ctx(G, 1, 0)
    src = np.stack([cfg.acq.src[0], cfg.acq.src[0] + np.array([37.0, -23.0, 0, 0, 0], np.float32)])
    return cfg, G, ctx, p, src


def _systems(cfg, src):
    freqs = np.array([0.5, 0.5, 1.0, 1.0], np.float32)
    srcs = np.stack([src[0], src[1], src[0], src[1]])[:, :3]
    return freqs, srcs


def test_fp64_batch_matches_oracle(gpu, small_case):
    cfg, G, ctx, p, src = small_case
    freqs, srcs = _systems(cfg, src)
    rec = cfg.acq.rec
    r64 = cs.solve_batch(ctx, freqs, srcs, chrec=("Ex", "Ey", "Ez"), rec=rec, precision=64, preco=1, niter=400,
                         tol=1e-8)
    assert all(s == "converged" for s in r64["status"])
    O = oracle_for(G, p)
    for s in range(len(freqs)):
        O.set_freq(float(freqs[s]))
        b = O.inject([0], srcs[s])
        tol = float(np.float32(np.float32(1e-8) / freqs[s]))
        x, h, it = O.solve(b, algopt=1, precond=1, niter=400, tol=tol)
        ref = O.extract([0, 1, 2], rec, x)
        x1, _, _ = O.solve(b * (1 + 2.0 ** -52), algopt=1, precond=1, niter=400, tol=tol)
        ref1 = O.extract([0, 1, 2], rec, x1)
        for c in range(3):
            bound = min(1e-6, max(1e-9, 100 * relerr(ref1[c], ref[c])))
            assert relerr(r64["dcal"][s, c], ref[c]) <= bound, (s, c, bound)
        assert abs(r64["iters"][s] - it) <= max(2, 0.15 * it)


def test_mixed_batch_matches_fp64(gpu, small_case):
    cfg, G, ctx, p, src = small_case
    freqs, srcs = _systems(cfg, src)
    rec = cfg.acq.rec
    r64 = cs.solve_batch(ctx, freqs, srcs, rec=rec, precision=64, preco=1, niter=400, tol=1e-8)
    r32 = cs.solve_batch(ctx, freqs, srcs, rec=rec, precision=32, preco=1, niter=400, tol=1e-8, inner_tol=1e-4)
    assert all(s == "converged" for s in r32["status"]), r32
    for s in range(len(freqs)):
        assert r32["relres"][s] < float(np.float32(np.float32(1e-8) / freqs[s]))
        for c in range(3):
            assert relerr(r32["dcal"][s, c], r64["dcal"][s, c]) <= 1e-6, (s, c, relerr(r32["dcal"][s, c], r64["dcal"][s, c]))


def test_autotuned_batch_matches_fp64(gpu, small_case):
    """With the LU-SGS autotuner on, the batch still converges to the complex128 answer."""
    cfg, G, ctx, p, src = small_case
    freqs, srcs = _systems(cfg, src)
    rec = cfg.acq.rec
    r64 = cs.solve_batch(ctx, freqs, srcs, rec=rec, precision=64, preco=1, niter=400, tol=1e-8)
    ctx.set_option("autotune", 1)
    try:
        r32 = cs.solve_batch(ctx, freqs, srcs, rec=rec, precision=32, preco=1, niter=400, tol=1e-8)
    finally:
        ctx.set_option("autotune", 0)
    assert all(s == "converged" for s in r32["status"]), r32
    for s in range(len(freqs)):
        for c in range(3):
            assert relerr(r32["dcal"][s, c], r64["dcal"][s, c]) <= 1e-6


def test_mixed_batch_aphi(gpu, small_case):
    """The reference's A-phi preconditioner (with its sigma-lookup and diagonal quirks)
    does not bring BiCGStab to 1e-8 on these models even in complex128 (the oracle stalls
    between 1e-3 and 0.3 after 1000 iterations), so the mixed A-phi path is held to what
    the complex128 path reaches with the same number of preconditioner applications:
    finite, no breakdown, progress, and a true residual within 10x of the complex128
    one (both trajectories are erratic before convergence)."""
    cfg, G, ctx, p, src = small_case
    freqs, srcs = _systems(cfg, src)
    rec = cfg.acq.rec
    r = cs.solve_batch(ctx, freqs[:2], srcs[:2], rec=rec, precision=32, preco=3, niter=300, tol=1e-8,
                       max_outer=1, inner_tol=1e-12)
    r64 = cs.solve_batch(ctx, freqs[:2], srcs[:2], rec=rec, precision=64, preco=3, niter=300, tol=1e-8)
    for s in range(2):
        assert r["status"][s] in ("converged", "maxiter"), r["status"]
        assert np.all(np.isfinite(r["dcal"][s]))
        assert r["relres"][s] < 1 and r["relres"][s] <= 10 * r64["relres"][s], (r["relres"], r64["relres"])


def test_mixed_gmres_matches_fp64(gpu, small_case):
    """Batched complex64 flexible GMRES(10) inner solves with LU-SGS inside complex128
    defect correction reach the same answer as the complex128 solver."""
    cfg, G, ctx, p, src = small_case
    freqs, srcs = _systems(cfg, src)
    rec = cfg.acq.rec
    r64 = cs.solve_batch(ctx, freqs, srcs, rec=rec, precision=64, preco=1, niter=400, tol=1e-8)
    r32 = cs.solve_batch(ctx, freqs, srcs, rec=rec, precision=32, algopt=2, nrestart=10, preco=1, niter=1000,
                         tol=1e-8)
    assert all(s == "converged" for s in r32["status"]), r32
    for s in range(len(freqs)):
        assert r32["relres"][s] < float(np.float32(np.float32(1e-8) / freqs[s]))
        for c in range(3):
            assert relerr(r32["dcal"][s, c], r64["dcal"][s, c]) <= 1e-6


def test_mixed_gmres_aphi(gpu, small_case):
    """GMRES(10) with A-phi (the combination of the uneven-size batch configuration):
    the reference's A-phi does not converge on these models, so the batched complex64
    path is held to the complex128 GMRES's residual after the same budget."""
    cfg, G, ctx, p, src = small_case
    freqs, srcs = _systems(cfg, src)
    rec = cfg.acq.rec
    r = cs.solve_batch(ctx, freqs[:2], srcs[:2], rec=rec, precision=32, algopt=2, nrestart=10, preco=3, niter=200,
                       tol=1e-8, max_outer=1, inner_tol=1e-12)
    r64 = cs.solve_batch(ctx, freqs[:2], srcs[:2], rec=rec, precision=64, algopt=2, nrestart=10, preco=3, niter=200,
                         tol=1e-8)
    for s in range(2):
        assert r["status"][s] in ("converged", "maxiter"), r["status"]
        assert np.all(np.isfinite(r["dcal"][s]))
        assert r["relres"][s] < 1 and r["relres"][s] <= 10 * r64["relres"][s], (r["relres"], r64["relres"])


def test_graph_replay_is_bit_identical(gpu, small_case):
    """The iterations between status reads replayed as CUDA graphs launch the same kernels
    in the same order as direct launches: identical bits and iteration counts."""
    cfg, G, ctx, p, src = small_case
    freqs, srcs = _systems(cfg, src)
    out = {}
    for graphs in (1, 0):
        ctx.set_option("graphs", graphs)
        out[graphs] = cs.solve_batch(ctx, freqs, srcs, rec=cfg.acq.rec, precision=32, preco=1, niter=400, tol=1e-8)
    ctx.set_option("graphs", 1)
    assert np.array_equal(out[1]["dcal"], out[0]["dcal"])
    assert np.array_equal(out[1]["iters"], out[0]["iters"]) and out[1]["status"] == out[0]["status"]


def test_concurrent_contexts_match_separate_solves(gpu, tmp_path):
    """Uneven-size batch: three models of different grid sizes (and paddings) on three
    contexts, solved at the same time by csem_solve_batches_host (one host thread and one
    stream per context), give exactly the results of solving each context alone."""
    ctxs, cfgs = [], []
    for q, (nx, ny, nz, nb) in enumerate([(24, 20, 14, 4), (30, 18, 12, 3), (20, 26, 16, 5)]):
        cfg = synthetic.random_small(70 + q, nx=nx, ny=ny, nz=nz, nb=nb, airbc=1, n1fft=64, n2fft=64)
        d = tmp_path / f"m{q}"
        d.mkdir()
        synthetic.write_config(cfg, str(d))
        p = {k: str(v) for k, v in cfg.params.items()}
        ctxs.append(cs.Ctx(product_grid(str(d), p), 1, 0))
        cfgs.append(cfg)
    jobs = []
    for q, (ctx, cfg) in enumerate(zip(ctxs, cfgs)):
        srcs = np.stack([cfg.acq.src[0], cfg.acq.src[0] + np.array([19.0, 11.0, 0, 0, 0], np.float32)])
        jobs.append(dict(ctx=ctx, freqs=np.array([0.5, 1.0], np.float32), srcs=srcs, rec=cfg.acq.rec, niter=400,
                         tol=1e-8, algopt=1 + (q % 2), nrestart=10))
    together = cs.solve_batches(jobs)
    for j, got in zip(jobs, together):
        args = {k: v for k, v in j.items() if k not in ("ctx", "freqs", "srcs")}
        alone = cs.solve_batch(j["ctx"], j["freqs"], j["srcs"], **args)
        assert got["status"] == alone["status"] == ["converged", "converged"]
        assert np.array_equal(got["dcal"], alone["dcal"]) and np.array_equal(got["iters"], alone["iters"])


def test_batch_is_deterministic(gpu, small_case):
    cfg, G, ctx, p, src = small_case
    freqs, srcs = _systems(cfg, src)
    a = cs.solve_batch(ctx, freqs, srcs, rec=cfg.acq.rec, precision=32, preco=1, niter=400, tol=1e-8)
    b = cs.solve_batch(ctx, freqs, srcs, rec=cfg.acq.rec, precision=32, preco=1, niter=400, tol=1e-8)
    assert np.array_equal(a["dcal"], b["dcal"]) and np.array_equal(a["iters"], b["iters"])


def test_zero_source_is_reported(gpu, small_case):
    cfg, G, ctx, p, src = small_case
    # a source channel code that injects nothing gives b = 0 (solver.c:116-125)
    r = cs.solve_batch(ctx, [0.5], src[:1, :3], chsrc=(3,), rec=cfg.acq.rec, precision=32)
    assert r["status"] == ["zero_rhs"] and np.all(r["dcal"] == 0)
