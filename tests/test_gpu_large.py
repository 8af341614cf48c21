"""The large memory-bound batch: 400x400x200 core cells of 50 m padded to 420x420x220
(about 116M complex edge unknowns per system), 192 systems solved in waves that fit
180 GB of device memory.

Checks, on the full grid: the wave size the capacity planner gives for 180 GB; one wave
of that many systems through a few batched mixed-precision iterations (finite results,
no allocation failure); and the complex128 LU-SGS of the lockstep sweeps (including the
Ez sweep's 419 rows, handed over through a CTA barrier) against the one-launch-per-
diagonal schedule, bit for bit."""
import tempfile

import numpy as np
import pytest

import demo_matrixfree_csem_gb300 as cs
from demo_matrixfree_csem_gb300 import synthetic

pytestmark = pytest.mark.gpu

BUDGET = 180e9


@pytest.fixture(scope="module")
def large(gpu):
    import torch
    if torch.cuda.get_device_properties(0).total_memory < 200e9:
        pytest.skip("needs a device with more than 200 GB")
    cfg = synthetic.large_420()
    with tempfile.TemporaryDirectory() as d:
        G = synthetic.build_grid(cfg, d)
    ctx = cs.Ctx(G, 1, 0)
    assert (ctx.n1, ctx.n2, ctx.n3f) == (420, 420, 220)
    return cfg, ctx


def test_wave_size_fits_budget(large):
    cfg, ctx = large
    n = ctx.batch_capacity(BUDGET)
    assert 8 <= n <= 16, n
    assert ctx.batch_bytes(n) <= BUDGET < ctx.batch_bytes(n + 1)


def test_one_wave_runs(large):
    import torch
    cfg, ctx = large
    n = ctx.batch_capacity(BUDGET)
    freqs = np.full(n, 0.5, np.float32)
    srcs = cfg.acq.src[:n, :3]
    r = cs.solve_batch(ctx, freqs, srcs, rec=cfg.acq.rec, precision=32, preco=1, niter=6, tol=1e-30,
                       max_outer=1, check_every=6)
    assert all(s == "maxiter" for s in r["status"]), r["status"]
    assert np.all(np.isfinite(r["dcal"])) and np.all(r["relres"] < 1.0)
    free, total = torch.cuda.mem_get_info()
    assert total - free < 270e9


def test_large_grid_lusgs_schedules_agree(large):
    cfg, ctx = large
    rng = np.random.default_rng(4)
    x = rng.standard_normal(ctx.lE) + 1j * rng.standard_normal(ctx.lE)
    iom = cs.iom_of(0.5)
    ctx.set_option("lusgs_pipelined", 1)
    a = ctx.lusgs_apply(iom, x)
    ctx.set_option("lusgs_pipelined", 0)
    b = ctx.lusgs_apply(iom, x)
    ctx.set_option("lusgs_pipelined", 1)
    assert np.array_equal(a, b)


def test_all_192_systems_stream_in_waves(large):
    """The whole workload once: 6 frequencies x 32 sources = 192 systems admitted in
    waves of the planner's size for 180 GB, each wave a bounded run of the batched
    mixed-precision solve (4 complex64 iterations, one defect correction), injection
    and receiver extraction included. Every system comes back finite, and the time per
    wave is reported."""
    import time

    import torch
    cfg, ctx = large
    n = ctx.batch_capacity(BUDGET)
    freqs = [float(f) for f in cfg.params["freqs"].split(",")]
    systems = [(f, s) for f in freqs for s in range(len(cfg.acq.src))]
    assert len(systems) == 192
    seen, times = 0, []
    for w in range(0, len(systems), n):
        sel = systems[w:w + n]
        f = np.array([t[0] for t in sel], np.float32)
        src = cfg.acq.src[[t[1] for t in sel], :3]
        t0 = time.perf_counter()
        r = cs.solve_batch(ctx, f, src, rec=cfg.acq.rec, precision=32, preco=1, niter=4, tol=1e-30, max_outer=1,
                           check_every=4)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
        assert all(s == "maxiter" for s in r["status"]), r["status"]
        assert np.all(np.isfinite(r["dcal"])) and np.all(r["relres"] < 1.0)
        seen += len(sel)
    assert seen == 192
    print(f"192 systems in {len(times)} waves of up to {n}: {sum(times):.1f} s, "
          f"{min(times):.2f}-{max(times):.2f} s per wave")
