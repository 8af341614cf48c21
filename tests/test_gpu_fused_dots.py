"""The BiCGStab dot products folded into the complex64 stencil (fused_dots=1, an option):
after v = A p the stencil also sums v.r0, after t = A s it sums s.t and t.t, each CTA
writing one deterministic partial that the dot products' fixed-order final reduction adds
up. Through the batched mixed-precision solve (C ABI):
  * the fused form is the one that runs: every inner iteration launches two kernels fewer
    than with fused_dots=0 (the two dot-product passes; their final reductions remain);
  * the solve converges to the receivers of the separate dot products within 1e-6
    relative (the two partition the sums differently, so the iterates differ in rounding;
    both stop on the complex128 residual, 1e-8/f), in about as many iterations;
  * repeated runs give the same bits (the partition is fixed).
"""
import numpy as np
import pytest

import demo_matrixfree_csem_gb300 as cs
from cases import product_grid, relerr
from demo_matrixfree_csem_gb300 import api, synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def model(tmp_path_factory):
    d = tmp_path_factory.mktemp("fused")
    cfg = synthetic.random_small(72, nx=40, ny=27, nz=19, nb=4, airbc=1, fvm=0, n1fft=64, n2fft=64)
    synthetic.write_config(cfg, str(d))
    p = {k: str(v) for k, v in dict(cfg.params, nb=4).items()}
    return cfg, cs.Ctx(product_grid(str(d), p), 1, 0)


def _solve(cfg, ctx, fused, niter=1000, check_every=4):
    ctx.set_option("fused_dots", fused)
    freqs = np.array([0.5, 0.75, 1.0, 0.5, 0.75, 1.0], np.float32)
    src = np.repeat(cfg.acq.src[:1, :3], len(freqs), axis=0)
    src[:, 0] += np.arange(len(freqs), dtype=np.float32) * 31.0
    n0 = api.launch_count()
    r = cs.solve_batch(ctx, freqs, src, rec=cfg.acq.rec, precision=32, preco=1, niter=niter, tol=1e-8,
                       check_every=check_every, max_outer=1 if niter < 100 else 30)
    return r, api.launch_count() - n0


def test_fused_dots_remove_two_launches_per_iteration(gpu, model):
    """A fixed amount of work (one inner solve of 8 iterations, status read every 8):
    the separate dot products launch 2 more kernels per system-batch iteration."""
    cfg, ctx = model
    ctx.set_option("graphs", 0)  # direct launches, counted one by one
    try:
        a, na = _solve(cfg, ctx, 0, niter=8, check_every=8)
        b, nb = _solve(cfg, ctx, 1, niter=8, check_every=8)
    finally:
        ctx.set_option("graphs", 1)
        ctx.set_option("fused_dots", 0)
    assert na - nb == 2 * 8, (na, nb)


def test_fused_dots_converge_to_the_same_receivers(gpu, model):
    cfg, ctx = model
    sep, _ = _solve(cfg, ctx, 0)
    fus, _ = _solve(cfg, ctx, 1)
    again, _ = _solve(cfg, ctx, 1)
    ctx.set_option("fused_dots", 0)
    assert sep["status"] == ["converged"] * 6 and fus["status"] == ["converged"] * 6
    for q in range(6):
        assert relerr(fus["dcal"][q], sep["dcal"][q]) <= 1e-6, q
    assert np.all(np.abs(fus["iters"] - sep["iters"]) <= 0.1 * sep["iters"] + 8), (fus["iters"], sep["iters"])
    assert np.array_equal(fus["dcal"], again["dcal"]) and np.array_equal(fus["iters"], again["iters"])
