"""csem_solve_batch_multi: the systems of one model split over several slots, one
context and host thread each, outputs gathered at their original positions.

This run has one GPU, so the slots name the same device twice (two independent
contexts on it; nothing waits on another slot). Each system's arithmetic does not depend
on which other systems share its batch, so the gathered receivers, iteration counts and
statuses are bit-identical to one batch of all systems on one context."""
import numpy as np
import pytest

import demo_matrixfree_csem_gb300 as cs
from cases import product_grid
from demo_matrixfree_csem_gb300 import synthetic

pytestmark = pytest.mark.gpu


def test_split_over_two_slots_equals_one_batch(gpu, tmp_path):
    cfg = synthetic.random_small(52, nx=24, ny=20, nz=14, nb=4, airbc=1, n1fft=64, n2fft=64, freqs=(0.5, 1.0))
    synthetic.write_config(cfg, str(tmp_path))
    G = product_grid(str(tmp_path), {k: str(v) for k, v in cfg.params.items()})
    freqs = np.array([0.25, 0.5, 1.0, 0.5, 2.0, 1.0], np.float32)
    srcs = np.repeat(cfg.acq.src[:1, :3], 6, axis=0)
    srcs[:, 0] += 41.0 * np.arange(6)
    ctx = cs.Ctx(G, 1, 0)
    one = cs.solve_batch(ctx, freqs, srcs, rec=cfg.acq.rec, precision=32, preco=1, niter=1000, tol=1e-8)
    ctx.close()
    two = cs.solve_batch_multi(G, [0, 0], freqs, srcs, airbc=1, rec=cfg.acq.rec, precision=32, preco=1, niter=1000,
                               tol=1e-8)
    owner, load = cs.partition_systems(2, freqs, unknowns=1.0)
    assert np.array_equal(two["owner"], owner) and set(owner.tolist()) == {0, 1}
    assert one["status"] == two["status"] == ["converged"] * 6
    assert np.array_equal(one["dcal"], two["dcal"])
    assert np.array_equal(one["iters"], two["iters"])
    # complex128 through the same split
    r64 = cs.solve_batch_multi(G, [0, 0, 0], freqs[:3], srcs[:3], airbc=1, rec=cfg.acq.rec, precision=64, preco=1,
                               niter=1000, tol=1e-8)
    assert r64["status"] == ["converged"] * 3
    for q in range(3):
        assert np.abs(r64["dcal"][q] - one["dcal"][q]).max() <= 1e-6 * np.abs(r64["dcal"][q]).max()


def test_bad_device_is_an_error(gpu, tmp_path):
    cfg = synthetic.random_small(53, nx=8, ny=8, nz=6, nb=2)
    synthetic.write_config(cfg, str(tmp_path))
    G = product_grid(str(tmp_path), {k: str(v) for k, v in cfg.params.items()})
    with pytest.raises(cs.CsemError) as e:
        cs.solve_batch_multi(G, [0, 999], [0.5], cfg.acq.src[:1, :3], rec=cfg.acq.rec)
    assert e.value.code == -1
