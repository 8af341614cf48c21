"""Line-tiled complex64 LU-SGS sweeps (lusgs_tiled) against the oracle and the pipelined
complex64 sweeps, through the C ABI.

The tiled schedule evaluates every point with the same linear-form update as the
pipelined complex64 sweeps, in an order that respects the lexicographic dependencies of
the reference's sweeps (fdfd.c:347-503), so the two give the same values. Tolerances:
  * against the complex128 oracle: <= 2e-5 relative (max norm), the complex64 bound of
    test_gpu_parity.py;
  * against the pipelined complex64 sweeps: <= 1e-6 relative (the same operations; only
    the compiler's multiply-add contraction may differ between the two kernels).
Grids cover line counts that are not multiples of 32, warps whose row blocks end inside
the grid, a single warp, both airbc settings (with airbc the air planes live in the cap
scratch) and fvm.
"""
import numpy as np
import pytest

import demo_matrixfree_csem_gb300 as cs
from cases import oracle_for, probe, product_grid, relerr
from demo_matrixfree_csem_gb300 import synthetic

pytestmark = pytest.mark.gpu

SHAPES = [  # (seed, nx, ny, nz, nb, airbc, fvm)
    (71, 40, 27, 19, 4, 0, 0),
    (72, 40, 27, 19, 4, 1, 0),
    (73, 33, 45, 12, 3, 1, 1),
    (74, 70, 9, 41, 5, 0, 0),
    (75, 5, 6, 4, 2, 0, 0),
]


def _setup(tmp_path, seed, nx, ny, nz, nb, airbc, fvm):
    cfg = synthetic.random_small(seed, nx=nx, ny=ny, nz=nz, nb=nb, airbc=airbc, fvm=fvm, n1fft=64, n2fft=64)
    synthetic.write_config(cfg, str(tmp_path))
    p = {k: str(v) for k, v in dict(cfg.params, nb=nb).items()}
    G = product_grid(str(tmp_path), p)
    ctx = cs.Ctx(G, airbc, fvm)
    ctx.set_option("lusgs_split", 0)  # the one-pass pipelined sweeps, which the tiled ones restate
    O = oracle_for(G, p)
    return G, ctx, O, cfg


@pytest.mark.parametrize("shape", SHAPES, ids=[f"{s[1]}x{s[2]}x{s[3]}_air{s[5]}_fvm{s[6]}" for s in SHAPES])
def test_tiled_sweeps_match_pipelined_and_oracle(gpu, tmp_path, shape):
    G, ctx, O, _ = _setup(tmp_path, *shape)
    f = 0.75
    O.set_freq(f)
    iom = cs.iom_of(f)
    x = probe(ctx.lE, shape[0])
    mo = O.lusgs(x)
    ctx.set_option("lusgs_tiled", 0)
    ref = ctx.lusgs_apply(iom, x, c64=True)
    assert relerr(ref, mo) <= 2e-5
    for rows in (4, 8, 16):
        for vw in (1, 2, 4):
            ctx.set_option("lusgs_tiled", 1)
            ctx.set_option("lusgs_tile_rows", rows)
            ctx.set_option("lusgs_tile_vw", vw)
            got = ctx.lusgs_apply(iom, x, c64=True)
            assert np.all(np.isfinite(got)), (rows, vw)
            assert relerr(got, ref) <= 1e-6, (rows, vw, relerr(got, ref))
            assert relerr(got, mo) <= 2e-5, (rows, vw)
    ctx.set_option("lusgs_tiled", 0)


def test_tiled_sweeps_leave_complex128_alone(gpu, tmp_path):
    """The option selects complex64 kernels only: complex128 stays bit-identical to the
    oracle (the reference's arithmetic)."""
    G, ctx, O, _ = _setup(tmp_path, *SHAPES[1])
    O.set_freq(0.5)
    x = probe(ctx.lE, 3)
    ctx.set_option("lusgs_tiled", 1)
    assert np.array_equal(ctx.lusgs_apply(cs.iom_of(0.5), x), O.lusgs(x))
    ctx.set_option("lusgs_tiled", 0)


def test_tiled_batch_matches_pipelined_batch(gpu, tmp_path):
    """The batched mixed-precision solve with the tiled sweeps converges to the same
    receivers as with the pipelined sweeps (the two preconditioners agree to rounding)."""
    G, ctx, O, cfg = _setup(tmp_path, *SHAPES[1])
    rec = cfg.acq.rec
    freqs = np.array([0.5, 1.0], np.float32)
    src = np.repeat(cfg.acq.src[:1, :3], 2, axis=0)
    ctx.set_option("lusgs_tiled", 0)
    a = cs.solve_batch(ctx, freqs, src, rec=rec, precision=32, preco=1, niter=1000, tol=1e-8)
    ctx.set_option("lusgs_tiled", 1)
    b = cs.solve_batch(ctx, freqs, src, rec=rec, precision=32, preco=1, niter=1000, tol=1e-8)
    ctx.set_option("lusgs_tiled", 0)
    assert a["status"] == ["converged"] * 2 and b["status"] == ["converged"] * 2
    for q in range(2):
        assert relerr(b["dcal"][q], a["dcal"][q]) <= 1e-6


@pytest.mark.parametrize("shape", SHAPES, ids=[f"{s[1]}x{s[2]}x{s[3]}_air{s[5]}_fvm{s[6]}" for s in SHAPES])
def test_pipelined_conveyor_of_lines_agrees(gpu, tmp_path, shape):
    """The complex64 pipelined sweeps with several lines per CTA (lusgs_lines, a conveyor:
    a row that finishes a line starts the next one while the rows behind it are still on
    the previous line) give the values of one line per CTA, for every points-per-thread
    width and for line counts that do not divide the grid. Each configuration is its own
    kernel path, and the compiler may contract multiply-adds differently, so the bound
    is 1e-6 relative; against the complex128 oracle the complex64 bound 2e-5 holds."""
    G, ctx, O, _ = _setup(tmp_path, *shape)
    O.set_freq(0.75)
    iom = cs.iom_of(0.75)
    x = probe(ctx.lE, shape[0] + 1)
    mo = O.lusgs(x)
    for vw in (1, 2, 4):
        ctx.set_option("lusgs_vw", vw)
        ctx.set_option("lusgs_lines", 1)
        ref = ctx.lusgs_apply(iom, x, c64=True)
        assert relerr(ref, mo) <= 2e-5
        for lines in (2, 3, 7):
            ctx.set_option("lusgs_lines", lines)
            got = ctx.lusgs_apply(iom, x, c64=True)
            assert relerr(got, ref) <= 1e-6, (vw, lines, relerr(got, ref))
    ctx.set_option("lusgs_lines", 1)
    ctx.set_option("lusgs_vw", 0)


@pytest.mark.parametrize("shape", SHAPES, ids=[f"{s[1]}x{s[2]}x{s[3]}_air{s[5]}_fvm{s[6]}" for s in SHAPES])
def test_stencil_shapes_give_identical_bits(gpu, tmp_path, shape):
    """The stencil's tile height (stencil_by: 4, 8, 16 output rows per CTA) and plane-chunk
    depth (stencil_ctas) only regroup the same per-point work: complex128 and complex64
    results are bit-identical for every shape, and complex128 equals the oracle (through
    the airwave FFT: 1e-12). Where n2 < n3 (70x9x41) the reference's Hy scratch, sized
    n1*(n2+1)*n2 (fdfd.c:59), overlaps Hz and its fdfd_apply mixes the two; the GPU keeps
    H disjoint, which is the reference's own result whenever n2 >= n3, so that shape is
    compared with the oracle at the disjoint length."""
    G, ctx, O, _ = _setup(tmp_path, *shape)
    if ctx.n2 < ctx.n3:
        O.set_hy_length(False)
    O.set_freq(0.5)
    iom = cs.iom_of(0.5)
    x = probe(ctx.lE, shape[0] + 2)
    ref64 = ctx.fdfd_apply(iom, x)
    ref32 = ctx.fdfd_apply(iom, x, c64=True)
    yo = O.fdfd(x)
    assert (relerr(ref64, yo) <= 1e-12) if shape[5] else np.array_equal(ref64, yo)
    for by in (4, 8, 16):
        for ctas in (1, 4, 16):
            ctx.set_option("stencil_by", by)
            ctx.set_option("stencil_ctas", ctas)
            assert np.array_equal(ctx.fdfd_apply(iom, x), ref64), (by, ctas)
            assert np.array_equal(ctx.fdfd_apply(iom, x, c64=True), ref32), (by, ctas)
    ctx.set_option("stencil_by", 8)
    ctx.set_option("stencil_ctas", 4)
