"""Complex64 LU-SGS sweep variants against the single-system pipelined sweeps and the
oracle, through the C ABI (csem_lusgs_apply_dev on a batch and the batched
mixed-precision solve):
  * several systems of one frequency per CTA (lusgs_systems 2 or 4, k_lusgs4.cu);
  * split sweeps (lusgs_split, the complex64 default, k_lusgs5.cu): a coalesced pass
    stores every point's (B, w), then the row pipeline runs the chain.

The batch mixes frequencies so that groups are partly filled: 7 systems at 0.75, 0.5,
0.75, 1.0, 0.75, 0.5, 0.75 Hz form the groups (0,2,4,6), (1,5), (3) of four and (0,2),
(4,6), (1,5), (3) of two. Every system must get what the single-system sweeps give it
to 1e-6 relative (the same operations per point; only the compiler's multiply-add
contraction may differ between the kernels) and stay within the complex64 bound 2e-5 of
the complex128 oracle. Grids: those of test_gpu_tiled_sweeps (line counts that are not
multiples of 32, both airbc settings, fvm, a single warp) and, for the split sweeps, a
grid whose Ez sweep has more than 256 rows (CTAs of up to 512 threads).
"""
import ctypes as C

import numpy as np
import pytest

import demo_matrixfree_csem_gb300 as cs
from cases import oracle_for, probe, product_grid, relerr
from demo_matrixfree_csem_gb300 import api, synthetic

pytestmark = pytest.mark.gpu

SHAPES = [  # (seed, nx, ny, nz, nb, airbc, fvm)
    (71, 40, 27, 19, 4, 0, 0),
    (72, 40, 27, 19, 4, 1, 0),
    (73, 33, 45, 12, 3, 1, 1),
    (74, 70, 9, 41, 5, 0, 0),
    (75, 5, 6, 4, 2, 0, 0),
]
FREQS = [0.75, 0.5, 0.75, 1.0, 0.75, 0.5, 0.75]


def _setup(tmp_path, seed, nx, ny, nz, nb, airbc, fvm):
    cfg = synthetic.random_small(seed, nx=nx, ny=ny, nz=nz, nb=nb, airbc=airbc, fvm=fvm, n1fft=64, n2fft=64)
    synthetic.write_config(cfg, str(tmp_path))
    p = {k: str(v) for k, v in dict(cfg.params, nb=nb).items()}
    G = product_grid(str(tmp_path), p)
    return cfg, G, cs.Ctx(G, airbc, fvm), oracle_for(G, p)


def _lusgs_batch(ctx, freqs, X):
    """complex64 LU-SGS on every row of X (systems), one call on the device."""
    import torch
    x = torch.from_numpy(np.ascontiguousarray(X, np.complex64)).cuda()
    y = torch.zeros_like(x)
    iom = np.zeros(2 * len(freqs))
    for q, f in enumerate(freqs):
        z = cs.iom_of(f)
        iom[2 * q], iom[2 * q + 1] = z.real, z.imag
    torch.cuda.synchronize()
    rc = api.lib().csem_lusgs_apply_dev(ctx.h, 32, len(freqs), iom.ctypes.data_as(C.POINTER(C.c_double)),
                                        C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), None)
    assert rc == 0, api.lib().csem_last_error().decode()
    torch.cuda.synchronize()
    return y.cpu().numpy().astype(np.complex128)


@pytest.mark.parametrize("shape", SHAPES, ids=[f"{s[1]}x{s[2]}x{s[3]}_air{s[5]}_fvm{s[6]}" for s in SHAPES])
def test_grouped_sweeps_match_single_system_sweeps_and_oracle(gpu, tmp_path, shape):
    cfg, G, ctx, O = _setup(tmp_path, *shape)
    ctx.set_option("lusgs_split", 0)
    X = np.stack([probe(ctx.lE, shape[0] + 10 + q) for q in range(len(FREQS))])
    ctx.set_option("lusgs_systems", 1)
    ref = _lusgs_batch(ctx, FREQS, X)
    for q, f in enumerate(FREQS):
        O.set_freq(f)
        assert relerr(ref[q], O.lusgs(X[q])) <= 2e-5, q
    for ns, vw in ((2, 0), (2, 2), (4, 0)):
        ctx.set_option("lusgs_systems", ns)
        ctx.set_option("lusgs_vw", vw)
        got = _lusgs_batch(ctx, FREQS, X)
        for q in range(len(FREQS)):
            assert np.all(np.isfinite(got[q])), (ns, vw, q)
            assert relerr(got[q], ref[q]) <= 1e-6, (ns, vw, q, relerr(got[q], ref[q]))
    ctx.set_option("lusgs_systems", 1)
    ctx.set_option("lusgs_vw", 0)


def test_grouped_sweeps_in_the_mixed_solve(gpu, tmp_path):
    """The batched mixed-precision solve with two systems of one frequency per CTA
    converges to the receivers of the single-system sweeps (the two preconditioners
    agree to rounding; both stop on the complex128 residual, 1e-8/f)."""
    cfg, G, ctx, O = _setup(tmp_path, *SHAPES[1])
    ctx.set_option("lusgs_split", 0)
    freqs = np.array(FREQS[:5], np.float32)
    src = np.repeat(cfg.acq.src[:1, :3], len(freqs), axis=0)
    src[:, 0] += np.arange(len(freqs), dtype=np.float32) * 37.0
    out = {}
    for ns in (1, 2, 4):
        ctx.set_option("lusgs_systems", ns)
        out[ns] = cs.solve_batch(ctx, freqs, src, rec=cfg.acq.rec, precision=32, preco=1, niter=1000, tol=1e-8)
        assert out[ns]["status"] == ["converged"] * len(freqs), (ns, out[ns]["status"])
    ctx.set_option("lusgs_systems", 1)
    for ns in (2, 4):
        for q in range(len(freqs)):
            assert relerr(out[ns]["dcal"][q], out[1]["dcal"][q]) <= 1e-6, (ns, q)


@pytest.mark.parametrize("shape", SHAPES + [(61, 12, 290, 9, 4, 0, 0)],
                         ids=[f"{s[1]}x{s[2]}x{s[3]}_air{s[5]}_fvm{s[6]}" for s in SHAPES + [(61, 12, 290, 9, 4, 0, 0)]])
def test_split_sweeps_match_pipelined_sweeps_and_oracle(gpu, tmp_path, shape):
    cfg, G, ctx, O = _setup(tmp_path, *shape)
    X = np.stack([probe(ctx.lE, shape[0] + 20 + q) for q in range(3)])
    freqs = FREQS[:3]
    ctx.set_option("lusgs_split", 0)
    ref = _lusgs_batch(ctx, freqs, X)
    for q, f in enumerate(freqs):
        O.set_freq(f)
        assert relerr(ref[q], O.lusgs(X[q])) <= 2e-5, q
    for vw in (1, 2, 4):
        ctx.set_option("lusgs_split", 1)
        ctx.set_option("lusgs_vw", vw)
        got = _lusgs_batch(ctx, freqs, X)
        for q in range(len(freqs)):
            assert np.all(np.isfinite(got[q])), (vw, q)
            assert relerr(got[q], ref[q]) <= 1e-6, (vw, q, relerr(got[q], ref[q]))
    ctx.set_option("lusgs_split", 1)
    ctx.set_option("lusgs_vw", 0)


def test_split_sweeps_in_the_mixed_solve(gpu, tmp_path):
    """The batched mixed-precision solve with the split sweeps converges to the receivers
    of the pipelined sweeps."""
    cfg, G, ctx, O = _setup(tmp_path, *SHAPES[1])
    freqs = np.array(FREQS[:4], np.float32)
    src = np.repeat(cfg.acq.src[:1, :3], len(freqs), axis=0)
    out = {}
    for split in (0, 1):
        ctx.set_option("lusgs_split", split)
        out[split] = cs.solve_batch(ctx, freqs, src, rec=cfg.acq.rec, precision=32, preco=1, niter=1000, tol=1e-8)
        assert out[split]["status"] == ["converged"] * len(freqs), (split, out[split]["status"])
    ctx.set_option("lusgs_split", 1)
    for q in range(len(freqs)):
        assert relerr(out[1]["dcal"][q], out[0]["dcal"][q]) <= 1e-6, q


@pytest.mark.parametrize("shape", [SHAPES[0], SHAPES[1], SHAPES[2]],
                         ids=[f"{s[1]}x{s[2]}x{s[3]}_air{s[5]}_fvm{s[6]}" for s in SHAPES[:3]])
def test_split_sweeps_on_two_streams_give_the_same_bits(gpu, tmp_path, shape):
    """With 8 or more systems the split sweeps run as two halves of the slots on two
    streams (lusgs_overlap, the default): each half's passes and pipelines are the same
    kernels on disjoint systems, so every system gets exactly the bits of the single-stream
    schedule. 9 systems at mixed frequencies: halves of 4 and 5, each with its own groups.
    The pipelines on two streams run a capped grid (lusgs_cap CTAs per SM) whose CTAs take
    lines in turn: with a cap of 1 the CTAs here take one to three lines each."""
    cfg, G, ctx, O = _setup(tmp_path, *shape)
    freqs = FREQS + [0.5, 1.0]
    X = np.stack([probe(ctx.lE, shape[0] + 30 + q) for q in range(len(freqs))])
    ctx.set_option("lusgs_overlap", 0)
    one = _lusgs_batch(ctx, freqs, X)
    ctx.set_option("lusgs_overlap", 1)
    for cap in (4, 1, 0):
        ctx.set_option("lusgs_cap", cap)
        two = _lusgs_batch(ctx, freqs, X)
        assert np.array_equal(one, two), cap
    ctx.set_option("lusgs_cap", 4)
    O.set_freq(freqs[3])
    assert relerr(two[3], O.lusgs(X[3])) <= 2e-5


def test_split_sweeps_on_two_streams_in_the_mixed_solve(gpu, tmp_path):
    """The batched mixed-precision solve of 10 systems (halves of 5 while all run) gives the
    same receivers, bit for bit, with one or two streams."""
    cfg, G, ctx, O = _setup(tmp_path, *SHAPES[1])
    freqs = np.array([0.5, 0.75, 1.0, 0.5, 0.75, 1.0, 0.5, 0.75, 1.0, 0.5], np.float32)
    src = np.repeat(cfg.acq.src[:1, :3], len(freqs), axis=0)
    src[:, 0] += np.arange(len(freqs), dtype=np.float32) * 29.0
    out = {}
    for ov in (0, 1):
        ctx.set_option("lusgs_overlap", ov)
        out[ov] = cs.solve_batch(ctx, freqs, src, rec=cfg.acq.rec, precision=32, preco=1, niter=1000, tol=1e-8)
        assert out[ov]["status"] == ["converged"] * len(freqs), (ov, out[ov]["status"])
    assert np.array_equal(out[0]["dcal"], out[1]["dcal"])
    assert np.array_equal(out[0]["iters"], out[1]["iters"])
