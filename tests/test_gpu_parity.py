"""GPU kernels against the oracle and the reference's golden fixtures, through the C ABI.

Tolerances:
  * complex128 operators, preconditioners, injection, extraction: bit-identical to the
    reference (no FFT involved) - asserted with array_equal;
  * anything through the airwave FFT (cuFFT vs the oracle's radix-2 DFT): max-norm
    relative difference <= 1e-12;
  * dot products (parallel tree vs sequential sum): <= 1e-13 relative;
  * complex64 operators vs the complex128 oracle: <= 2e-5 relative (max norm);
  * short FP64 solves (different dot summation order only): <= 1e-9 relative.
"""
import numpy as np
import pytest

import demo_matrixfree_csem_gb300 as cs
from cases import (GOLDEN_CASES, channels, load_golden, oracle_for, parse_args, probe, product_grid, read_rows,
                   relerr, tol_of)
from demo_matrixfree_csem_gb300 import synthetic

pytestmark = pytest.mark.gpu


def _ctx(case):
    d, args, gold = load_golden(case)
    p = parse_args(args)
    G = product_grid(d, p)
    return d, p, gold, G, cs.Ctx(G, int(p.get("airbc", 0)), int(p.get("fvm", 0)))


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_fdfd_apply_fp64(gpu, case):
    d, p, gold, G, ctx = _ctx(case)
    y = ctx.fdfd_apply(cs.iom_of(gold["freqs"][0]), gold["x"])
    if int(p.get("airbc", 0)):
        assert relerr(y, gold["Ax"]) <= 1e-12
    else:
        assert np.array_equal(y, gold["Ax"])


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_preconditioner_fp64_bit_exact(gpu, case):
    d, p, gold, G, ctx = _ctx(case)
    preco = int(p.get("preco", 1))
    if preco not in (1, 3):
        pytest.skip("no LU-SGS / A-phi in this case")
    iom = cs.iom_of(gold["freqs"][0])
    y = ctx.lusgs_apply(iom, gold["x"]) if preco == 1 else ctx.aphi_apply(iom, gold["x"])
    assert np.array_equal(y, gold["Mx"])


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_inject_extract_bit_exact(gpu, case):
    d, p, gold, G, ctx = _ctx(case)
    iom = cs.iom_of(gold["freqs"][0])
    src = read_rows(f"{d}/sources.txt")[0]
    b = ctx.inject_source(iom, channels(p, "chsrc"), src)
    assert np.array_equal(b, gold["b"])
    rec = read_rows(f"{d}/receivers.txt")
    out = ctx.extract_emf(channels(p, "chrec"), rec, gold["x_solve"])
    assert np.array_equal(out.astype(np.complex64), gold["dcal"])
    O = oracle_for(G, p)
    assert np.array_equal(out, O.extract(channels(p, "chrec"), rec, gold["x_solve"]))


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_short_solve_tracks_reference(gpu, case):
    """The GPU solve differs from the reference only in the summation order of its dot
    products. How far that moves the iterate depends on the system: the tolerance is the
    larger of 1e-9 and 100x the change the oracle itself shows when b is perturbed by
    one ulp (some small cases here, e.g. unpreconditioned BiCGStab, are chaotic)."""
    d, p, gold, G, ctx = _ctx(case)
    iom = cs.iom_of(gold["freqs"][0])
    b = gold["b"]
    kw = dict(algopt=int(p["algopt"]), niter=int(p["niter"]), tol=tol_of(p, 0, gold["freqs"]),
              nrestart=int(p.get("nrestart", 10)), mp=int(p.get("mp", 30)))
    x, hist, it, st = ctx.solve_fp64(iom, b, preco=int(p["preco"]), **kw)
    O = oracle_for(G, p)
    O.set_freq(float(gold["freqs"][0]))
    x0, h0, _ = O.solve(b, precond=int(p["preco"]), **kw)
    assert np.array_equal(x0, gold["x_solve"])
    x1, h1, _ = O.solve(b * (1 + 2.0 ** -52), precond=int(p["preco"]), **kw)
    sens = relerr(x1, x0)
    assert relerr(x, gold["x_solve"]) <= max(1e-9, 100 * sens)
    printed = gold["hist_printed"]
    if sens < 1e-10:
        np.testing.assert_allclose(hist[:len(printed)], printed, rtol=2e-6)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_reference_order_dots_reproduce_reference_solve(gpu, case):
    """dot_order=1: dot products in the reference's sequential order. Then the complex128
    solve repeats the reference's arithmetic: without airbc its iterate is the reference's
    (the fixture's x_solve) bit for bit, and its residual history and iteration count are
    the oracle's exactly; with airbc only the airwave FFT's rounding differs (cuFFT
    against the DFT the oracle and the fixtures use), bounded as the short solves above."""
    d, p, gold, G, ctx = _ctx(case)
    ctx.set_option("dot_order", 1)
    iom = cs.iom_of(gold["freqs"][0])
    b = gold["b"]
    kw = dict(algopt=int(p["algopt"]), niter=int(p["niter"]), tol=tol_of(p, 0, gold["freqs"]),
              nrestart=int(p.get("nrestart", 10)), mp=int(p.get("mp", 30)))
    x, hist, it, st = ctx.solve_fp64(iom, b, preco=int(p["preco"]), **kw)
    O = oracle_for(G, p)
    O.set_freq(float(gold["freqs"][0]))
    x0, h0, it0 = O.solve(b, precond=int(p["preco"]), **kw)
    if int(p.get("airbc", 0)) == 0:
        assert np.array_equal(x, gold["x_solve"])
        assert it == it0 and np.array_equal(hist[:len(h0)], h0), (it, it0)
    else:
        x1, _, _ = O.solve(b * (1 + 2.0 ** -52), precond=int(p["preco"]), **kw)
        assert relerr(x, gold["x_solve"]) <= max(1e-9, 100 * relerr(x1, x0))


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_c64_operators_close_to_fp64(gpu, case):
    d, p, gold, G, ctx = _ctx(case)
    iom = cs.iom_of(gold["freqs"][0])
    x = gold["x"]
    assert relerr(ctx.fdfd_apply(iom, x, c64=True), gold["Ax"]) <= 2e-5
    preco = int(p.get("preco", 1))
    if preco == 1:
        assert relerr(ctx.lusgs_apply(iom, x, c64=True), gold["Mx"]) <= 2e-5
    elif preco == 3:
        assert relerr(ctx.aphi_apply(iom, x, c64=True), gold["Mx"]) <= 2e-5


@pytest.mark.parametrize("airbc,fvm", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_larger_grid_bit_exact(gpu, tmp_path, airbc, fvm):
    """A grid spanning several CTAs in every direction and several k-chunks."""
    cfg = synthetic.random_small(21 + airbc + 2 * fvm, nx=40, ny=27, nz=19, nb=4, airbc=airbc, fvm=fvm,
                                 n1fft=64, n2fft=64)
    synthetic.write_config(cfg, str(tmp_path))
    p = dict(cfg.params, nb=4)
    G = product_grid(str(tmp_path), {k: str(v) for k, v in p.items()})
    ctx = cs.Ctx(G, airbc, fvm)
    O = oracle_for(G, {k: str(v) for k, v in p.items()})
    f = 0.75
    O.set_freq(f)
    iom = cs.iom_of(f)
    x = probe(ctx.lE, 5)
    ya = ctx.fdfd_apply(iom, x)
    yo = O.fdfd(x)
    if airbc:
        assert relerr(ya, yo) <= 1e-12
    else:
        assert np.array_equal(ya, yo)
    mo = O.lusgs(x)
    # lockstep row pipelines (any points-per-thread width) and one launch per diagonal
    # visit the points in dependency order with the same arithmetic: same bits
    for sched, vw in ((1, 0), (1, 1), (1, 2), (1, 4), (0, 0)):
        ctx.set_option("lusgs_pipelined", sched)
        ctx.set_option("lusgs_vw", vw)
        assert np.array_equal(ctx.lusgs_apply(iom, x), mo), (sched, vw)
        assert relerr(ctx.lusgs_apply(iom, x, c64=True), mo) <= 2e-5, (sched, vw)
    ctx.set_option("lusgs_pipelined", 1)
    ctx.set_option("lusgs_vw", 0)


@pytest.mark.parametrize("airbc", [0, 1])
def test_tall_grid_lusgs_bit_exact(gpu, tmp_path, airbc):
    """More than 256 rows in the Ez sweep (n2 - 1 > 256): CTAs of up to 512 threads that
    hand over through a CTA barrier instead of the named-barrier pairs."""
    cfg = synthetic.random_small(61 + airbc, nx=12, ny=290, nz=9, nb=4, airbc=airbc, n1fft=32, n2fft=512)
    synthetic.write_config(cfg, str(tmp_path))
    p = {k: str(v) for k, v in cfg.params.items()}
    G = product_grid(str(tmp_path), p)
    ctx = cs.Ctx(G, airbc, 0)
    assert ctx.n2 - 1 > 256
    O = oracle_for(G, p)
    O.set_freq(0.5)
    iom = cs.iom_of(0.5)
    x = probe(ctx.lE, 8)
    mo = O.lusgs(x)
    for vw in (1, 2):
        ctx.set_option("lusgs_vw", vw)
        assert np.array_equal(ctx.lusgs_apply(iom, x), mo), vw
        assert relerr(ctx.lusgs_apply(iom, x, c64=True), mo) <= 2e-5, vw
    ctx.set_option("lusgs_vw", 0)


@pytest.mark.parametrize("airbc", [0, 1])
def test_aphi_larger_grid_bit_exact(gpu, tmp_path, airbc):
    cfg = synthetic.random_small(31 + airbc, nx=33, ny=21, nz=17, nb=3, airbc=airbc, n1fft=32, n2fft=32, preco=3)
    synthetic.write_config(cfg, str(tmp_path))
    p = {k: str(v) for k, v in cfg.params.items()}
    G = product_grid(str(tmp_path), p)
    ctx = cs.Ctx(G, airbc, 0)
    O = oracle_for(G, p)
    O.set_freq(1.0)
    x = probe(ctx.lE, 6)
    assert np.array_equal(ctx.aphi_apply(cs.iom_of(1.0), x), O.aphi(x))


def test_airwave_ghosts(gpu, tmp_path):
    cfg = synthetic.random_small(41, nx=30, ny=26, nz=10, nb=4, airbc=1, n1fft=128, n2fft=128)
    synthetic.write_config(cfg, str(tmp_path))
    p = {k: str(v) for k, v in cfg.params.items()}
    G = product_grid(str(tmp_path), p)
    ctx = cs.Ctx(G, 1, 0)
    O = oracle_for(G, p)
    hz0 = probe(ctx.n1 * ctx.n2, 7)
    hx, hy = ctx.airbc_apply(hz0)
    ox, oy = O.airbc(hz0)
    assert relerr(hx, ox) <= 1e-12 and relerr(hy, oy) <= 1e-12


def test_dot_products(gpu):
    from oracle import Oracle
    rng = np.random.default_rng(3)
    for n in (1, 31, 1000, 300001):
        a = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        ref = Oracle.cdot(a, b)
        got = cs.cdot(a, b)
        assert abs(got - ref) <= 1e-13 * np.sqrt(n) * np.abs(a).max() * np.abs(b).max() * 4
        a32, b32 = a.astype(np.complex64), b.astype(np.complex64)
        exact = np.sum(a32.astype(np.complex128) * np.conj(b32.astype(np.complex128)))
        got32 = cs.cdot(a32, b32, c64=True)
        assert abs(got32 - exact) <= 1e-12 * np.sum(np.abs(a32) * np.abs(b32)) + 1e-300
    # deterministic: the same call twice gives the same bits
    a = rng.standard_normal(50000) + 1j * rng.standard_normal(50000)
    assert cs.cdot(a, a[::-1].copy()) == cs.cdot(a, a[::-1].copy())


def test_gmres_preconditioner(gpu):
    d, p, gold, G, ctx = _ctx("gmrespre_air0")
    O = oracle_for(G, p)
    O.set_freq(float(gold["freqs"][0]))
    y = ctx.gmres_apply(cs.iom_of(gold["freqs"][0]), gold["x"], mp=5)
    assert relerr(y, O.gmres_pre(gold["x"], 5)) <= 1e-10


@pytest.mark.parametrize("case", ["lusgs_air0", "plain_bicg_air0"])
def test_stencil_couplings_match_reference_assembled_operator(gpu, case):
    """The GPU stencil against the reference's assembled operator (Acsr_apply after
    Acsr_init, Acsr.c:22-716; fixture from tests/golden/make_known_answers.py): every
    off-diagonal coupling of every interior row agrees, up to the factor I*omega*mu0 the
    assembled form carries, to 1e-13 (the two sum the same terms in different orders).
    The assembled diagonal is not comparable: the reference stores it in column row - 1
    with a different geometric part."""
    import os

    from cases import GOLDEN
    d, p, gold, G, ctx = _ctx(case)
    z = np.load(os.path.join(GOLDEN, case, "acsr.npz"))
    y = ctx.fdfd_apply(cs.iom_of(float(z["freq"])), z["x"])
    m = z["interior"]
    lhs = (z["Ax_csr"] - z["self_term"])[m]
    rhs = (complex(z["iom"]) * (y - z["fdfd_diag"] * z["x"]))[m]
    assert relerr(rhs, lhs) <= 1e-13


def test_fdfd_keeps_h_disjoint_where_reference_overlaps(gpu):
    """Where n2 < n3 the reference's Hy scratch (n1*(n2+1)*n2 long, fdfd.c:59) overlaps
    Hz and its fdfd_apply mixes them (known answer tests/golden/hy_overlap/fdfd.npz). The
    GPU stencil never stores H, so it computes the curl-curl operator that the reference
    computes whenever n2 >= n3: bit-identical to the oracle at the disjoint Hy length, and
    different from the reference's overlapped result."""
    import json
    import os

    from cases import GOLDEN
    d = os.path.join(GOLDEN, "hy_overlap")
    p = parse_args(json.load(open(os.path.join(d, "case.json"))))
    z = np.load(os.path.join(d, "fdfd.npz"))
    G = product_grid(d, p)
    ctx = cs.Ctx(G, 0, 0)
    assert ctx.n2 < ctx.n3
    O = oracle_for(G, p)
    O.set_hy_length(False)
    O.set_freq(float(z["freq"]))
    y = ctx.fdfd_apply(cs.iom_of(float(z["freq"])), z["x"])
    assert np.array_equal(y, O.fdfd(z["x"]))
    assert not np.array_equal(y, z["Ax"])
