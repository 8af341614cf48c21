"""The CPU oracle and the product's host set-up, pinned against fixtures produced by the
reference itself (tests/golden, generated by tests/golden/make_golden.py from the
reference built from its sources). Runs anywhere, no GPU."""
import numpy as np
import pytest

from cases import GOLDEN_CASES, channels, load_golden, oracle_for, parse_args, product_grid, read_rows, tol_of

GRID_KEYS = ("x1", "x2", "x3", "x1s", "x2s", "x3s", "d1", "d2", "d3", "d1s", "d2s", "d3s",
             "sigma11", "sigma22", "sigma33")


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_host_setup_matches_reference(case):
    d, args, gold = load_golden(case)
    p = parse_args(args)
    G = product_grid(d, p)
    A = G.arrays()
    for k in GRID_KEYS:
        assert np.array_equal(A[k], gold[k]), k
    if "sH1" in gold:
        assert np.array_equal(A["sH1"], gold["sH1"])
        assert np.array_equal(A["sH2"], gold["sH2"])
    assert np.float32(G.g.rho_water) == np.float32(gold["rho_water"])


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_oracle_operators_bit_exact(case):
    d, args, gold = load_golden(case)
    p = parse_args(args)
    O = oracle_for(product_grid(d, p), p)
    O.set_freq(float(gold["freqs"][0]))
    x = gold["x"]
    assert np.array_equal(O.fdfd(x), gold["Ax"])
    preco = int(p.get("preco", 1))
    if preco == 1:
        assert np.array_equal(O.lusgs(x), gold["Mx"])
    elif preco == 3:
        assert np.array_equal(O.aphi(x), gold["Mx"])
    src = read_rows(f"{d}/sources.txt")[0]
    assert np.array_equal(O.inject(channels(p, "chsrc"), src), gold["b"])


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_oracle_solver_bit_exact(case):
    d, args, gold = load_golden(case)
    p = parse_args(args)
    O = oracle_for(product_grid(d, p), p)
    O.set_freq(float(gold["freqs"][0]))
    src = read_rows(f"{d}/sources.txt")[0]
    b = O.inject(channels(p, "chsrc"), src)
    x, hist, it = O.solve(b, algopt=int(p["algopt"]), precond=int(p["preco"]), niter=int(p["niter"]),
                          tol=tol_of(p, 0, gold["freqs"]), nrestart=int(p.get("nrestart", 10)),
                          mp=int(p.get("mp", 30)))
    assert np.array_equal(x, gold["x_solve"])
    printed = gold["hist_printed"]
    # the reference prints %e (7 significant digits) and not the final value
    np.testing.assert_allclose(hist[:len(printed)], printed, rtol=6e-7, atol=0)
    rec = read_rows(f"{d}/receivers.txt")
    out = O.extract(channels(p, "chrec"), rec, x)
    assert np.array_equal(out.astype(np.complex64), gold["dcal"])


def test_host_setup_matches_reference_at_bench_scale(tmp_path):
    """The product's set-up of the 96-system bench model (nb=10 stretched padding to
    120 km, the bottom-padding quirk of extend_model.c:169-173, 1024x1024 airwave
    filters) is bit-identical to the reference's: every array hashes to the checksum the
    reference's own set-up produced (tests/golden/make_setup_checksums.py). The oracle
    takes its model from the same host set-up library (oracle.pyoracle.setup_grid)."""
    import hashlib
    import json
    import os

    from cases import GOLDEN
    from demo_matrixfree_csem_gb300 import synthetic
    from oracle.pyoracle import setup_grid
    want = json.load(open(os.path.join(GOLDEN, "marlim_like_96", "setup_sha256.json")))
    cfg = synthetic.workload("marlim_like_96")
    synthetic.write_config(cfg, str(tmp_path))
    g = setup_grid(str(tmp_path), {k: str(v) for k, v in cfg.params.items()})
    assert (g.n1, g.n2, g.n3f, g.nb, g.n1fft, g.n2fft) == (want["n1"], want["n2"], want["n3"], want["nb"],
                                                          want["n1fft"], want["n2fft"])
    nv = want["valid_airwave_nodes"]  # the reference leaves the nodes past the model unwritten
    got = {k: hashlib.sha256(np.ascontiguousarray(getattr(g, k)[:nv[k]] if k in nv else getattr(g, k)).tobytes())
           .hexdigest() for k in want["sha256"]}
    bad = [k for k in want["sha256"] if got[k] != want["sha256"][k]]
    assert not bad, bad


@pytest.mark.parametrize("case", ["lusgs_air0", "lusgs_air1"])
def test_param_extended_export_matches_reference(case, tmp_path):
    """csem_grid_write_extended writes the padded model the reference exports with
    param_extended=1 (extend_model.c:254-289: resistivities and node coordinates as
    doubles), byte for byte."""
    import os

    from cases import GOLDEN
    d, args, gold = load_golden(case)
    G = product_grid(d, parse_args(args))
    G.write_extended(str(tmp_path))
    want = os.path.join(GOLDEN, case, "extended")
    for name in sorted(os.listdir(want)):
        assert open(os.path.join(tmp_path, name), "rb").read() == open(os.path.join(want, name), "rb").read(), name


@pytest.mark.parametrize("case", ["lusgs_air0", "plain_bicg_air0"])
def test_stencil_couplings_match_reference_assembled_operator(case):
    """Known answer from the reference's assembled operator (Acsr_init / Acsr_apply,
    Acsr.c:22-716, recorded by tests/golden/make_known_answers.py): on every interior
    row the assembled product equals I*omega*mu0 times the matrix-free one once each
    side's own diagonal term is taken out (the reference stores the assembled diagonal
    in column row - 1 with a different geometric part, so only the off-diagonal
    couplings are comparable)."""
    import os

    from cases import GOLDEN, relerr
    d, args, gold = load_golden(case)
    p = parse_args(args)
    O = oracle_for(product_grid(d, p), p)
    z = np.load(os.path.join(GOLDEN, case, "acsr.npz"))
    O.set_freq(float(z["freq"]))
    y = O.fdfd(z["x"])
    m = z["interior"]
    lhs = (z["Ax_csr"] - z["self_term"])[m]
    rhs = (complex(z["iom"]) * (y - z["fdfd_diag"] * z["x"]))[m]
    assert relerr(rhs, lhs) <= 1e-13


def _hy_overlap_case():
    import json
    import os

    from cases import GOLDEN
    d = os.path.join(GOLDEN, "hy_overlap")
    p = parse_args(json.load(open(os.path.join(d, "case.json"))))
    return d, p, np.load(os.path.join(d, "fdfd.npz"))


def test_oracle_reproduces_reference_hy_overlap():
    """Known answer (tests/golden/make_known_answers.py): on a model with n2 < n3 the
    reference's Hy scratch, sized n1*(n2+1)*n2 (fdfd.c:59), overlaps Hz, and its
    fdfd_apply mixes the two. The oracle at the reference's length reproduces that bit
    for bit; at the disjoint length n1*(n2+1)*n3 it gives another result, so the overlap
    is what changes it."""
    d, p, z = _hy_overlap_case()
    O = oracle_for(product_grid(d, p), p)
    assert O.g.n2 < O.n3
    O.set_freq(float(z["freq"]))
    assert np.array_equal(O.fdfd(z["x"]), z["Ax"])
    O.set_hy_length(False)
    assert not np.array_equal(O.fdfd(z["x"]), z["Ax"])


def test_hy_length_is_irrelevant_when_n2_at_least_n3():
    """The two Hy lengths give the same bits whenever the scratch does not overlap."""
    d, args, gold = load_golden("lusgs_air0")
    p = parse_args(args)
    O = oracle_for(product_grid(d, p), p)
    assert O.g.n2 >= O.n3
    O.set_freq(float(gold["freqs"][0]))
    a = O.fdfd(gold["x"])
    O.set_hy_length(False)
    assert np.array_equal(O.fdfd(gold["x"]), a)
