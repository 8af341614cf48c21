"""The C ABI library loads without a GPU and exports every function its headers declare."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# csem_refabi.h declares the reference's own symbol names, exported by libcsem_refabi.so
REFABI_HEADERS = ("csem_refabi.h",)


def declared_functions(headers=None):
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h") or (headers is not None and h not in headers):
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(\w+)\s*\([^;{]*\)\s*;", src, flags=re.M):
            if not m.group(0).lstrip().startswith(("typedef", "#")):
                names.add(m.group(1))
    return sorted(names)


def test_headers_declare_entry_points():
    names = declared_functions()
    assert "csem_fdfd_apply_host" in names and "csem_grid_extend" in names and len(names) > 30


def test_library_exports_every_declared_symbol(csem_lib):
    own = [h for h in os.listdir(os.path.join(ROOT, "include")) if h.endswith(".h") and h not in REFABI_HEADERS]
    lib = ctypes.CDLL(csem_lib._name)
    missing = [n for n in declared_functions(own) if not hasattr(lib, n)]
    assert not missing, missing
    from demo_matrixfree_csem_gb300 import build
    ref = ctypes.CDLL(build.REFABI)
    missing = [n for n in declared_functions(REFABI_HEADERS) if not hasattr(ref, n)]
    assert not missing, missing


def test_no_device_is_reported_not_faked(csem_lib):
    import demo_matrixfree_csem_gb300 as cs
    if cs.device_count() > 0:
        pytest.skip("a GPU is visible")
    from cases import GOLDEN_CASES, load_golden, parse_args, product_grid
    d, args, gold = load_golden(GOLDEN_CASES[0])
    G = product_grid(d, parse_args(args))
    with pytest.raises(cs.CsemError) as e:
        cs.Ctx(G, 0, 0)
    assert e.value.code == -6
    with pytest.raises(cs.CsemError):
        cs.cdot(np.ones(4), np.ones(4))


def test_getpar_semantics(csem_lib, tmp_path):
    import demo_matrixfree_csem_gb300 as cs
    L = cs.lib()
    pf = tmp_path / "par.txt"
    pf.write_text("nb=7 freqs=1,2 'name=a b'\n tol=1e-3\n")
    argv = [b"prog", b"nb=3", b"freqs=0.25,0.75,1.25", b"junk", b"nb=10", f"par={pf}".encode(), b"rho_air=1e6"]
    arr = (ctypes.c_char_p * len(argv))(*argv)
    L.csem_initargs(len(argv), arr)
    v = ctypes.c_int()
    assert L.csem_getparint(b"nb", ctypes.byref(v)) == 1 and v.value == 10   # last occurrence wins
    assert L.csem_countparval(b"freqs") == 3                                    # command line overrides par file
    f = (ctypes.c_float * 3)()
    assert L.csem_getparfloat(b"freqs", f) == 3
    assert f[0] == np.float32(0.25) and f[2] == np.float32(1.25)
    t = ctypes.c_float()
    assert L.csem_getparfloat(b"tol", ctypes.byref(t)) == 1 and t.value == np.float32(1e-3)  # from par file
    assert L.csem_getparint(b"missing", ctypes.byref(v)) == 0


def test_freq_sort_and_emf_writer(csem_lib, tmp_path):
    import demo_matrixfree_csem_gb300 as cs
    L = cs.lib()
    f = np.array([1.25, 0.25, 0.75], np.float32)
    L.csem_sort_freqs(f.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), 3)
    assert list(f) == [np.float32(0.25), np.float32(0.75), np.float32(1.25)]
    d = np.arange(2 * 3 * 2, dtype=np.complex64).reshape(2, 3, 2) * (1.5 - 0.5j)
    fn = str(tmp_path / "emf_0001.txt")
    assert L.csem_write_emf(fn.encode(), 1, 2, 3, 2, d.view(np.float32).ctypes.data_as(ctypes.POINTER(ctypes.c_float))) == 0
    lines = open(fn).read().splitlines()
    assert lines[0] == "iTx \t iRx    ichrec  ifreq \t emf_real \t emf_imag"
    assert lines[1] == "1 \t 1 \t 1 \t 1 \t %e \t %e" % (d[0, 0, 0].real, d[0, 0, 0].imag)
    assert lines[4] == "1 \t 2 \t 1 \t 2 \t %e \t %e" % (d[0, 1, 1].real, d[0, 1, 1].imag)
    assert len(lines) == 1 + 12


def test_input_errors_are_codes(csem_lib, tmp_path):
    import demo_matrixfree_csem_gb300 as cs
    with pytest.raises(cs.CsemError) as e:
        cs.Grid.from_files(*(str(tmp_path / n) for n in ("fx1", "fx2", "fx3", "r1", "r2", "r3")))
    assert e.value.code == -2
    (tmp_path / "fx1").write_bytes(np.arange(4, dtype=np.float32).tobytes())
    (tmp_path / "fx2").write_bytes(np.arange(4, dtype=np.float32).tobytes())
    (tmp_path / "fx3").write_bytes(np.arange(4, dtype=np.float32).tobytes())
    for n in ("r1", "r2", "r3"):
        (tmp_path / n).write_bytes(np.ones(20, np.float32).tobytes())  # 27 needed: short file
    with pytest.raises(cs.CsemError) as e:
        cs.Grid.from_files(*(str(tmp_path / n) for n in ("fx1", "fx2", "fx3", "r1", "r2", "r3")))
    assert e.value.code == -2 and "size not match" in str(e.value)


def test_history_logging_rule(csem_lib):
    """How many residual-history entries the reference writes to iterate_*.txt
    (csem_history_logged): BiCGStab never logs the last residual it computed; gmres does
    not log a converged one, fgmres does; a zero right-hand side logs nothing."""
    import demo_matrixfree_csem_gb300 as cs
    f = cs.lib().csem_history_logged
    f.argtypes = [ctypes.c_int] * 4
    CONV, MAXIT, ZERO = 1, 2, 5
    assert f(1, 1, CONV, 5) == 4      # converged in the 4th step: initial + 3 logged
    assert f(1, 0, MAXIT, 9) == 8     # niter=8: initial + steps 1..7
    assert f(1, 1, MAXIT, 1) == 1     # niter=0: the initial residual only
    assert f(2, 0, CONV, 12) == 11    # gmres: the converged residual is not logged
    assert f(2, 3, CONV, 12) == 12    # fgmres: it is
    assert f(2, 0, MAXIT, 31) == 31
    assert f(1, 1, ZERO, 0) == 0 and f(2, 3, ZERO, 1) == 0


def test_batch_options_are_checked_before_any_device_work(csem_lib):
    """csem_solve_batch_host rejects option combinations the solvers cannot run with
    CSEM_EINVAL before it touches the context or the GPU: GMRES without a restart length
    (the reference runs niter / nrestart cycles, main.c:106,109), the inner-GMRES
    preconditioner without steps, preconditioners and algorithms out of range, for both
    precisions."""
    import demo_matrixfree_csem_gb300 as cs
    from demo_matrixfree_csem_gb300.api import _BatchOpts
    L = cs.lib()
    f = np.array([1.0], np.float32)
    s = np.zeros(3, np.float32)
    ch = np.zeros(1, np.int32)
    out = np.zeros(2)
    it = np.zeros(1, np.int32)

    def call(**kw):
        d = dict(precision=64, algopt=1, preco=1, niter=10, tol=1e-8, inner_tol=0.2, check_every=4, max_outer=30,
                 nrestart=10, mp=30)
        d.update(kw)
        o = _BatchOpts(*[d[k] for k in ("precision", "algopt", "preco", "niter", "tol", "inner_tol", "check_every",
                                        "max_outer", "nrestart", "mp")])
        fp = ctypes.POINTER(ctypes.c_float)
        ip = ctypes.POINTER(ctypes.c_int)
        dp = ctypes.POINTER(ctypes.c_double)
        return L.csem_solve_batch_host(None, 1, f.ctypes.data_as(fp), s.ctypes.data_as(fp), 1, ch.ctypes.data_as(ip),
                                       1, ch.ctypes.data_as(ip), 0, s.ctypes.data_as(fp), ctypes.byref(o),
                                       out.ctypes.data_as(dp), it.ctypes.data_as(ip), it.ctypes.data_as(ip),
                                       it.ctypes.data_as(ip), out.ctypes.data_as(dp))

    EINVAL = -1
    assert call(precision=64, algopt=2, nrestart=0) == EINVAL
    assert call(precision=64, preco=2, mp=0) == EINVAL
    assert call(precision=64, preco=4) == EINVAL
    assert call(precision=64, algopt=3) == EINVAL
    assert call(precision=32, algopt=2, nrestart=0) == EINVAL
    assert call(precision=32, preco=2) == EINVAL
    assert call(precision=16) == EINVAL


def test_sweep_groups_partition_the_slots_by_frequency():
    """csem_sweep_groups: the groups the batched complex64 LU-SGS uses (host logic only)."""
    from demo_matrixfree_csem_gb300 import api
    a, b, c = 1j * 3.9e-6, 1j * 5.9e-6, 1j * 7.9e-6
    iom = [a, b, a, c, a, b, a, a, c]
    g, na, nga = api.sweep_groups(iom, 2)
    assert g.tolist() == [[0, 2], [4, 6], [7, -1], [1, 5], [3, 8]] and (na, nga) == (0, 0)
    g16, _, _ = api.sweep_groups(iom, 16)
    assert [sorted(x for x in r if x >= 0) for r in g16.tolist()] == [[0, 2, 4, 6, 7], [1, 5], [3, 8]]
    # two halves of the slots, each numbered from 0 (the split sweeps on two streams)
    g, na, nga = api.sweep_groups(iom, 2, halves=True)
    assert (na, nga) == (4, 3)
    assert g.tolist() == [[0, 2], [1, -1], [3, -1], [0, 2], [3, -1], [1, -1], [4, -1]]
    for lo, hi, rows in ((0, na, g[:nga]), (na, len(iom), g[nga:])):
        members = sorted(x for r in rows for x in r if x >= 0)
        assert members == list(range(hi - lo))
        for r in rows:
            assert len({iom[lo + x] for x in r if x >= 0}) == 1
    # fewer than 8 slots: one set
    g, na, nga = api.sweep_groups(iom[:7], 4, halves=True)
    assert (na, nga) == (0, 0) and sorted(x for r in g.tolist() for x in r if x >= 0) == list(range(7))
