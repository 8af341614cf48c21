"""The same-symbol drop-in (libcsem_refabi.so) on the GPU, called the way the reference's
driver calls its hot path (main.c:93-123), without the reference's sources.

emf_t and acq_t are filled here from the product's host set-up (bit-identical to the
reference's extend_model_init, tests/test_oracle_golden.py) in the layout of
include/csem_refabi.h, which restates the reference's emf.h / acq.h. Then, per golden
case without airwave:
  fdfd_init(emf)                                    fdfd.c:30
  inject_source(acq, emf, b)                        inject_extract.c:24
  bicgstab / fbicgstab / gmres / fgmres with the
  library's own fdfd_apply / lusgs_apply /
  gmres_apply / aphi_apply as callbacks             solver.c:16-512, main.c:104-118
  extract_emf(acq, emf, x, 0)                       inject_extract.c:123
and b, x, the iterate_*.txt history and dcal_fd must equal the reference's golden
values. With CSEM_DOT_ORDER=1 the library's dot products run in the reference's order,
so x, the history and the receivers are bit-identical; with the default parallel tree
x is within max(1e-9, 100x the oracle's own one-ulp sensitivity) relative.
"""
import ctypes as C
import os

import numpy as np
import pytest

import demo_matrixfree_csem_gb300 as cs
from cases import load_golden, parse_args, product_grid, read_rows, relerr

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_z = C.c_double * 2
_zf = C.c_float * 2


class Emf(C.Structure):
    """emf_t of include/csem_refabi.h (the reference's emf.h:4-57)."""
    _fields_ = [("mode", C.c_int), ("verb", C.c_int), ("reciprocity", C.c_int), ("fvm", C.c_int),
                ("airbc", C.c_int), ("nfreq", C.c_int), ("freqs", _fp),
                ("rho_air", C.c_float), ("lextend", C.c_float), ("rho_water", C.c_float),
                ("rhomin", C.c_float), ("rhomax", C.c_float), ("nchsrc", C.c_int), ("nchrec", C.c_int),
                ("chsrc", C.POINTER(C.c_char_p)), ("chrec", C.POINTER(C.c_char_p)),
                ("istretch", C.c_int), ("rstretch", C.c_float),
                ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("nb", C.c_int),
                ("n1", C.c_int), ("n2", C.c_int), ("n3", C.c_int)] + \
               [(n, C.c_int) for n in ("lv", "lE", "lH", "lEx", "lEy", "lEz", "lHx", "lHy", "lHz")] + \
               [(n, _fp) for n in ("x1node", "x2node", "x3node")] + \
               [(n, _dp) for n in ("x1", "x2", "x3", "x1s", "x2s", "x3s", "d1", "d2", "d3", "d1s", "d2s", "d3s")] + \
               [(n, C.c_double) for n in ("d1min", "d2min", "d3min", "x1min", "x2min", "x3min", "x1max",
                                          "x2max", "x3max")] + \
               [("n1fft", C.c_int), ("n2fft", C.c_int), ("d1fft", C.c_double), ("d2fft", C.c_double),
                ("d3fft", C.c_double), ("sH1kxky", C.c_void_p), ("sH2kxky", C.c_void_p),
                ("rho11", C.c_void_p), ("rho22", C.c_void_p), ("rho33", C.c_void_p),
                ("sigma11", C.c_void_p), ("sigma22", C.c_void_p), ("sigma33", C.c_void_p),
                ("E1", C.c_void_p), ("E2", C.c_void_p), ("E3", C.c_void_p), ("dcal_fd", C.c_void_p),
                ("ne", C.c_int), ("nh", C.c_int), ("xe", C.c_void_p), ("xh", C.c_void_p), ("be", C.c_void_p),
                ("v", C.c_void_p), ("bv", C.c_void_p), ("xx", C.c_void_p), ("yy", C.c_void_p),
                ("I_omega_mu0", _z), ("preco", C.c_int), ("algopt", C.c_int), ("niter", C.c_int),
                ("nrestart", C.c_int), ("mp", C.c_int), ("tol", C.c_float), ("param_extended", C.c_int)]


class Acq(C.Structure):
    """acq_t of include/csem_refabi.h (the reference's acq.h:4-19)."""
    _fields_ = [("nsrc", C.c_int), ("nrec", C.c_int), ("nsubsrc", C.c_int), ("nsubrec", C.c_int),
                ("lensrc", C.c_float), ("lenrec", C.c_float)] + \
               [(n, _fp) for n in ("src_x1", "src_x2", "src_x3", "src_azimuth", "src_dip",
                                   "rec_x1", "rec_x2", "rec_x3", "rec_azimuth", "rec_dip")] + \
               [(n, C.c_float) for n in ("x1min", "x1max", "x2min", "x2max", "x3min", "x3max")] + \
               [("nsrc_total", C.c_int), ("nrec_total", C.c_int), ("shot_idx", C.c_void_p)]


def _refabi():
    from demo_matrixfree_csem_gb300 import build
    cs.lib()
    L = C.CDLL(build.REFABI)
    L.csem_refabi_layout.argtypes = [C.POINTER(C.c_long)]
    return L


def test_ctypes_mirror_matches_library_layout(csem_lib):
    """The structs above have the library's (hence the reference's) sizes and offsets."""
    L = _refabi()
    out = (C.c_long * 8)()
    L.csem_refabi_layout(out)
    assert list(out) == [C.sizeof(Emf), C.sizeof(Acq), Emf.sigma11.offset, Emf.I_omega_mu0.offset,
                         Emf.dcal_fd.offset, Emf.param_extended.offset, Acq.rec_x1.offset, Acq.shot_idx.offset]


class _Model:
    """emf_t / acq_t of one golden case and the buffers they point into."""

    def __init__(self, case):
        d, args, gold = load_golden(case)
        p = parse_args(args)
        self.p, self.gold = p, gold
        self.G = G = product_grid(d, p)
        A = G.arrays()
        g = G.g
        keep = []

        def arr(a, t):
            a = np.ascontiguousarray(a)
            keep.append(a)
            return a.ctypes.data_as(t)

        def ptr3(a):  # a double*** whose [0][0][0] is the contiguous array (all fdfd_init reads)
            p1 = (C.c_void_p * 1)(a.ctypes.data)
            p2 = (C.c_void_p * 1)(C.addressof(p1))
            keep.extend([a, p1, p2])
            return C.addressof(p2)

        e = Emf()
        e.fvm, e.airbc = int(p.get("fvm", 0)), int(p.get("airbc", 0))
        self.freqs = np.asarray([float(f) for f in p["freqs"].split(",")], np.float32)
        e.nfreq, e.freqs = len(self.freqs), arr(self.freqs, _fp)
        e.rho_air, e.lextend, e.rho_water = g.rho_air, g.lextend, g.rho_water
        self.chsrc = [c.encode() for c in p.get("chsrc", "Ex").split(",")]
        self.chrec = [c.encode() for c in p.get("chrec", "Ex").split(",")]
        cs_ = (C.c_char_p * len(self.chsrc))(*self.chsrc)
        cr_ = (C.c_char_p * len(self.chrec))(*self.chrec)
        keep += [cs_, cr_]
        e.nchsrc, e.chsrc, e.nchrec, e.chrec = len(self.chsrc), cs_, len(self.chrec), cr_
        e.nx, e.ny, e.nz, e.nb = g.nx, g.ny, g.nz, g.nb
        e.n1, e.n2, e.n3 = g.n1, g.n2, g.n3
        for nm in ("x1node", "x2node", "x3node"):
            setattr(e, nm, getattr(g, nm))
        for nm in ("x1", "x2", "x3", "x1s", "x2s", "x3s", "d1", "d2", "d3", "d1s", "d2s", "d3s"):
            setattr(e, nm, arr(A[nm], _dp))
        e.sigma11, e.sigma22, e.sigma33 = ptr3(A["sigma11"]), ptr3(A["sigma22"]), ptr3(A["sigma33"])
        e.preco, e.algopt, e.niter = int(p.get("preco", 1)), int(p.get("algopt", 1)), int(p.get("niter", 1000))
        e.nrestart, e.mp, e.tol = int(p.get("nrestart", 10)), int(p.get("mp", 30)), float(p.get("tol", 1e-8))
        src = read_rows(os.path.join(d, "sources.txt"))[:1]
        rec = read_rows(os.path.join(d, "receivers.txt"))
        a = Acq()
        a.nsrc, a.nrec = 1, len(rec)  # the reference solves the first source row (acq_init_free.c:56,90)
        for q, nm in enumerate(("src_x1", "src_x2", "src_x3", "src_azimuth", "src_dip")):
            setattr(a, nm, arr(src[:, q].astype(np.float32), _fp))
        for q, nm in enumerate(("rec_x1", "rec_x2", "rec_x3", "rec_azimuth", "rec_dip")):
            setattr(a, nm, arr(rec[:, q].astype(np.float32), _fp))
        # dcal_fd[nchrec][nfreq][nrec] complex64 (emf.h:42), as alloc3complexf lays it out
        self.dcal = np.zeros((len(self.chrec), len(self.freqs), len(rec)), np.complex64)
        rows = [(C.c_void_p * len(self.freqs))(*[self.dcal[c, f].ctypes.data for f in range(len(self.freqs))])
                for c in range(len(self.chrec))]
        top = (C.c_void_p * len(rows))(*[C.addressof(r) for r in rows])
        keep += [self.dcal, rows, top]
        e.dcal_fd = C.addressof(top)
        self.emf, self.acq, self.keep = e, a, keep


@pytest.mark.gpu
@pytest.mark.parametrize("dot_order", [1, 0])
@pytest.mark.parametrize("case", ["lusgs_air0", "plain_bicg_air0", "gmrespre_air0", "plain_gmres_air0",
                                  "aphi_air0_fvm"])
def test_same_symbol_library_runs_reference_calls(gpu, tmp_path, monkeypatch, case, dot_order):
    L = _refabi()
    monkeypatch.setenv("CSEM_DOT_ORDER", str(dot_order))
    monkeypatch.chdir(tmp_path)  # iterate_*.txt is written to the working directory
    M = _Model(case)
    e, acq, gold = M.emf, M.acq, M.gold
    L.fdfd_init(C.byref(e))
    try:
        info = gold["info"]
        assert (e.n1, e.n2, e.n3, e.lE) == (info[0], info[1], info[2], info[7])
        f0 = M.freqs[0]
        e.I_omega_mu0 = _z(0.0, cs.iom_of(f0).imag)  # main.c:95
        b = np.zeros(e.lE, np.complex128)
        L.inject_source(C.byref(acq), C.byref(e), b.ctypes.data_as(C.c_void_p))
        assert np.array_equal(b, gold["b"])
        x = np.zeros(e.lE, np.complex128)
        tol = C.c_double(float(np.float32(e.tol) / np.float32(f0)))  # main.c:94, in float
        op = lambda name: C.cast(getattr(L, name), C.c_void_p)  # noqa: E731
        A = op("fdfd_apply")
        Mop = {1: "lusgs_apply", 2: "gmres_apply", 3: "aphi_apply"}.get(e.preco)
        xp, bp = x.ctypes.data_as(C.c_void_p), b.ctypes.data_as(C.c_void_p)
        if e.preco == 2:
            L.gmres_init(e.lE, e.mp, A)
        if e.algopt == 1 and e.preco == 0:
            L.bicgstab(e.lE, xp, bp, A, e.niter, tol, 1)
            hfile = "iterate_bicgstab.txt"
        elif e.algopt == 1:
            L.fbicgstab(e.lE, xp, bp, A, op(Mop), e.niter, tol, 1)
            hfile = "iterate_fbicgstab.txt"
        elif e.preco == 0:
            L.gmres(e.lE, xp, bp, A, e.niter // e.nrestart, tol, e.nrestart, 1)
            hfile = "iterate_gmres.txt"
        else:
            L.fgmres(e.lE, xp, bp, A, op(Mop), e.niter // e.nrestart, tol, e.nrestart, 1)
            hfile = "iterate_fgmres.txt"
        if e.preco == 2:
            L.gmres_free()
        hist = [float(ln.split()[1]) for ln in open(hfile).read().splitlines()[1:]]
        L.extract_emf(C.byref(acq), C.byref(e), xp, 0)
        dcal = M.dcal[:, 0, :]
        if dot_order == 1:
            assert np.array_equal(x, gold["x_solve"])
            assert hist == [float(v) for v in gold["hist_printed"]]
            assert np.array_equal(dcal, gold["dcal"])
        else:
            # tree-order dots move the iterate by rounding only; how far that goes depends on
            # the system (unpreconditioned BiCGStab is chaotic here): the bound is the larger
            # of 1e-9 and 100x the change the oracle shows when b moves by one ulp
            from cases import oracle_for
            O = oracle_for(M.G, M.p)
            O.set_freq(float(f0))
            kw = dict(algopt=e.algopt, precond=e.preco, niter=e.niter, tol=tol.value, nrestart=e.nrestart, mp=e.mp)
            x0, _, _ = O.solve(gold["b"], **kw)
            x1, _, _ = O.solve(gold["b"] * (1 + 2.0 ** -52), **kw)
            bound = max(1e-9, 100 * relerr(x1, x0))
            assert relerr(x, gold["x_solve"]) <= bound
            assert len(hist) == len(gold["hist_printed"])
            assert relerr(dcal, gold["dcal"]) <= max(1e-6, bound)  # complex64 receivers
    finally:
        L.fdfd_free(C.byref(e))
