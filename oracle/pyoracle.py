"""ctypes access to the CPU oracle and to the reference built from its sources.

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py)."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "libcsemoracle.so")
# CSEM_REF_VARIANT=fma selects the multiply-add-contracting build (build_ref.sh)
REF_VARIANT = os.environ.get("CSEM_REF_VARIANT", "")
REF_LIB = os.path.join(HERE, "_ref_fma" if REF_VARIANT == "fma" else "_ref", "libcsemref.so")
# the reference checkout: CSEM_REFERENCE_DIR, else a sibling directory "reference" of this
# repository
REF_SRC = os.environ.get("CSEM_REFERENCE_DIR") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_fp = C.POINTER(C.c_float)


def build_oracle(force: bool = False) -> str:
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    srcs = [os.path.join(HERE, "csem_oracle.c"), os.path.join(HERE, "fft2d.c")]
    if not force and os.path.exists(ORACLE_LIB):
        t = os.path.getmtime(ORACLE_LIB)
        if all(os.path.getmtime(s) < t for s in srcs + [os.path.join(HERE, "csem_oracle.h")]):
            return ORACLE_LIB
    cmd = ["gcc", "-O3", "-fPIC", "-ffp-contract=off", "-std=gnu99", "-shared", "-o",
           ORACLE_LIB] + srcs + ["-lm"]
    subprocess.run(cmd, check=True)
    return ORACLE_LIB


def ref_available() -> bool:
    return os.path.exists(os.path.join(REF_SRC, "fdfd.c"))


def build_ref(force: bool = False) -> str | None:
    """Build the reference from its sources when they are present (never on a
    machine without them)."""
    if not ref_available():
        return REF_LIB if os.path.exists(REF_LIB) else None
    if force or not os.path.exists(REF_LIB):
        subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], check=True,
                       env=dict(os.environ, REF=REF_SRC, REF_VARIANT=REF_VARIANT), stdout=subprocess.DEVNULL)
    return REF_LIB


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


def cvec(x) -> np.ndarray:
    """complex128 vector -> contiguous complex128 (interleaved doubles in memory)."""
    return np.ascontiguousarray(x, dtype=np.complex128)


@dataclass
class GridArrays:
    """Everything the hot path reads about one padded model."""
    n1: int
    n2: int
    n3f: int
    nb: int
    nz: int
    airbc: int
    fvm: int
    x1: np.ndarray
    x2: np.ndarray
    x3: np.ndarray
    x1s: np.ndarray
    x2s: np.ndarray
    x3s: np.ndarray
    d1: np.ndarray
    d2: np.ndarray
    d3: np.ndarray
    d1s: np.ndarray
    d2s: np.ndarray
    d3s: np.ndarray
    sigma11: np.ndarray
    sigma22: np.ndarray
    sigma33: np.ndarray
    rho_water: float
    n1fft: int = 0
    n2fft: int = 0
    d1fft: float = 0.0
    d2fft: float = 0.0
    sH1: np.ndarray | None = None
    sH2: np.ndarray | None = None
    jx: np.ndarray | None = None
    jy: np.ndarray | None = None
    wx: np.ndarray | None = None
    wy: np.ndarray | None = None

    @property
    def n3(self) -> int:
        """operator grid depth"""
        return self.nz + self.nb if self.airbc else self.n3f

    def lengths(self):
        n1, n2, n3 = self.n1, self.n2, self.n3
        lEx = n1 * (n2 + 1) * (n3 + 1)
        lEy = (n1 + 1) * n2 * (n3 + 1)
        lEz = (n1 + 1) * (n2 + 1) * n3
        return lEx, lEy, lEz


class _Desc(C.Structure):
    _fields_ = [("n1", C.c_int), ("n2", C.c_int), ("n3f", C.c_int), ("nb", C.c_int),
                ("nz", C.c_int), ("airbc", C.c_int), ("fvm", C.c_int)] + \
               [(nm, _dp) for nm in ("x1", "x2", "x3", "x1s", "x2s", "x3s", "d1", "d2", "d3",
                                     "d1s", "d2s", "d3s", "sigma11", "sigma22", "sigma33")] + \
               [("rho_water", C.c_double), ("n1fft", C.c_int), ("n2fft", C.c_int),
                ("d1fft", C.c_double), ("d2fft", C.c_double), ("sH1", _dp), ("sH2", _dp),
                ("jx", _ip), ("jy", _ip), ("wx", _dp), ("wy", _dp)]


def setup_grid(d: str, params: dict) -> GridArrays:
    """The padded model of a case directory (fx1..3, frho11..33) for the oracle, through
    the host set-up library alone (libcsem_host.so: csem_grid_read / extend / airbc, the
    restatement of extend_model.c, create_nugrid.c, find_index.c and airbc_init_free.c:24-109
    that tests/test_oracle_golden.py pins bit for bit to the reference; no CUDA is loaded)."""
    import sys
    root = os.path.dirname(HERE)
    if root not in sys.path:
        sys.path.insert(0, root)
    from demo_matrixfree_csem_gb300 import build as pbuild
    from demo_matrixfree_csem_gb300.api import _Grid
    if not os.path.exists(pbuild.HOST_LIB):
        pbuild.build()
    L = C.CDLL(pbuild.HOST_LIB)
    L.csem_last_error.restype = C.c_char_p
    g = _Grid()
    names = [os.path.join(d, n).encode() for n in ("fx1", "fx2", "fx3", "frho11", "frho22", "frho33")]
    if L.csem_grid_read(C.byref(g), *names):
        raise RuntimeError(L.csem_last_error().decode())
    if L.csem_grid_extend(C.byref(g), int(params.get("nb", 15)), C.c_float(float(params.get("lextend", -1))),
                          C.c_float(float(params.get("rho_air", 1e6))), int(params.get("istretch", 1))):
        raise RuntimeError(L.csem_last_error().decode())
    airbc = int(params.get("airbc", 0))
    if airbc and L.csem_grid_airbc(C.byref(g), int(params.get("n1fft", 1024)), int(params.get("n2fft", 1024))):
        raise RuntimeError(L.csem_last_error().decode())
    n1, n2, n3 = g.n1, g.n2, g.n3

    def a(name, n, dtype=np.float64):
        return np.ctypeslib.as_array(getattr(g, name), (n,)).astype(dtype, copy=True)

    kw = {}
    if airbc:
        N = g.n1fft * g.n2fft
        kw = dict(n1fft=g.n1fft, n2fft=g.n2fft, d1fft=g.d1fft, d2fft=g.d2fft,
                  sH1=a("sH1", 2 * N).view(np.complex128), sH2=a("sH2", 2 * N).view(np.complex128),
                  jx=a("jx", g.n1fft, np.int32), jy=a("jy", g.n2fft, np.int32), wx=a("wx", g.n1fft),
                  wy=a("wy", g.n2fft))
    out = GridArrays(n1, n2, n3, g.nb, g.nz, airbc, int(params.get("fvm", 0)),
                     *[a(nm, ln) for nm, ln in (("x1", n1 + 1), ("x2", n2 + 1), ("x3", n3 + 1), ("x1s", n1 + 1),
                                                ("x2s", n2 + 1), ("x3s", n3 + 1), ("d1", n1 + 1), ("d2", n2 + 1),
                                                ("d3", n3 + 1), ("d1s", n1 + 1), ("d2s", n2 + 1), ("d3s", n3 + 1))],
                     a("sigma11", n1 * (n2 + 1) * (n3 + 1)), a("sigma22", (n1 + 1) * n2 * (n3 + 1)),
                     a("sigma33", (n1 + 1) * (n2 + 1) * n3), rho_water=float(g.rho_water), **kw)
    L.csem_grid_free(C.byref(g))
    return out


class Oracle:
    """The C restatement of the reference's hot path (oracle/csem_oracle.c)."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            build_oracle()
            L = C.CDLL(ORACLE_LIB)
            L.orc_create.restype = C.c_void_p
            L.orc_create.argtypes = [C.POINTER(_Desc)]
            L.orc_destroy.argtypes = [C.c_void_p]
            L.orc_set_iom.argtypes = [C.c_void_p, C.c_double, C.c_double]
            L.orc_set_freq.argtypes = [C.c_void_p, C.c_float]
            L.orc_sizes.argtypes = [C.c_void_p, C.POINTER(C.c_long)]
            L.orc_set_hy_length.argtypes = [C.c_void_p, C.c_int]
            for nm in ("orc_fdfd_apply", "orc_fdfd_apply_old", "orc_lusgs_apply", "orc_aphi_apply",
                       "orc_get_h"):
                getattr(L, nm).argtypes = [C.c_void_p, _dp, _dp] if nm != "orc_get_h" else [C.c_void_p, _dp]
            L.orc_gmres_pre_apply.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
            L.orc_airbc_apply.argtypes = [C.c_void_p, _dp, _dp, _dp]
            L.orc_cdot.argtypes = [C.c_long, _dp, _dp, _dp]
            L.orc_bicgstab.argtypes = [C.c_void_p, _dp, _dp, C.c_int, C.c_double, _dp, C.c_int, _ip]
            L.orc_fbicgstab.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, C.c_int, C.c_double,
                                        _dp, C.c_int, _ip]
            L.orc_gmres.argtypes = [C.c_void_p, _dp, _dp, C.c_int, C.c_double, C.c_int, _dp, C.c_int, _ip]
            L.orc_fgmres.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, C.c_int, C.c_double,
                                     C.c_int, _dp, C.c_int, _ip]
            L.orc_inject.argtypes = [C.c_void_p, C.c_int, _ip, _fp, _dp]
            L.orc_extract.argtypes = [C.c_void_p, C.c_int, _ip, C.c_int, _fp, _dp, _dp]
            for nm in ("orc_bicgstab", "orc_fbicgstab", "orc_gmres", "orc_fgmres"):
                getattr(L, nm).restype = C.c_int
            cls._lib = L
        return cls._lib

    def __init__(self, g: GridArrays):
        self.g = g
        L = self.lib()
        keep = {}

        def arr(name, dtype=np.float64):
            a = getattr(g, name)
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=dtype)
            keep[name] = a
            return a

        d = _Desc()
        d.n1, d.n2, d.n3f, d.nb, d.nz, d.airbc, d.fvm = g.n1, g.n2, g.n3f, g.nb, g.nz, g.airbc, g.fvm
        for nm in ("x1", "x2", "x3", "x1s", "x2s", "x3s", "d1", "d2", "d3", "d1s", "d2s", "d3s",
                   "sigma11", "sigma22", "sigma33"):
            setattr(d, nm, _p(arr(nm)))
        d.rho_water = float(g.rho_water)
        if g.airbc:
            d.n1fft, d.n2fft, d.d1fft, d.d2fft = g.n1fft, g.n2fft, g.d1fft, g.d2fft
            d.sH1 = _p(arr("sH1", np.complex128).view(np.float64))
            d.sH2 = _p(arr("sH2", np.complex128).view(np.float64))
            d.jx = _p(arr("jx", np.int32), _ip)
            d.jy = _p(arr("jy", np.int32), _ip)
            d.wx = _p(arr("wx"))
            d.wy = _p(arr("wy"))
        self._keep = keep
        self._desc = d
        self.ctx = L.orc_create(C.byref(d))
        s = (C.c_long * 7)()
        L.orc_sizes(self.ctx, s)
        self.lE, self.lEx, self.lEy, self.lEz, self.lH, self.lv, self.n3 = list(s)

    def __del__(self):
        if getattr(self, "ctx", None) and self._lib is not None:
            self._lib.orc_destroy(self.ctx)
            self.ctx = None

    def set_freq(self, f: float):
        self.lib().orc_set_freq(self.ctx, C.c_float(f))

    def set_iom(self, z: complex):
        self.lib().orc_set_iom(self.ctx, z.real, z.imag)

    def _op(self, fn, x):
        x = cvec(x)
        y = np.zeros(self.lE, np.complex128)
        fn(self.ctx, _p(x.view(np.float64)), _p(y.view(np.float64)))
        return y

    def set_hy_length(self, sic: bool):
        """sic=True (default): the reference's Hy length n1*(n2+1)*n2 (fdfd.c:59), which
        overlaps Hz when n2 < n3; False: n1*(n2+1)*n3."""
        L = self.lib()
        L.orc_set_hy_length(self.ctx, int(bool(sic)))
        s = (C.c_long * 7)()
        L.orc_sizes(self.ctx, s)
        self.lH = s[4]

    def fdfd(self, x):
        return self._op(self.lib().orc_fdfd_apply, x)

    def fdfd_old(self, x):
        return self._op(self.lib().orc_fdfd_apply_old, x)

    def lusgs(self, x):
        return self._op(self.lib().orc_lusgs_apply, x)

    def aphi(self, x):
        return self._op(self.lib().orc_aphi_apply, x)

    def gmres_pre(self, x, mp=30):
        x = cvec(x)
        y = np.zeros(self.lE, np.complex128)
        self.lib().orc_gmres_pre_apply(self.ctx, mp, _p(x.view(np.float64)), _p(y.view(np.float64)))
        return y

    def h(self):
        h = np.zeros(self.lH, np.complex128)
        self.lib().orc_get_h(self.ctx, _p(h.view(np.float64)))
        return h

    def airbc(self, hz0):
        g = self.g
        hz0 = cvec(hz0)
        hx = np.zeros((g.n1 + 1) * g.n2, np.complex128)
        hy = np.zeros(g.n1 * (g.n2 + 1), np.complex128)
        self.lib().orc_airbc_apply(self.ctx, _p(hz0.view(np.float64)), _p(hx.view(np.float64)),
                                   _p(hy.view(np.float64)))
        return hx, hy

    @classmethod
    def cdot(cls, a, b) -> complex:
        a, b = cvec(a), cvec(b)
        o = np.zeros(2)
        cls.lib().orc_cdot(len(a), _p(a.view(np.float64)), _p(b.view(np.float64)), _p(o))
        return complex(o[0], o[1])

    def solve(self, b, algopt=1, precond=1, niter=1000, tol=1e-8, nrestart=10, mp=30, x0=None):
        """Dispatch as the reference driver does (main.c:104-118). Returns
        (x, history, iterations)."""
        L = self.lib()
        b = cvec(b)
        x = np.zeros(self.lE, np.complex128) if x0 is None else cvec(x0).copy()
        cap = 4 * niter * max(nrestart, 1) + 16
        hist = np.zeros(cap)
        nh = C.c_int(0)
        xp, bp = _p(x.view(np.float64)), _p(b.view(np.float64))
        if precond == 0 and algopt == 1:
            it = L.orc_bicgstab(self.ctx, xp, bp, niter, tol, _p(hist), cap, C.byref(nh))
        elif precond == 0 and algopt == 2:
            it = L.orc_gmres(self.ctx, xp, bp, niter // nrestart, tol, nrestart, _p(hist), cap, C.byref(nh))
        elif algopt == 1:
            it = L.orc_fbicgstab(self.ctx, precond, mp, xp, bp, niter, tol, _p(hist), cap, C.byref(nh))
        else:
            it = L.orc_fgmres(self.ctx, precond, mp, xp, bp, niter // nrestart, tol, nrestart,
                              _p(hist), cap, C.byref(nh))
        return x, hist[:min(nh.value, cap)].copy(), it

    def inject(self, chsrc, src_xyz):
        ch = np.asarray(chsrc, np.int32)
        s = np.asarray(src_xyz, np.float32)[:3].copy()
        b = np.zeros(self.lE, np.complex128)
        self.lib().orc_inject(self.ctx, len(ch), _p(ch, _ip), _p(s, _fp), _p(b.view(np.float64)))
        return b

    def extract(self, chrec, rec, x):
        ch = np.asarray(chrec, np.int32)
        r = np.ascontiguousarray(rec, np.float32)
        x = cvec(x)
        out = np.zeros((len(ch), len(r)), np.complex128)
        self.lib().orc_extract(self.ctx, len(ch), _p(ch, _ip), len(r), _p(r, _fp),
                               _p(x.view(np.float64)), _p(out.view(np.float64)))
        return out


class Ref:
    """The unmodified reference, built from its sources with link stubs
    (oracle/build_ref.sh); one model per process (the reference keeps globals)."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            path = build_ref()
            if path is None or not os.path.exists(path):
                raise RuntimeError("reference build unavailable")
            L = C.CDLL(path)
            L.ref_setup.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
            L.ref_info.argtypes = [_ip]
            L.ref_finfo.argtypes = [_dp]
            L.ref_freqs.argtypes = [_fp]
            L.ref_grid.argtypes = [C.c_int, _dp]
            L.ref_sigma.argtypes = [C.c_int, _dp]
            L.ref_airfilter.argtypes = [C.c_int, _dp]
            L.ref_set_freq.argtypes = [C.c_int]
            L.ref_set_iwmu.argtypes = [C.c_double, C.c_double]
            L.ref_apply.argtypes = [C.c_int, _dp, _dp]
            L.ref_get_h.argtypes = [_dp]
            L.ref_airbc.argtypes = [_dp, _dp, _dp]
            L.ref_inject.argtypes = [_dp]
            L.ref_extract.argtypes = [_dp, C.c_int]
            L.ref_dcal.argtypes = [_fp]
            L.ref_cdot.argtypes = [C.c_int, _dp, _dp, _dp]
            L.ref_acsr_init.argtypes = [C.c_int]
            L.ref_gmres_init.argtypes = [C.c_int]
            L.ref_solve.argtypes = [C.c_int, _dp, _dp, C.c_int, C.c_int]
            L.ref_solve.restype = C.c_double
            L.ref_run_main.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
            cls._lib = L
        return cls._lib

    def __init__(self, args: list[str]):
        L = self.lib()
        argv = (C.c_char_p * (len(args) + 1))(*[a.encode() for a in args], None)
        L.ref_setup(len(args), argv)
        info = (C.c_int * 26)()
        L.ref_info(info)
        (self.n1, self.n2, self.n3, self.nb, self.nx, self.ny, self.nz, self.lE, self.lEx, self.lEy,
         self.lEz, self.lH, self.lv, self.nrec, self.nfreq, self.nchrec, self.airbc, self.fvm,
         self.preco, self.algopt, self.niter, self.nrestart, self.mp, self.n1fft, self.n2fft,
         self.nchsrc) = list(info)
        fi = (C.c_double * 9)()
        L.ref_finfo(fi)
        self.rho_water, self.rho_air, self.lextend, self.tol, self.d1fft, self.d2fft, self.d3fft = list(fi)[:7]
        fr = np.zeros(self.nfreq, np.float32)
        L.ref_freqs(_p(fr, _fp))
        self.freqs = fr

    def grid_arrays(self) -> GridArrays:
        L = self.lib()
        n1f, n2f, n3f = self.nx + 2 * self.nb, self.ny + 2 * self.nb, self.nz + 2 * self.nb
        lens = [n1f + 1, n2f + 1, n3f + 1] * 4
        g = []
        for w in range(12):
            a = np.zeros(lens[w])
            L.ref_grid(w, _p(a))
            g.append(a)
        sl = [n1f * (n2f + 1) * (n3f + 1), (n1f + 1) * n2f * (n3f + 1), (n1f + 1) * (n2f + 1) * n3f]
        sig = []
        for w in range(3):
            a = np.zeros(sl[w])
            L.ref_sigma(w, _p(a))
            sig.append(a)
        kw = {}
        if self.airbc:
            N = self.n1fft * self.n2fft
            sH = []
            for w in range(2):
                a = np.zeros(N, np.complex128)
                L.ref_airfilter(w, _p(a.view(np.float64)))
                sH.append(a)
            jx = np.ctypeslib.as_array(C.cast(C.c_void_p.in_dll(L, "jx").value, _ip), (self.n1fft,)).copy()
            jy = np.ctypeslib.as_array(C.cast(C.c_void_p.in_dll(L, "jy").value, _ip), (self.n2fft,)).copy()
            wx = np.ctypeslib.as_array(C.cast(C.c_void_p.in_dll(L, "wx").value, _dp), (self.n1fft,)).copy()
            wy = np.ctypeslib.as_array(C.cast(C.c_void_p.in_dll(L, "wy").value, _dp), (self.n2fft,)).copy()
            kw = dict(n1fft=self.n1fft, n2fft=self.n2fft, d1fft=self.d1fft, d2fft=self.d2fft,
                      sH1=sH[0], sH2=sH[1], jx=jx, jy=jy, wx=wx, wy=wy)
        return GridArrays(n1f, n2f, n3f, self.nb, self.nz, self.airbc, self.fvm, *g, *sig,
                          rho_water=self.rho_water, **kw)

    def set_freq(self, ifreq: int):
        self.lib().ref_set_freq(ifreq)

    def set_iom(self, z: complex):
        self.lib().ref_set_iwmu(z.real, z.imag)

    def apply(self, op: int, x):
        """op: 0 fdfd_apply, 1 lusgs_apply, 2 aphi_apply, 3 fdfd_apply_old,
        4 gmres_apply (after gmres_init), 5 Acsr_apply, 6 Acsr_lusgs_apply"""
        x = cvec(x).copy()
        y = np.zeros(self.lE, np.complex128)
        self.lib().ref_apply(op, _p(x.view(np.float64)), _p(y.view(np.float64)))
        return y

    def h(self):
        h = np.zeros(self.lH, np.complex128)
        self.lib().ref_get_h(_p(h.view(np.float64)))
        return h

    def airbc(self, hz0):
        hz0 = cvec(hz0).copy()
        hx = np.zeros((self.n1 + 1) * self.n2, np.complex128)
        hy = np.zeros(self.n1 * (self.n2 + 1), np.complex128)
        self.lib().ref_airbc(_p(hz0.view(np.float64)), _p(hx.view(np.float64)), _p(hy.view(np.float64)))
        return hx, hy

    def inject(self):
        b = np.zeros(self.lE, np.complex128)
        self.lib().ref_inject(_p(b.view(np.float64)))
        return b

    def extract(self, x, ifreq=0):
        x = cvec(x).copy()
        self.lib().ref_extract(_p(x.view(np.float64)), ifreq)
        d = np.zeros((self.nchrec, self.nfreq, self.nrec), np.complex64)
        self.lib().ref_dcal(_p(d.view(np.float32), _fp))
        return d

    def cdot(self, a, b) -> complex:
        a, b = cvec(a), cvec(b)
        o = np.zeros(2)
        self.lib().ref_cdot(len(a), _p(a.view(np.float64)), _p(b.view(np.float64)), _p(o))
        return complex(o[0], o[1])

    def gmres_init(self, m):
        self.lib().ref_gmres_init(m)

    def solve(self, ifreq: int, niter: int = -1, verb: int = 0):
        x = np.zeros(self.lE, np.complex128)
        b = np.zeros(self.lE, np.complex128)
        t = self.lib().ref_solve(ifreq, _p(x.view(np.float64)), _p(b.view(np.float64)), niter, verb)
        return x, b, t
