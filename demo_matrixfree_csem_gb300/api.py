"""ctypes bindings of libcsem_gpu.so (include/csem_host.h, include/csem_gpu.h).

This is the Python mirror of the reference's interface for the solve: a Grid is the
padded model of emf_t (emf.h) after emf_init/extend_model_init/airbc_init, a Ctx owns it
on the GPU and exposes fdfd_apply / lusgs_apply / aphi_apply / gmres_apply /
airbc_apply / inject_source / extract_emf / cdotprod and the solver dispatch of the
reference driver (main.c:104-118). There is no CPU fallback: every compute entry point
runs on the GPU and raises when the library or the GPU is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_long)

CSEM_OK = 0
ERRORS = {-1: "EINVAL", -2: "EIO", -3: "ENOMEM", -4: "EDOMAIN", -5: "ECUDA", -6: "ENODEV", -7: "ETOOBIG"}
STATUS = {0: "running", 1: "converged", 2: "maxiter", 3: "breakdown", 4: "nonfinite", 5: "zero_rhs"}
CHANNELS = {"Ex": 0, "Ey": 1, "Ez": 2, "Hx": 3, "Hy": 4, "Hz": 5}


class CsemError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"csem error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


class _Grid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("x1node", _fp), ("x2node", _fp), ("x3node", _fp),
                ("rho11", _fp), ("rho22", _fp), ("rho33", _fp),
                ("rhomin", C.c_float), ("rhomax", C.c_float), ("rho_water", C.c_float),
                ("rho_air", C.c_float), ("lextend", C.c_float),
                ("nb", C.c_int), ("istretch", C.c_int), ("airbc", C.c_int), ("fvm", C.c_int),
                ("n1", C.c_int), ("n2", C.c_int), ("n3", C.c_int)] + \
               [(nm, _dp) for nm in ("x1", "x2", "x3", "x1s", "x2s", "x3s", "d1", "d2", "d3",
                                     "d1s", "d2s", "d3s", "sigma11", "sigma22", "sigma33")] + \
               [("rstretch", C.c_double * 6), ("d1min", C.c_double), ("d2min", C.c_double),
                ("d3min", C.c_double), ("n1fft", C.c_int), ("n2fft", C.c_int),
                ("d1fft", C.c_double), ("d2fft", C.c_double), ("d3fft", C.c_double),
                ("sH1", _dp), ("sH2", _dp), ("jx", _ip), ("jy", _ip), ("wx", _dp), ("wy", _dp)]


_LIB = None


def lib(build_if_missing: bool = True):
    """Load libcsem_gpu.so from the in-tree build (building it first if asked)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"libcsem_gpu.so not built ({path}); run demo_matrixfree_csem_gb300.build")
        _build.build()
    L = C.CDLL(path)
    sig = {
        "csem_last_error": (C.c_char_p, []),
        "csem_version": (C.c_char_p, []),
        "csem_device_count": (C.c_int, []),
        "csem_initargs": (None, [C.c_int, C.POINTER(C.c_char_p)]),
        "csem_countparval": (C.c_int, [C.c_char_p]),
        "csem_getparint": (C.c_int, [C.c_char_p, _ip]),
        "csem_getparfloat": (C.c_int, [C.c_char_p, _fp]),
        "csem_getpardouble": (C.c_int, [C.c_char_p, _dp]),
        "csem_getparstring": (C.c_int, [C.c_char_p, C.POINTER(C.c_char_p)]),
        "csem_grid_read": (C.c_int, [C.POINTER(_Grid)] + [C.c_char_p] * 6),
        "csem_grid_set": (C.c_int, [C.POINTER(_Grid), C.c_int, C.c_int, C.c_int] + [_fp] * 6),
        "csem_grid_extend": (C.c_int, [C.POINTER(_Grid), C.c_int, C.c_float, C.c_float, C.c_int]),
        "csem_grid_airbc": (C.c_int, [C.POINTER(_Grid), C.c_int, C.c_int]),
        "csem_grid_free": (None, [C.POINTER(_Grid)]),
        "csem_grid_write_extended": (C.c_int, [C.POINTER(_Grid), C.c_char_p]),
        "csem_write_emf": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, _fp]),
        "csem_sort_freqs": (None, [_fp, C.c_int]),
        "csem_ctx_create": (C.c_int, [C.POINTER(_Grid), C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
        "csem_ctx_destroy": (None, [C.c_void_p]),
        "csem_ctx_sizes": (C.c_int, [C.c_void_p, _lp]),
        "csem_ctx_sync": (C.c_int, [C.c_void_p]),
        "csem_ctx_stream": (C.c_void_p, [C.c_void_p]),
        "csem_ctx_set_option": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int]),
        "csem_batch_bytes": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, _dp]),
        "csem_solve_batches_host": (C.c_int, [C.c_int, C.c_void_p]),
        "csem_partition_systems": (C.c_int, [C.c_int, _fp, _dp, C.c_double, C.c_int, _ip, _dp]),
        "csem_solve_batch_multi": (C.c_int, [C.c_int, _ip, C.c_void_p, C.c_int, C.c_int, C.c_int, _fp, _fp, C.c_int,
                                             _ip, C.c_int, _ip, C.c_int, _fp, C.c_void_p, _dp, _ip, _ip, _ip, _dp,
                                             _ip]),
        "csem_batch_capacity": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double, _ip]),
        "csem_fdfd_apply_host": (C.c_int, [C.c_void_p, C.c_double, C.c_double, _dp, _dp]),
        "csem_lusgs_apply_host": (C.c_int, [C.c_void_p, C.c_double, C.c_double, _dp, _dp]),
        "csem_aphi_apply_host": (C.c_int, [C.c_void_p, C.c_double, C.c_double, _dp, _dp]),
        "csem_gmres_pre_apply_host": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int, _dp, _dp]),
        "csem_airbc_apply_host": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
        "csem_fdfd_apply_c64_host": (C.c_int, [C.c_void_p, C.c_double, C.c_double, _fp, _fp]),
        "csem_lusgs_apply_c64_host": (C.c_int, [C.c_void_p, C.c_double, C.c_double, _fp, _fp]),
        "csem_aphi_apply_c64_host": (C.c_int, [C.c_void_p, C.c_double, C.c_double, _fp, _fp]),
        "csem_cdot_host": (C.c_int, [C.c_long, _dp, _dp, _dp]),
        "csem_cdot_c64_host": (C.c_int, [C.c_long, _fp, _fp, _dp]),
        "csem_inject_host": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int, _ip, _fp, _dp]),
        "csem_extract_host": (C.c_int, [C.c_void_p, C.c_int, _ip, C.c_int, _fp, _dp, _dp]),
        "csem_solve_fp64_host": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int,
                                           C.c_double, C.c_double, _dp, _dp, _dp, C.c_int, _ip, _ip, _ip]),
        "csem_fdfd_apply_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, C.c_void_p, C.c_void_p, C.c_void_p]),
        "csem_lusgs_apply_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, C.c_void_p, C.c_void_p, C.c_void_p]),
        "csem_aphi_apply_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, C.c_void_p, C.c_void_p, C.c_void_p]),
        "csem_cdot_dev": (C.c_int, [C.c_int, C.c_long, C.c_int, C.c_void_p, C.c_void_p, _dp, C.c_void_p]),
        "csem_solve_batch_host": (C.c_int, [C.c_void_p, C.c_int, _fp, _fp, C.c_int, _ip, C.c_int, _ip, C.c_int, _fp,
                                            C.c_void_p, _dp, _ip, _ip, _ip, _dp]),
        "csem_csr_compare": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int, _dp]),
        "csem_history_logged": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int]),
        "csem_profile": (C.c_int, [C.c_int]),
        "csem_profile_read": (C.c_int, [C.c_int, _dp, _lp, _lp]),
        "csem_launch_count": (C.c_longlong, []),
        "csem_sweep_groups": (C.c_int, [C.c_int, _dp, C.c_int, C.c_int, _ip, _ip, _ip, _ip]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _LIB = L
    return L


def _check(rc: int) -> None:
    if rc != CSEM_OK:
        raise CsemError(rc, lib().csem_last_error().decode())


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


def _c128(x) -> np.ndarray:
    return np.ascontiguousarray(x, dtype=np.complex128)


def _c64(x) -> np.ndarray:
    return np.ascontiguousarray(x, dtype=np.complex64)


def iom_of(freq: float) -> complex:
    """I*omega*mu0 exactly as the reference driver forms it (main.c:95): the product
    I*2*PI*f*mu0 evaluated left to right in double on (0,1), f a float."""
    pi = 3.14159265358979323846264
    mu0 = 4.0 * pi * 1e-7
    im = ((2.0 * pi) * float(np.float32(freq))) * mu0
    return complex(0.0, im)


def device_count() -> int:
    return lib().csem_device_count()


class Grid:
    """A padded model: emf_init + extend_model_init (+ airbc_init) on the host."""

    def __init__(self):
        self.g = _Grid()
        self._owned = False

    @classmethod
    def from_files(cls, fx1, fx2, fx3, frho11, frho22, frho33) -> "Grid":
        self = cls()
        _check(lib().csem_grid_read(C.byref(self.g), *[s.encode() for s in (fx1, fx2, fx3, frho11, frho22, frho33)]))
        self._owned = True
        return self

    @classmethod
    def from_arrays(cls, x1, x2, x3, rho11, rho22, rho33) -> "Grid":
        self = cls()
        a = [np.ascontiguousarray(v, np.float32) for v in (x1, x2, x3, rho11, rho22, rho33)]
        nx, ny, nz = len(a[0]) - 1, len(a[1]) - 1, len(a[2]) - 1
        _check(lib().csem_grid_set(C.byref(self.g), nx, ny, nz, *[_p(v, _fp) for v in a]))
        self._owned = True
        return self

    def extend(self, nb: int, lextend: float = -1.0, rho_air: float = 1e6, istretch: int = 1) -> "Grid":
        _check(lib().csem_grid_extend(C.byref(self.g), nb, lextend, rho_air, istretch))
        return self

    def airbc(self, n1fft: int = 1024, n2fft: int = 1024) -> "Grid":
        _check(lib().csem_grid_airbc(C.byref(self.g), n1fft, n2fft))
        return self

    def __del__(self):
        if getattr(self, "_owned", False) and _LIB is not None:
            _LIB.csem_grid_free(C.byref(self.g))
            self._owned = False

    # ---- views
    def _arr(self, name, n, dtype=np.float64):
        ptr = getattr(self.g, name)
        if not ptr:
            return None
        return np.ctypeslib.as_array(ptr, (n,)).astype(dtype, copy=True)

    @property
    def shape_full(self):
        return self.g.n1, self.g.n2, self.g.n3

    def arrays(self) -> dict:
        g = self.g
        n1, n2, n3 = g.n1, g.n2, g.n3
        out = {}
        for nm, n in (("x1", n1 + 1), ("x2", n2 + 1), ("x3", n3 + 1), ("x1s", n1 + 1), ("x2s", n2 + 1),
                      ("x3s", n3 + 1), ("d1", n1 + 1), ("d2", n2 + 1), ("d3", n3 + 1), ("d1s", n1 + 1),
                      ("d2s", n2 + 1), ("d3s", n3 + 1)):
            out[nm] = self._arr(nm, n)
        out["sigma11"] = self._arr("sigma11", n1 * (n2 + 1) * (n3 + 1))
        out["sigma22"] = self._arr("sigma22", (n1 + 1) * n2 * (n3 + 1))
        out["sigma33"] = self._arr("sigma33", (n1 + 1) * (n2 + 1) * n3)
        if g.sH1:
            N = g.n1fft * g.n2fft
            out["sH1"] = self._arr("sH1", 2 * N).view(np.complex128)
            out["sH2"] = self._arr("sH2", 2 * N).view(np.complex128)
            out["jx"] = self._arr("jx", g.n1fft, np.int32)
            out["jy"] = self._arr("jy", g.n2fft, np.int32)
            out["wx"] = self._arr("wx", g.n1fft)
            out["wy"] = self._arr("wy", g.n2fft)
        return out

    def write_extended(self, d: str) -> None:
        _check(lib().csem_grid_write_extended(C.byref(self.g), d.encode()))


class Ctx:
    """One padded model resident on the GPU (csem_ctx)."""

    def __init__(self, grid: Grid, airbc: int = 0, fvm: int = 0):
        self.grid = grid
        h = C.c_void_p()
        _check(lib().csem_ctx_create(C.byref(grid.g), airbc, fvm, C.byref(h)))
        self.h = h
        s = (C.c_long * 10)()
        _check(lib().csem_ctx_sizes(self.h, s))
        (self.lE, self.lEx, self.lEy, self.lEz, self.lv, self.n1, self.n2, self.n3, self.n3f, self.nb) = list(s)
        self.airbc, self.fvm = airbc, fvm

    def batch_bytes(self, nsys: int, precision: int = 32, preco: int = 1) -> float:
        """Device bytes a batched solve of nsys systems needs beyond the model."""
        b = C.c_double(0)
        _check(lib().csem_batch_bytes(self.h, precision, preco, nsys, C.byref(b)))
        return b.value

    def batch_capacity(self, budget_bytes: float, precision: int = 32, preco: int = 1) -> int:
        """Largest number of systems one batched solve can hold within budget_bytes."""
        n = C.c_int(0)
        _check(lib().csem_batch_capacity(self.h, precision, preco, float(budget_bytes), C.byref(n)))
        return n.value

    def set_option(self, name: str, value: int) -> None:
        """Kernel-schedule options, e.g. set_option("lusgs_pipelined", 0)."""
        _check(lib().csem_ctx_set_option(self.h, name.encode(), int(value)))

    @property
    def stream(self) -> int:
        """The context's cudaStream_t as an integer handle."""
        return int(lib().csem_ctx_stream(self.h) or 0)

    def close(self):
        if getattr(self, "h", None) and _LIB is not None:
            _LIB.csem_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _op(self, fn, iom, x, c64=False):
        if c64:
            x = _c64(x)
            y = np.zeros(self.lE, np.complex64)
            _check(fn(self.h, iom.real, iom.imag, _p(x.view(np.float32), _fp), _p(y.view(np.float32), _fp)))
        else:
            x = _c128(x)
            y = np.zeros(self.lE, np.complex128)
            _check(fn(self.h, iom.real, iom.imag, _p(x.view(np.float64)), _p(y.view(np.float64))))
        return y

    def fdfd_apply(self, iom: complex, x, c64=False):
        L = lib()
        return self._op(L.csem_fdfd_apply_c64_host if c64 else L.csem_fdfd_apply_host, iom, x, c64)

    def lusgs_apply(self, iom: complex, x, c64=False):
        L = lib()
        return self._op(L.csem_lusgs_apply_c64_host if c64 else L.csem_lusgs_apply_host, iom, x, c64)

    def aphi_apply(self, iom: complex, x, c64=False):
        L = lib()
        return self._op(L.csem_aphi_apply_c64_host if c64 else L.csem_aphi_apply_host, iom, x, c64)

    def gmres_apply(self, iom: complex, x, mp: int = 30):
        x = _c128(x)
        y = np.zeros(self.lE, np.complex128)
        _check(lib().csem_gmres_pre_apply_host(self.h, iom.real, iom.imag, mp, _p(x.view(np.float64)),
                                                _p(y.view(np.float64))))
        return y

    def airbc_apply(self, hz0):
        hz0 = _c128(hz0)
        hx = np.zeros((self.n1 + 1) * self.n2, np.complex128)
        hy = np.zeros(self.n1 * (self.n2 + 1), np.complex128)
        _check(lib().csem_airbc_apply_host(self.h, _p(hz0.view(np.float64)), _p(hx.view(np.float64)),
                                           _p(hy.view(np.float64))))
        return hx, hy

    def inject_source(self, iom: complex, chsrc, src_xyz):
        ch = np.asarray([CHANNELS[c] if isinstance(c, str) else c for c in chsrc], np.int32)
        s = np.asarray(src_xyz, np.float32)[:3].copy()
        b = np.zeros(self.lE, np.complex128)
        _check(lib().csem_inject_host(self.h, iom.real, iom.imag, len(ch), _p(ch, _ip), _p(s, _fp),
                                      _p(b.view(np.float64))))
        return b

    def extract_emf(self, chrec, rec, x):
        ch = np.asarray([CHANNELS[c] if isinstance(c, str) else c for c in chrec], np.int32)
        r = np.ascontiguousarray(rec, np.float32)
        x = _c128(x)
        out = np.zeros((len(ch), len(r)), np.complex128)
        _check(lib().csem_extract_host(self.h, len(ch), _p(ch, _ip), len(r), _p(r, _fp),
                                       _p(x.view(np.float64)), _p(out.view(np.float64))))
        return out

    def csr_compare(self, iom: complex, prec: int = 64, nrep: int = 5) -> dict:
        """The operator assembled in CSR (by probing) against the matrix-free stencil:
        ms per cuSPARSE SpMV and per stencil application, their max relative difference,
        stored entries and the bytes one SpMV moves (csem_csr_compare; airbc=0 only)."""
        out = (C.c_double * 5)()
        _check(lib().csem_csr_compare(self.h, int(prec), iom.real, iom.imag, int(nrep), out))
        return dict(ms_csr=out[0], ms_stencil=out[1], relerr=out[2], nnz=int(out[3]), csr_bytes=out[4])

    def solve_fp64(self, iom: complex, b, algopt=1, preco=1, niter=1000, tol=1e-8, nrestart=10, mp=30, x0=None):
        """Returns (x, history, iterations, status)."""
        b = _c128(b)
        x = np.zeros(self.lE, np.complex128) if x0 is None else _c128(x0).copy()
        cap = niter + 8 + (niter * 2 if algopt == 2 else 0)
        hist = np.zeros(cap)
        nh, it, st = C.c_int(0), C.c_int(0), C.c_int(0)
        _check(lib().csem_solve_fp64_host(self.h, algopt, preco, niter, tol, nrestart, mp, iom.real, iom.imag,
                                          _p(b.view(np.float64)), _p(x.view(np.float64)), _p(hist), cap,
                                          C.byref(nh), C.byref(it), C.byref(st)))
        return x, hist[:min(nh.value, cap)].copy(), it.value, STATUS.get(st.value, st.value)


class _BatchOpts(C.Structure):
    _fields_ = [("precision", C.c_int), ("algopt", C.c_int), ("preco", C.c_int), ("niter", C.c_int),
                ("tol", C.c_float), ("inner_tol", C.c_double), ("check_every", C.c_int), ("max_outer", C.c_int),
                ("nrestart", C.c_int), ("mp", C.c_int)]


def solve_batch(ctx: Ctx, freqs, srcs, chsrc=("Ex",), chrec=("Ex", "Ey", "Ez"), rec=None, precision=32, algopt=1,
                preco=1, niter=1000, tol=1e-8, inner_tol=0.2, check_every=4, max_outer=30, nrestart=10, mp=30):
    """Solve len(freqs) systems (frequency freqs[s], dipole at srcs[s]) and extract the
    receivers rec ([nrec][5] rows). Returns a dict with dcal [nsys][nchrec][nrec]
    (complex128), iters, outer, status, relres."""
    f = np.ascontiguousarray(freqs, np.float32)
    s = np.ascontiguousarray(np.asarray(srcs, np.float32)[:, :3])
    nsys = len(f)
    assert s.shape == (nsys, 3)
    cs_ = np.asarray([CHANNELS[c] if isinstance(c, str) else c for c in chsrc], np.int32)
    cr = np.asarray([CHANNELS[c] if isinstance(c, str) else c for c in chrec], np.int32)
    r = np.ascontiguousarray(rec if rec is not None else np.zeros((0, 5)), np.float32)
    o = _BatchOpts(precision, algopt, preco, niter, tol, inner_tol, check_every, max_outer, nrestart, mp)
    dcal = np.zeros((nsys, len(cr), len(r)), np.complex128)
    it = np.zeros(nsys, np.int32)
    ou = np.zeros(nsys, np.int32)
    st = np.zeros(nsys, np.int32)
    rr = np.zeros(nsys)
    _check(lib().csem_solve_batch_host(ctx.h, nsys, _p(f, _fp), _p(s, _fp), len(cs_), _p(cs_, _ip), len(cr),
                                       _p(cr, _ip), len(r), _p(r, _fp), C.byref(o), _p(dcal.view(np.float64)),
                                       _p(it, _ip), _p(ou, _ip), _p(st, _ip), _p(rr)))
    return dict(dcal=dcal, iters=it, outer=ou, status=[STATUS.get(int(v), int(v)) for v in st], relres=rr)


def partition_systems(ndev: int, freqs=None, cost=None, unknowns: float = 1.0):
    """Balanced split of systems over ndev devices (csem_partition_systems): returns
    (owner slot per system, summed work per slot). Work is cost[s] when given, else
    unknowns * freqs[s]^(-2/3)."""
    f = np.ascontiguousarray(freqs if freqs is not None else np.zeros(0), np.float32)
    c = None if cost is None else np.ascontiguousarray(cost, np.float64)
    n = len(c) if c is not None else len(f)
    owner = np.zeros(n, np.int32)
    load = np.zeros(ndev)
    _check(lib().csem_partition_systems(n, _p(f, _fp) if len(f) else None, _p(c) if c is not None else None,
                                        float(unknowns), int(ndev), _p(owner, _ip), _p(load)))
    return owner, load


def solve_batch_multi(grid: "Grid", devices, freqs, srcs, airbc=0, fvm=0, chsrc=("Ex",), chrec=("Ex", "Ey", "Ez"),
                      rec=None, precision=32, algopt=1, preco=1, niter=1000, tol=1e-8, inner_tol=0.2, check_every=4,
                      max_outer=30, nrestart=10, mp=30):
    """Solve the systems of one model on several devices (csem_solve_batch_multi): one
    context and host thread per entry of `devices`, the systems split by
    partition_systems, outputs gathered in the original order. Returns solve_batch's
    dict plus 'owner' (slot of each system)."""
    f = np.ascontiguousarray(freqs, np.float32)
    s = np.ascontiguousarray(np.asarray(srcs, np.float32)[:, :3])
    nsys = len(f)
    dv = np.ascontiguousarray(devices, np.int32)
    cs_ = np.asarray([CHANNELS[c] if isinstance(c, str) else c for c in chsrc], np.int32)
    cr = np.asarray([CHANNELS[c] if isinstance(c, str) else c for c in chrec], np.int32)
    r = np.ascontiguousarray(rec if rec is not None else np.zeros((0, 5)), np.float32)
    o = _BatchOpts(precision, algopt, preco, niter, tol, inner_tol, check_every, max_outer, nrestart, mp)
    dcal = np.zeros((nsys, len(cr), len(r)), np.complex128)
    it, ou, st, own = (np.zeros(nsys, np.int32) for _ in range(4))
    rr = np.zeros(nsys)
    _check(lib().csem_solve_batch_multi(len(dv), _p(dv, _ip), C.byref(grid.g), airbc, fvm, nsys, _p(f, _fp),
                                        _p(s, _fp), len(cs_), _p(cs_, _ip), len(cr), _p(cr, _ip), len(r), _p(r, _fp),
                                        C.byref(o), _p(dcal.view(np.float64)), _p(it, _ip), _p(ou, _ip), _p(st, _ip),
                                        _p(rr), _p(own, _ip)))
    return dict(dcal=dcal, iters=it, outer=ou, status=[STATUS.get(int(v), int(v)) for v in st], relres=rr, owner=own)


class _BatchJob(C.Structure):
    _fields_ = [("ctx", C.c_void_p), ("nsys", C.c_int), ("freq", _fp), ("src3", _fp), ("nchsrc", C.c_int),
                ("chsrc", _ip), ("nchrec", C.c_int), ("chrec", _ip), ("nrec", C.c_int), ("rec", _fp),
                ("opt", C.POINTER(_BatchOpts)), ("dcal", _dp), ("iters", _ip), ("outer", _ip), ("status", _ip),
                ("relres", _dp), ("rc", C.c_int)]


def solve_batches(jobs):
    """Solve several batches on distinct contexts at the same time (csem_solve_batches_host).
    jobs: list of dicts with the arguments of solve_batch (ctx, freqs, srcs and optional
    keywords). Returns one result dict per job, as solve_batch."""
    keep, cjobs, outs = [], [], []
    for j in jobs:
        j = dict(j)
        ctx = j.pop("ctx")
        f = np.ascontiguousarray(j.pop("freqs"), np.float32)
        sr = np.ascontiguousarray(np.asarray(j.pop("srcs"), np.float32)[:, :3])
        chsrc = j.pop("chsrc", ("Ex",))
        chrec = j.pop("chrec", ("Ex", "Ey", "Ez"))
        rec = j.pop("rec", None)
        d = dict(precision=32, algopt=1, preco=1, niter=1000, tol=1e-8, inner_tol=0.2, check_every=4, max_outer=30,
                 nrestart=10, mp=30)
        d.update(j)
        o = _BatchOpts(d["precision"], d["algopt"], d["preco"], d["niter"], d["tol"], d["inner_tol"],
                       d["check_every"], d["max_outer"], d["nrestart"], d["mp"])
        cs_ = np.asarray([CHANNELS[c] if isinstance(c, str) else c for c in chsrc], np.int32)
        cr = np.asarray([CHANNELS[c] if isinstance(c, str) else c for c in chrec], np.int32)
        r = np.ascontiguousarray(rec if rec is not None else np.zeros((0, 5)), np.float32)
        nsys = len(f)
        out = dict(dcal=np.zeros((nsys, len(cr), len(r)), np.complex128), iters=np.zeros(nsys, np.int32),
                   outer=np.zeros(nsys, np.int32), st=np.zeros(nsys, np.int32), relres=np.zeros(nsys))
        keep += [f, sr, cs_, cr, r, o]
        outs.append(out)
        cjobs.append(_BatchJob(ctx.h, nsys, _p(f, _fp), _p(sr, _fp), len(cs_), _p(cs_, _ip), len(cr), _p(cr, _ip),
                               len(r), _p(r, _fp), C.pointer(o), _p(out["dcal"].view(np.float64)),
                               _p(out["iters"], _ip), _p(out["outer"], _ip), _p(out["st"], _ip), _p(out["relres"]), 0))
    arr = (_BatchJob * len(cjobs))(*cjobs)
    _check(lib().csem_solve_batches_host(len(cjobs), arr))
    return [dict(dcal=o["dcal"], iters=o["iters"], outer=o["outer"],
                 status=[STATUS.get(int(v), int(v)) for v in o["st"]], relres=o["relres"]) for o in outs]


PROF_NAMES = ["A64", "A32", "lusgs64", "lusgs32", "aphi64", "aphi32", "air64", "air32", "stencil64", "stencil32"]


def profile(enable: bool) -> None:
    """Start (clearing earlier records) or stop per-operator device timing."""
    _check(lib().csem_profile(1 if enable else 0))


def profile_read() -> dict:
    """{category: (milliseconds, applications, systems)} from the recorded CUDA events."""
    n = len(PROF_NAMES)
    ms = np.zeros(n)
    cnt = np.zeros(n, np.int64)
    units = np.zeros(n, np.int64)
    _check(lib().csem_profile_read(n, _p(ms), cnt.ctypes.data_as(_lp), units.ctypes.data_as(_lp)))
    return {PROF_NAMES[i]: (float(ms[i]), int(cnt[i]), int(units[i])) for i in range(n)}


def launch_count() -> int:
    """Kernel launches issued by libcsem_gpu.so so far (cuFFT's own kernels excluded)."""
    return int(lib().csem_launch_count())


def cdot(a, b, c64=False) -> complex:
    o = np.zeros(2)
    if c64:
        a, b = _c64(a), _c64(b)
        _check(lib().csem_cdot_c64_host(len(a), _p(a.view(np.float32), _fp), _p(b.view(np.float32), _fp), _p(o)))
    else:
        a, b = _c128(a), _c128(b)
        _check(lib().csem_cdot_host(len(a), _p(a.view(np.float64)), _p(b.view(np.float64)), _p(o)))
    return complex(o[0], o[1])


def sweep_groups(iom, ns: int, halves: bool = False):
    """The same-frequency slot groups of the batched complex64 LU-SGS (csem_sweep_groups):
    (groups as an (ngroups, ns) array, -1 padded; nA; ngA)."""
    z = np.asarray(iom, np.complex128).ravel()
    a = np.ascontiguousarray(np.stack([z.real, z.imag], axis=1).ravel())
    out = np.zeros(len(z) * ns, np.int32)
    ng, na, nga = C.c_int(), C.c_int(), C.c_int()
    _check(lib().csem_sweep_groups(len(z), _p(a), ns, int(bool(halves)), _p(out, _ip), C.byref(ng), C.byref(na),
                                   C.byref(nga)))
    return out[:ng.value * ns].reshape(ng.value, ns), na.value, nga.value
