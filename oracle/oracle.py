"""ctypes wrapper of the CPU oracle (oracle/fair_oracle.c).

TEST INFRASTRUCTURE ONLY: the tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` load this module to check or time the GPU
library; the product never does. Parity of the oracle with the reference is
unpinned by the reference itself (it ships no tests or golden vectors and is
Fortran that cannot be compiled here); the analytic known-answer tests in
tests/test_oracle_kat.py pin it.

Every function mirrors the reference procedure of the same name, citing its
file:line in the reference project, with arrays as numpy float64/int32 and
CSR matrices as ``OracleCSR`` (IA offsets with IA[0] = 0, JA 1-based).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libfair_oracle.so")
_lib = None

ERR_TEXT = {
    1: "Vector input size incorrect.",
    2: "Unknown method.",
    3: "++ Something went wrong",
    4: "Invalid argument.",
    5: "Newton method did not converge.",
    6: "Allocation failed.",
}


class OracleError(RuntimeError):
    def __init__(self, code):
        super().__init__(f"oracle status {code}: {ERR_TEXT.get(code, 'error')}")
        self.code = code


class _CSR(C.Structure):
    _fields_ = [("m", C.c_int32), ("n", C.c_int32), ("nnz", C.c_int64),
                ("IA", C.POINTER(C.c_int64)), ("JA", C.POINTER(C.c_int32)),
                ("vA", C.POINTER(C.c_double))]


class _Opts(C.Structure):
    _fields_ = [("relaxpar", C.c_double), ("ubound", C.c_double),
                ("lbound", C.c_double), ("damp", C.c_double),
                ("verbose", C.c_int32), ("upb", C.c_int32), ("lwrb", C.c_int32),
                ("rowprobability", C.c_int32)]


def build():
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = C.CDLL(_LIB_PATH)
        _declare(_lib)
    return _lib


def _declare(L):
    P = C.POINTER
    d, i32, i64, vp = C.c_double, C.c_int, C.c_int64, C.c_void_p
    L.or_random_seed.argtypes = [C.c_uint64]
    L.or_random_number.restype = d
    L.or_random_counter.restype = C.c_uint64
    L.or_linspace.argtypes = [d, d, i32, vp]
    L.or_paralleltomo.argtypes = [i32, i32, i32, vp, P(_CSR)]
    L.or_paralleltomo_mt.argtypes = [i32, i32, i32, vp, i32, P(_CSR)]
    L.or_fanlineartomo.argtypes = [i32, i32, i32, d, d, d, vp, i32, P(_CSR)]
    L.or_fanlineartomo_mt.argtypes = [i32, i32, i32, d, d, d, vp, i32, i32, P(_CSR)]
    L.or_csr_free.argtypes = [P(_CSR)]
    L.or_add_white_noise.argtypes = [i64, vp, d, vp, vp]
    L.or_rowvecmult.argtypes = [P(_CSR), i32, vp]
    L.or_rowvecmult.restype = d
    L.or_matvecmul.argtypes = [P(_CSR), vp, vp, i32]
    L.or_transvecmul.argtypes = [P(_CSR), vp, vp]
    L.or_transvecmul_mt.argtypes = [P(_CSR), vp, vp, i32]
    L.or_transvecmul_racy.argtypes = [P(_CSR), vp, vp, i32]
    L.or_set_mmcs_mode.argtypes = [i32]
    L.or_reorder.argtypes = [P(_CSR), P(_CSR)]
    L.or_row_norms.argtypes = [P(_CSR), i32, vp, i32]
    L.or_column_norms.argtypes = [P(_CSR), i32, vp]
    L.or_add_mult_row.argtypes = [P(_CSR), i32, d, vp, vp, vp]
    L.or_scalar_mult.argtypes = [P(_CSR), d]
    L.or_initialise_options.argtypes = [P(_Opts)]
    L.or_sirt.argtypes = [C.c_char_p, P(_CSR), vp, i32, vp, P(_Opts), vp, i32]
    L.or_gradient_descent.argtypes = [P(_CSR), vp, i32, vp, d, d, P(_Opts), vp, vp,
                                      P(C.c_int), i32]
    L.or_normest.argtypes = [P(_CSR), d, i32, vp, i32]
    L.or_normest.restype = d
    L.or_scramble.argtypes = [i32, vp]
    L.or_sirt_adjoint.argtypes = [C.c_char_p, P(_CSR), vp, vp, i32, d, P(_Opts), vp, vp, vp,
                                  vp, P(C.c_double)]
    L.or_art.argtypes = [C.c_char_p, P(_CSR), vp, vp, i32, vp, vp, vp, i32, P(_Opts), vp]
    L.or_twin_art.argtypes = [C.c_char_p, C.c_char_p, P(_CSR), vp, vp, i32, vp, vp, vp,
                              i32, i32, P(_Opts), vp, P(C.c_int), vp, vp, vp]
    L.or_shepplogan.argtypes = [i32, vp]
    for f in ('or_smooth', 'or_grains', 'or_threephases'):
        getattr(L, f).argtypes = [i32, vp]


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


def _check(st):
    if st:
        raise OracleError(st)


@dataclass
class OracleCSR:
    """Host CSR in the reference's layout (sparse_matrices.f90:33-49)."""
    m: int
    n: int
    IA: np.ndarray  # int64, m+1, IA[0] = 0
    JA: np.ndarray  # int32, 1-based
    vA: np.ndarray  # float64

    @property
    def nnz(self):
        return int(self.IA[-1])

    def _c(self):
        s = _CSR()
        s.m, s.n, s.nnz = self.m, self.n, self.nnz
        s.IA = self.IA.ctypes.data_as(C.POINTER(C.c_int64))
        s.JA = self.JA.ctypes.data_as(C.POINTER(C.c_int32))
        s.vA = self.vA.ctypes.data_as(C.POINTER(C.c_double))
        return s


def _take(s: _CSR) -> OracleCSR:
    L = lib()
    m, n, nnz = s.m, s.n, s.nnz
    IA = np.ctypeslib.as_array(s.IA, shape=(m + 1,)).copy()
    JA = np.ctypeslib.as_array(s.JA, shape=(max(nnz, 1),))[:nnz].copy()
    vA = np.ctypeslib.as_array(s.vA, shape=(max(nnz, 1),))[:nnz].copy()
    L.or_csr_free(C.byref(s))
    return OracleCSR(m, n, IA, JA, vA)


def random_seed(seed: int):
    lib().or_random_seed(C.c_uint64(seed))


def random_number(k: int) -> np.ndarray:
    L = lib()
    return np.array([L.or_random_number() for _ in range(k)], dtype=np.float64)


def random_counter() -> int:
    return int(lib().or_random_counter())


def linspace(a, b, n):
    """system_generation.f90:17-35"""
    x = np.empty(n, np.float64)
    lib().or_linspace(a, b, n, _p(x))
    return x


def paralleltomo(n, nth, p, theta) -> OracleCSR:
    """system_generation.f90:309-492"""
    th = _f64(theta)
    s = _CSR()
    _check(lib().or_paralleltomo(n, nth, p, _p(th), C.byref(s)))
    return _take(s)


def paralleltomo_mt(n, nth, p, theta, nthreads) -> OracleCSR:
    """paralleltomo with rays split over threads (identical result)"""
    th = _f64(theta)
    s = _CSR()
    _check(lib().or_paralleltomo_mt(n, nth, p, _p(th), nthreads, C.byref(s)))
    return _take(s)


def fanlineartomo(n, nth, p, r, dw, sd, theta, geometry_fix=False) -> OracleCSR:
    """system_generation.f90:79-307 (geometry_fix=False keeps the odd-p angles of :122)"""
    th = _f64(theta)
    s = _CSR()
    _check(lib().or_fanlineartomo(n, nth, p, r, dw, sd, _p(th), int(geometry_fix), C.byref(s)))
    return _take(s)


def fanlineartomo_mt(n, nth, p, r, dw, sd, theta, nthreads, geometry_fix=False) -> OracleCSR:
    """fanlineartomo with rays split over threads (identical result)"""
    th = _f64(theta)
    s = _CSR()
    _check(lib().or_fanlineartomo_mt(n, nth, p, r, dw, sd, _p(th), int(geometry_fix), nthreads,
                                     C.byref(s)))
    return _take(s)


def add_white_noise(b, eta):
    """system_generation.f90:709-745; returns (bt, e)"""
    b = _f64(b)
    bt = np.empty_like(b)
    e = np.empty_like(b)
    _check(lib().or_add_white_noise(b.size, _p(b), eta, _p(bt), _p(e)))
    return bt, e


def rowvecmult(A: OracleCSR, k, v):
    v = _f64(v)
    return lib().or_rowvecmult(C.byref(A._c()), k, _p(v))


def matvecmul(A: OracleCSR, v, nthreads=1):
    """MMRS, sparse_matrices.f90:349-368"""
    v = _f64(v)
    if v.size != A.n:
        raise OracleError(1)
    w = np.empty(A.m, np.float64)
    lib().or_matvecmul(C.byref(A._c()), _p(v), _p(w), nthreads)
    return w


def transvecmul(A: OracleCSR, v, nthreads=1):
    """MMCS, sparse_matrices.f90:370-393: the serial scatter order, or with
    nthreads > 1 the race-free multi-threaded form (per-thread copies added
    in thread order) used to time the reference's CPU path"""
    v = _f64(v)
    if v.size != A.m:
        raise OracleError(1)
    w = np.empty(A.n, np.float64)
    if nthreads > 1:
        _check(lib().or_transvecmul_mt(C.byref(A._c()), _p(v), _p(w), nthreads))
    else:
        lib().or_transvecmul(C.byref(A._c()), _p(v), _p(w))
    return w


def transvecmul_racy(A: OracleCSR, v, nthreads):
    """MMCS as shipped under OpenMP (sparse_matrices.f90:382-392): every thread
    scatters into one shared vector, so updates can be lost; for timing only"""
    v = _f64(v)
    if v.size != A.m:
        raise OracleError(1)
    w = np.empty(A.n, np.float64)
    lib().or_transvecmul_racy(C.byref(A._c()), _p(v), _p(w), nthreads)
    return w


def set_mmcs_mode(mode: str):
    """The threaded transposed product of sirt(..., nthreads > 1): 'racefree'
    (per-thread copies, default) or 'racy' (the shipped shared scatter)"""
    lib().or_set_mmcs_mode({"racefree": 0, "racy": 1}[mode])


def reorder(A: OracleCSR) -> OracleCSR:
    """sparse_matrices.f90:492-570 -> CSR of A^T"""
    s = _CSR()
    _check(lib().or_reorder(C.byref(A._c()), C.byref(s)))
    return _take(s)


def row_norms(A: OracleCSR, p, nthreads=1):
    out = np.empty(A.m, np.float64)
    lib().or_row_norms(C.byref(A._c()), p, _p(out), nthreads)
    return out


def column_norms(A: OracleCSR, p):
    out = np.empty(A.n, np.float64)
    _check(lib().or_column_norms(C.byref(A._c()), p, _p(out)))
    return out


def add_mult_row(A: OracleCSR, k, c, w, lwrb=None, upb=None):
    """sparse_matrices.f90:795-822 (w updated in place)"""
    lb = None if lwrb is None else np.array([lwrb], np.float64)
    ub = None if upb is None else np.array([upb], np.float64)
    lib().or_add_mult_row(C.byref(A._c()), k, c, _p(w), _p(lb), _p(ub))
    return w


def scalar_mult(A: OracleCSR, c):
    lib().or_scalar_mult(C.byref(A._c()), c)


def options(relaxpar=1.0, lbound=None, ubound=None, damp=0.0, rowprobability=False):
    o = _Opts()
    lib().or_initialise_options(C.byref(o))
    o.relaxpar = relaxpar
    o.damp = damp
    o.rowprobability = int(rowprobability)
    if lbound is not None:
        o.lwrb, o.lbound = 1, lbound
    if ubound is not None:
        o.upb, o.ubound = 1, ubound
    return o


def sirt(method, A: OracleCSR, b, K, x0=None, opts=None, nthreads=1):
    """AIRMs.f90:997-1127"""
    b, x0 = _f64(b), _f64(x0)
    x = np.empty(A.n, np.float64)
    _check(lib().or_sirt(method.encode(), C.byref(A._c()), _p(b), K, _p(x0),
                         C.byref(opts) if opts is not None else None, _p(x), nthreads))
    return x


def normest(A: OracleCSR, v0, tol=1e-5, maxit=100, nthreads=1):
    """AIRMs.f90:1129-1173 with the start vector given"""
    v0 = _f64(v0)
    return lib().or_normest(C.byref(A._c()), tol, maxit, _p(v0), nthreads)


def gradient_descent(A: OracleCSR, b, max_iter=100, x0=None, rho=1.5, tol=1e-6,
                     opts=None, v0=None, nthreads=1):
    """AIRMs.f90:860-995; returns (x, iterations that updated x)"""
    b, x0, v0 = _f64(b), _f64(x0), _f64(v0)
    x = np.empty(A.n, np.float64)
    it = C.c_int(0)
    _check(lib().or_gradient_descent(C.byref(A._c()), _p(b), max_iter, _p(x0), rho, tol,
                                     C.byref(opts) if opts is not None else None,
                                     _p(v0), _p(x), C.byref(it), nthreads))
    return x, it.value


def sirt_adjoint(method, A: OracleCSR, b, K, lam, gxK, x0=None, opts=None):
    """FP64 adjoint of K unrolled SIRT steps (iteration of AIRMs.f90:1089-1110);
    returns (x_K, dL/db, dL/dx0, dL/dlam) for gxK = dL/dx_K"""
    b, x0, gxK = _f64(b), _f64(x0), _f64(gxK)
    xK = np.empty(A.n)
    gb = np.empty(A.m)
    gx0 = np.empty(A.n)
    gl = C.c_double(0.0)
    _check(lib().or_sirt_adjoint(method.encode(), C.byref(A._c()), _p(b), _p(x0), K, lam,
                                 C.byref(opts) if opts is not None else None, _p(gxK), _p(xK),
                                 _p(gb), _p(gx0), C.byref(gl)))
    return xK, gb, gx0, gl.value


def scramble(n):
    """AIRMs.f90:1175-1212"""
    out = np.empty(n, np.int32)
    lib().or_scramble(n, _p(out))
    return out


def art(method, A: OracleCSR, b, Kin, x0=None, xref=None, order=None, opts=None):
    """AIRMs.f90:59-369; returns Xout (n x len(Kin))"""
    Kin = _i32(np.atleast_1d(Kin))
    b, x0, xref, order = _f64(b), _f64(x0), _f64(xref), _i32(order)
    X = np.empty((Kin.size, A.n), np.float64)
    _check(lib().or_art(method.encode(), C.byref(A._c()), _p(b), _p(Kin), Kin.size,
                        _p(x0), _p(xref), _p(order), 0 if order is None else order.size,
                        C.byref(opts) if opts is not None else None, _p(X)))
    return X.T


def twin_art(method, stoprule, A: OracleCSR, b, Kin, x0=None, y0=None, order=None,
             slack=-1, opts=None):
    """AIRMs.f90:371-811; returns (xout, final_it, Xstore, Ystore, EG)"""
    Kin = _i32(np.atleast_1d(Kin))
    b, x0, y0, order = _f64(b), _f64(x0), _f64(y0), _i32(order)
    xout = np.empty(A.n, np.float64)
    Xs = np.empty((Kin.size, A.n), np.float64)
    Ys = np.empty((Kin.size, A.n), np.float64)
    EG = np.empty(max(int(Kin.max()), 1), np.float64)
    fi = C.c_int(0)
    _check(lib().or_twin_art(method.encode(), stoprule.encode(), C.byref(A._c()), _p(b),
                             _p(Kin), Kin.size, _p(x0), _p(y0), _p(order),
                             0 if order is None else order.size, slack,
                             C.byref(opts) if opts is not None else None, _p(xout),
                             C.byref(fi), _p(Xs), _p(Ys), _p(EG)))
    return xout, fi.value, Xs.T, Ys.T, EG


def phantom(name, N):
    """smooth (phantomgallery.f90:166-199), grains (:529-600), 3phases
    (:201-254), drawing from the oracle's stream; shepplogan (:116-164)"""
    if name == "shepplogan":
        return shepplogan(N)
    f = {"smooth": "or_smooth", "grains": "or_grains", "3phases": "or_threephases"}[name]
    v = np.empty(N * N, np.float64)
    getattr(lib(), f)(N, _p(v))
    return v


def shepplogan(N):
    """phantomgallery.f90:116-164, vectorised column-major (:672-690)"""
    v = np.empty(N * N, np.float64)
    lib().or_shepplogan(N, _p(v))
    return v
