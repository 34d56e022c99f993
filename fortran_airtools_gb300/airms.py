"""Host mirror of module AIRMs (AIRMs.f90).

Every solver runs on the GPU through one C-ABI call; arguments keep the
reference's names, meaning and optional-argument defaults. Random numbers
(scramble, row sampling, the normest start vector) come from the library's
seeded stream (``random_seed``) instead of the unseeded Fortran
random_number, consumed in the same order.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._clib import Opts, check, f64, i32, lib, ptr
from .sparse_matrices import CSRMatrix


def options(relaxpar=1.0, lbound=None, ubound=None, damp=0.0, rowprobability=False,
            verbose=False) -> Opts:
    """initialise_options + set_lbound/set_ubound (AIRMs.f90:17-57)."""
    o = Opts().initialise()
    o.relaxpar = float(relaxpar)
    o.damp = float(damp)
    o.rowprobability = int(bool(rowprobability))
    o.verbose = int(bool(verbose))
    if lbound is not None:
        o.set_lbound(lbound)
    if ubound is not None:
        o.set_ubound(ubound)
    return o


def random_seed(seed: int):
    check(lib().fair_random_seed(C.c_uint64(int(seed))))


def random_number(k: int):
    u = np.empty(int(k), np.float64)
    check(lib().fair_random_number(ptr(u), int(k)))
    return u


def _kin(K):
    return i32(np.atleast_1d(K))


def sirt(sirt_method: str, A: CSRMatrix, b, Kin, x0=None, opts: Opts | None = None):
    """sirt, AIRMs.f90:997-1127: returns xout."""
    b, x0, Kin = f64(b), f64(x0), _kin(Kin)
    x = np.empty(A.n, np.float64)
    check(lib().fair_sirt(ptr(x), sirt_method.encode(), A.handle, ptr(b), ptr(Kin), Kin.size,
                          ptr(x0), C.byref(opts) if opts is not None else None))
    return x


def gradient_descent(A: CSRMatrix, b, max_iter=None, x0=None, rho_in=None, tolerance=None,
                     opts: Opts | None = None):
    """gradient_descent, AIRMs.f90:860-995: returns (xout, accepted steps)."""
    b, x0 = f64(b), f64(x0)
    x = np.empty(A.n, np.float64)
    mi = None if max_iter is None else np.array([max_iter], np.int32)
    rh = None if rho_in is None else np.array([rho_in], np.float64)
    tl = None if tolerance is None else np.array([tolerance], np.float64)
    it = np.zeros(1, np.int32)
    check(lib().fair_gradient_descent(ptr(x), A.handle, ptr(b), ptr(mi), ptr(x0), ptr(rh),
                                      ptr(tl), C.byref(opts) if opts is not None else None,
                                      ptr(it)))
    return x, int(it[0])


def normest(A: CSRMatrix, tolerance=None, max_its=None):
    """normest, AIRMs.f90:1129-1173."""
    tl = None if tolerance is None else np.array([tolerance], np.float64)
    mi = None if max_its is None else np.array([max_its], np.int32)
    s = np.zeros(1, np.float64)
    check(lib().fair_normest(A.handle, ptr(tl), ptr(mi), ptr(s)))
    return float(s[0])


def art(art_method: str, A: CSRMatrix, b, Kin, x0=None, xref=None, order=None,
        opts: Opts | None = None):
    """art, AIRMs.f90:59-369: returns Xout (n x len(Kin))."""
    b, x0, xref, order, Kin = f64(b), f64(x0), f64(xref), i32(order), _kin(Kin)
    X = np.empty((Kin.size, A.n), np.float64)
    check(lib().fair_art(ptr(X), art_method.encode(), A.handle, ptr(b), ptr(Kin), Kin.size,
                         ptr(x0), ptr(xref), ptr(order), 0 if order is None else order.size,
                         C.byref(opts) if opts is not None else None))
    return X.T


def twin_art(art_method: str, stoprule: str, A: CSRMatrix, b, Kin, x0=None, y0=None,
             order=None, slack=None, opts: Opts | None = None):
    """twin_art, AIRMs.f90:371-811: returns (xout, final_it, Xstore, Ystore, EG)."""
    b, x0, y0, order, Kin = f64(b), f64(x0), f64(y0), i32(order), _kin(Kin)
    n = A.n
    xout = np.empty(n, np.float64)
    Xs = np.empty((Kin.size, n), np.float64)
    Ys = np.empty((Kin.size, n), np.float64)
    EG = np.empty(max(int(Kin.max()), 1), np.float64)
    fi = np.zeros(1, np.int32)
    check(lib().fair_twin_art(ptr(xout), ptr(fi), ptr(Xs), ptr(Ys), ptr(EG),
                              art_method.encode(), stoprule.encode(), A.handle, ptr(b), ptr(Kin),
                              Kin.size, ptr(x0), ptr(y0), ptr(order),
                              0 if order is None else order.size,
                              -1 if slack is None else int(slack),
                              C.byref(opts) if opts is not None else None))
    return xout, int(fi[0]), Xs.T, Ys.T, EG


def sirt_adjoint(sirt_method: str, A: CSRMatrix, b, K: int, lam, gx, x0=None,
                 opts: Opts | None = None):
    """Reverse-mode adjoint of K unrolled SIRT steps (fair_sirt_adjoint).

    b: (m,) or (m, nrhs); lam: scalar or (nrhs,); gx = dL/dx_K with the shape of
    x_K. Returns (x_K, dL/db, dL/dx0, dL/dlam) with the shapes of x_K, b, x_K, lam.
    Only the bounds of ``opts`` are used (lam is the relaxation parameter)."""
    b = np.asarray(b, np.float64)
    single = b.ndim == 1
    B = b.reshape(b.shape[0], -1)
    nrhs = B.shape[1]
    lam_arr = np.broadcast_to(np.asarray(lam, np.float64), (nrhs,)).copy()
    Bc = np.asfortranarray(B)
    GX = np.asfortranarray(np.asarray(gx, np.float64).reshape(A.n, nrhs))
    X0 = None if x0 is None else np.asfortranarray(np.asarray(x0, np.float64).reshape(A.n, nrhs))
    XK = np.zeros((A.n, nrhs), order="F")
    GB = np.zeros((A.m, nrhs), order="F")
    GX0 = np.zeros((A.n, nrhs), order="F")
    GL = np.zeros(nrhs)
    check(lib().fair_sirt_adjoint(A.handle, sirt_method.encode(), nrhs, ptr(Bc), ptr(X0), int(K),
                                  ptr(lam_arr), C.byref(opts) if opts is not None else None,
                                  ptr(GX), ptr(XK), ptr(GB), ptr(GX0), ptr(GL)))
    if single:
        return XK[:, 0], GB[:, 0], GX0[:, 0], float(GL[0])
    return XK, GB, GX0, GL


def scramble(number_of_values: int):
    """scramble, AIRMs.f90:1175-1212."""
    out = np.empty(int(number_of_values), np.int32)
    check(lib().fair_scramble(int(number_of_values), ptr(out)))
    return out


__all__ = ["options", "random_seed", "random_number", "sirt", "gradient_descent", "normest",
           "art", "twin_art", "scramble"]
