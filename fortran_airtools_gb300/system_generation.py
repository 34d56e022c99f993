"""Host mirror of module system_generation (system_generation.f90).

``paralleltomo`` / ``fanlineartomo`` build the ray-traced CSR system matrix on
the GPU and return a ``CSRMatrix``; ``Data`` is type(data) with theta in
radians and r, dw, sd in units of n (the reference's scaling, :98-100).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from ._clib import Data as _CData, check, f64, lib, ptr
from .sparse_matrices import CSRMatrix

pi = 4.0 * np.arctan(1.0)  # system_generation.f90:4


@dataclass
class Data:
    """type(data), system_generation.f90:6-12."""
    n: int
    p: int
    nth: int
    r: float = 0.0
    dw: float = 0.0
    sd: float = 0.0
    theta: np.ndarray = field(default_factory=lambda: np.zeros(0))

    def _c(self):
        self._theta = f64(self.theta)
        if self._theta.size != self.nth:
            raise ValueError("Angle vector has the wrong length, nth is incorrect.")
        return _CData(self.n, self.p, self.nth, self.r, self.dw, self.sd,
                      self._theta.ctypes.data_as(C.c_void_p))


def linspace(a, b, n):
    """system_generation.f90:17-35 (x(i) = c*i + d)."""
    x = np.empty(n, np.float64)
    check(lib().fair_linspace(float(a), float(b), int(n), ptr(x)))
    return x


def paralleltomo(dat: Data) -> CSRMatrix:
    """system_generation.f90:309-492, built on the GPU."""
    A = CSRMatrix()
    d = dat._c()
    check(lib().fair_paralleltomo(C.byref(d), A.handle))
    return A


def paralleltomo_f32(dat: Data, block_angles: int = 0) -> CSRMatrix:
    """paralleltomo held in FP32 only (A and A' as FP32 values, int32 columns,
    int64 row offsets), built on the GPU by blocks of angles; for problems
    whose FP64 matrix does not fit. The handle runs FP32 products and SIRT."""
    A = CSRMatrix()
    d = dat._c()
    check(lib().fair_paralleltomo_f32(C.byref(d), int(block_angles), A.handle))
    return A


def fanlineartomo(dat: Data, geometry_fix: bool = False) -> CSRMatrix:
    """system_generation.f90:79-307, built on the GPU. geometry_fix=False keeps
    the reference's odd-p ray angles (system_generation.f90:122)."""
    A = CSRMatrix()
    d = dat._c()
    check(lib().fair_fanlineartomo(C.byref(d), int(bool(geometry_fix)), A.handle))
    return A


def add_white_noise(b, eta):
    """system_generation.f90:709-745; returns (bt, e). Draws from the library stream."""
    b = f64(b)
    bt = np.empty_like(b)
    e = np.empty_like(b)
    check(lib().fair_add_white_noise(ptr(bt), ptr(e), ptr(b), b.size, float(eta)))
    return bt, e


__all__ = ["Data", "linspace", "paralleltomo", "paralleltomo_f32", "fanlineartomo", "add_white_noise", "pi"]
