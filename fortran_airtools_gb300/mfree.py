"""Matrix-free projector / backprojector pairs (include/fair_mf.h).

No counterpart in the reference, which stores the system matrix of
``paralleltomo`` (system_generation.f90:309-492) and ``fanlineartomo``
(:79-307): the entries here are the same segment lengths computed on the fly,
and the backprojector is the exact adjoint of the projector.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._clib import PREC, check, f64, lib, ptr
from .airms import options


class MatrixFree:
    """The operator of ``dat``'s geometry: ``beam="parallel"`` (paralleltomo)
    or ``beam="fan"`` (fanlineartomo; ``geometry_fix`` as there)."""

    def __init__(self, dat, prec: str = "f32", beam: str = "parallel", geometry_fix: int = 0):
        self._h = C.c_void_p()
        d = dat._c()
        if beam == "parallel":
            check(lib().fair_mf_create_parallel(C.byref(self._h), C.byref(d), PREC[prec]))
        elif beam == "fan":
            check(lib().fair_mf_create_fan(C.byref(self._h), C.byref(d), int(geometry_fix),
                                           PREC[prec]))
        else:
            raise ValueError("beam must be 'parallel' or 'fan'")
        m, n = C.c_int32(), C.c_int32()
        check(lib().fair_mf_info(self._h, C.byref(m), C.byref(n)))
        self.m, self.n, self.prec = m.value, n.value, prec

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().fair_mf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_stream(self, cuda_stream_ptr: int | None):
        check(lib().fair_mf_set_stream(self._h, cuda_stream_ptr))

    def nnz(self) -> int:
        """Nonzeros the stored matrix of this geometry would hold."""
        v = C.c_int64()
        check(lib().fair_mf_nnz(self._h, C.byref(v)))
        return v.value

    def project(self, x) -> np.ndarray:
        x = f64(x)
        if x.size != self.n:
            raise ValueError("x must have N*N entries")
        y = np.empty(self.m, np.float64)
        check(lib().fair_mf_project(self._h, ptr(x), ptr(y)))
        return y

    def backproject(self, y) -> np.ndarray:
        y = f64(y)
        if y.size != self.m:
            raise ValueError("y must have nth*p entries")
        x = np.empty(self.n, np.float64)
        check(lib().fair_mf_backproject(self._h, ptr(y), ptr(x)))
        return x

    def sirt(self, method: str, b, K: int, x0=None, opts=None) -> np.ndarray:
        b, x0 = f64(b), f64(x0)
        x = np.empty(self.n, np.float64)
        o = opts if opts is not None else options()
        check(lib().fair_mf_sirt(self._h, method.encode(), ptr(b), int(K), ptr(x0), C.byref(o),
                                 ptr(x)))
        return x

    def prepare(self, method: str, opts=None):
        o = opts if opts is not None else options()
        check(lib().fair_mf_sirt_prepare(self._h, method.encode(), C.byref(o)))

    def run_device(self, d_b: int, d_x: int, K: int):
        check(lib().fair_mf_sirt_run_device(self._h, d_b, d_x, int(K)))

    def run_device_timed(self, d_b: int, d_x: int, K: int):
        a, b = C.c_float(), C.c_float()
        check(lib().fair_mf_sirt_run_device_timed(self._h, d_b, d_x, int(K), C.byref(a),
                                                  C.byref(b)))
        return a.value, b.value
