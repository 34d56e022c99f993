"""Host mirror of module sparse_matrices (sparse_matrices.f90).

``CSRMatrix`` is type(csr_matrix) (sparse_matrices.f90:157-173): the matrix
lives on the GPU inside a fair_csr handle and each type-bound procedure is
one C-ABI call. Vectors are numpy float64 arrays on the host; size errors
raise FairError with the reference's "Vector input size incorrect." text.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._clib import FairError, PREC, check, f64, i32, lib, ptr


class CSRMatrix:
    """type(csr_matrix) on the GPU."""

    def __init__(self):
        h = C.c_void_p()
        check(lib().fair_csr_create(C.byref(h)))
        self._h = h

    # -- lifetime -------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().fair_csr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- shape (sparse_matrices.f90:47) -----------------------------------------
    def info(self):
        m, n, nnz = C.c_int32(), C.c_int32(), C.c_int64()
        check(lib().fair_csr_info(self._h, C.byref(m), C.byref(n), C.byref(nnz)))
        return m.value, n.value, nnz.value

    @property
    def m(self):
        return self.info()[0]

    @property
    def n(self):
        return self.info()[1]

    @property
    def nnz(self):
        return self.info()[2]

    def set_precision(self, prec: str):
        """Value storage used by products and SIRT: 'f64', 'f32', 'f16' or 'q16'."""
        check(lib().fair_csr_set_precision(self._h, PREC[prec]))

    def packed_info(self, transposed: bool = False) -> dict:
        """Packed index stream of A (or A'), built by the first reduced-precision
        SIRT: {'has', 'ngroups', 'nesc', 'stride', 'low_bits', 'sliced',
        'nslots'} ('sliced': its SELL-32 copy is built, with 'nslots' slots)."""
        has, S, L, sl = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        ng, ne, ns = C.c_int64(), C.c_int64(), C.c_int64()
        which = 1 if transposed else 0
        check(lib().fair_csr_packed_info(self._h, which, C.byref(has),
                                         C.byref(ng), C.byref(ne), C.byref(S), C.byref(L)))
        check(lib().fair_csr_sliced_info(self._h, which, C.byref(sl), C.byref(ns)))
        return {"has": bool(has.value), "ngroups": ng.value, "nesc": ne.value,
                "stride": S.value, "low_bits": L.value, "sliced": bool(sl.value),
                "nslots": ns.value}

    def tiled_info(self, transposed: bool = False) -> dict:
        """Tiled copy of A (or A') for the SIRT passes on layouts 9, 10, 14:
        {'has', 'tile', 'tiles_per_side', 'angles_per_block', 'angle_blocks',
        'window', 'units', 'kind'}."""
        v = (C.c_int32 * 8)()
        check(lib().fair_csr_tiled_info(self._h, 1 if transposed else 0, v))
        keys = ("has", "tile", "tiles_per_side", "angles_per_block", "angle_blocks", "window",
                "units", "kind")
        d = dict(zip(keys, list(v)))
        d["has"] = bool(d["has"])
        return d

    def set_stream(self, cuda_stream_ptr: int | None):
        check(lib().fair_csr_set_stream(self._h, cuda_stream_ptr))

    # -- construction / transfer -------------------------------------------------
    @classmethod
    def construct(cls, m, n, vA, IA, JA):
        """construct_csr_matrix, sparse_matrices.f90:180-197 (JA 1-based)."""
        A = cls()
        vA, JA = f64(vA), i32(JA)
        IA = np.ascontiguousarray(IA)
        if IA.dtype == np.int64:
            check(lib().fair_construct_csr_matrix64(m, n, ptr(vA), ptr(IA), ptr(JA), A._h))
        else:
            IA = i32(IA)
            check(lib().fair_construct_csr_matrix(m, n, ptr(vA), ptr(IA), ptr(JA), A._h))
        return A

    def arrays(self):
        """(vA, IA int64 with IA[0] = 0, JA 1-based) copied to the host."""
        m, n, nnz = self.info()
        vA = np.empty(nnz, np.float64)
        IA = np.empty(m + 1, np.int64)
        JA = np.empty(nnz, np.int32)
        check(lib().fair_csr_download(self._h, ptr(vA), ptr(IA), ptr(JA)))
        return vA, IA, JA

    # -- type-bound procedures ------------------------------------------------------
    def matvecmul(self, v):
        """w = A*v, sparsematmul/MMRS (sparse_matrices.f90:272-298, :349-368)."""
        v = f64(v)
        w = np.empty(self.m, np.float64)
        check(lib().fair_matvecmul(self._h, ptr(v), v.size, ptr(w)))
        return w

    def transvecmul(self, v):
        """w = A'*v, sparsetransmul/MMCS (sparse_matrices.f90:300-347, :370-393)."""
        v = f64(v)
        w = np.empty(self.n, np.float64)
        check(lib().fair_transvecmul(self._h, ptr(v), v.size, ptr(w)))
        return w

    def rowvecmult(self, k, v):
        """csr_matrowvec, sparse_matrices.f90:252-270 (k 1-based)."""
        v = f64(v)
        f = np.zeros(1, np.float64)
        check(lib().fair_rowvecmult(self._h, int(k), ptr(v), v.size, ptr(f)))
        return float(f[0])

    def add_scalar_mult_row(self, k, c, w, lwrb=None, upb=None):
        """add_mult_row, sparse_matrices.f90:795-822; w (float64) updated in place."""
        if w.dtype != np.float64 or not w.flags.c_contiguous:
            raise TypeError("w must be a contiguous float64 array")
        lb = None if lwrb is None else np.array([lwrb], np.float64)
        ub = None if upb is None else np.array([upb], np.float64)
        check(lib().fair_add_scalar_mult_row(self._h, int(k), float(c), ptr(w), w.size,
                                             ptr(lb), ptr(ub)))
        return w

    def row_norms(self, p):
        """compute_row_norms, sparse_matrices.f90:740-780."""
        out = np.empty(self.m, np.float64)
        check(lib().fair_row_norms(self._h, int(p), ptr(out)))
        return out

    def column_norms(self, p):
        """compute_column_norms, sparse_matrices.f90:782-793."""
        out = np.empty(self.n, np.float64)
        check(lib().fair_column_norms(self._h, int(p), ptr(out)))
        return out

    def transpose(self):
        """transposition, sparse_matrices.f90:395-411 (in place)."""
        check(lib().fair_transpose(self._h))

    def multiply_by_scalar(self, c):
        """scalar_mult, sparse_matrices.f90:824-831."""
        check(lib().fair_multiply_by_scalar(self._h, float(c)))


__all__ = ["CSRMatrix", "FairError"]
