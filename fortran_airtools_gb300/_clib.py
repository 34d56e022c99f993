"""ctypes binding of libfair_gb300.so (include/fair_gpu.h).

The library must be built (``__graft_entry__.build()`` or
``python fortran_airtools_gb300/build.py``); importing the package without it
raises instead of falling back to any CPU path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libfair_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "fair_gpu.h")

FAIR_OK = 0
FAIR_ERR_SIZE = 1
FAIR_ERR_METHOD = 2
FAIR_ERR_GEOMETRY = 3
FAIR_ERR_ARG = 4
FAIR_ERR_NEWTON = 5
FAIR_ERR_ALLOC = 6
FAIR_ERR_CUDA = 7
FAIR_ERR_NULL = 8
FAIR_ERR_STATE = 9
FAIR_ERR_NOGPU = 10

PREC = {"f64": 0, "f32": 1, "f16": 2, "q16": 3}


class FairError(RuntimeError):
    """A non-zero status of the C-ABI; the message is the reference's text."""

    def __init__(self, status: int, detail: str = ""):
        text = _lib_handle.fair_error_string(status).decode() if _lib_handle else str(status)
        super().__init__(f"{text}" + (f" [{detail}]" if detail else ""))
        self.status = status
        self.detail = detail


class Data(C.Structure):
    """type(data), system_generation.f90:6-12 (theta in radians)."""
    _fields_ = [("n", C.c_int32), ("p", C.c_int32), ("nth", C.c_int32),
                ("r", C.c_double), ("dw", C.c_double), ("sd", C.c_double),
                ("theta", C.c_void_p)]


class Opts(C.Structure):
    """type(opts), AIRMs.f90:6-13."""
    _fields_ = [("relaxpar", C.c_double), ("ubound", C.c_double), ("lbound", C.c_double),
                ("damp", C.c_double), ("verbose", C.c_int32), ("upb", C.c_int32),
                ("lwrb", C.c_int32), ("rowprobability", C.c_int32)]

    def initialise(self):
        check(lib().fair_opts_initialise(C.byref(self)))
        return self

    def set_ubound(self, ub):
        check(lib().fair_opts_set_ubound(C.byref(self), float(ub)))
        return self

    def set_lbound(self, lb):
        check(lib().fair_opts_set_lbound(C.byref(self), float(lb)))
        return self


_lib_handle = None


def lib():
    global _lib_handle
    if _lib_handle is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        L = C.CDLL(LIB_PATH)
        _declare(L)
        _lib_handle = L
    return _lib_handle


def _declare(L):
    P, vp, d, i32, i64 = C.POINTER, C.c_void_p, C.c_double, C.c_int32, C.c_int64
    h = C.c_void_p
    sig = {
        "fair_error_string": ([C.c_int], C.c_char_p),
        "fair_last_error_detail": ([], C.c_char_p),
        "fair_csr_create": ([P(h)], C.c_int),
        "fair_csr_destroy": ([h], C.c_int),
        "fair_csr_set_stream": ([h, vp], C.c_int),
        "fair_csr_info": ([h, P(i32), P(i32), P(i64)], C.c_int),
        "fair_csr_set_precision": ([h, i32], C.c_int),
        "fair_construct_csr_matrix": ([i32, i32, vp, vp, vp, h], C.c_int),
        "fair_construct_csr_matrix64": ([i32, i32, vp, vp, vp, h], C.c_int),
        "fair_csr_download": ([h, vp, vp, vp], C.c_int),
        "fair_linspace": ([d, d, i32, vp], C.c_int),
        "fair_paralleltomo": ([P(Data), h], C.c_int),
        "fair_fanlineartomo": ([P(Data), i32, h], C.c_int),
        "fair_add_white_noise": ([vp, vp, vp, i64, d], C.c_int),
        "fair_matvecmul": ([h, vp, i64, vp], C.c_int),
        "fair_transvecmul": ([h, vp, i64, vp], C.c_int),
        "fair_rowvecmult": ([h, i32, vp, i64, vp], C.c_int),
        "fair_add_scalar_mult_row": ([h, i32, d, vp, i64, vp, vp], C.c_int),
        "fair_row_norms": ([h, i32, vp], C.c_int),
        "fair_column_norms": ([h, i32, vp], C.c_int),
        "fair_transpose": ([h], C.c_int),
        "fair_multiply_by_scalar": ([h, d], C.c_int),
        "fair_opts_initialise": ([P(Opts)], C.c_int),
        "fair_opts_set_ubound": ([P(Opts), d], C.c_int),
        "fair_opts_set_lbound": ([P(Opts), d], C.c_int),
        "fair_sirt": ([vp, C.c_char_p, h, vp, vp, i32, vp, P(Opts)], C.c_int),
        "fair_gradient_descent": ([vp, h, vp, vp, vp, vp, vp, P(Opts), vp], C.c_int),
        "fair_normest": ([h, vp, vp, vp], C.c_int),
        "fair_art": ([vp, C.c_char_p, h, vp, vp, i32, vp, vp, vp, i32, P(Opts)], C.c_int),
        "fair_twin_art": ([vp, vp, vp, vp, vp, C.c_char_p, C.c_char_p, h, vp, vp, i32, vp, vp,
                           vp, i32, i32, P(Opts)], C.c_int),
        "fair_scramble": ([i32, vp], C.c_int),
        "fair_random_seed": ([C.c_uint64], C.c_int),
        "fair_random_number": ([vp, i64], C.c_int),
        "fair_shepplogan": ([i32, vp], C.c_int),
        "fair_sirt_adjoint": ([h, C.c_char_p, i32, vp, vp, i32, vp, P(Opts), vp, vp, vp, vp, vp],
                              C.c_int),
        "fair_csr_packed_info": ([h, i32, P(i32), P(i64), P(i64), P(i32), P(i32)], C.c_int),
        "fair_csr_sliced_info": ([h, i32, P(i32), P(i64)], C.c_int),
        "fair_csr_tiled_info": ([h, i32, vp], C.c_int),
        "fair_sirt_set_tiles": ([h, vp], C.c_int),
        "fair_paralleltomo_f32": ([P(Data), i32, h], C.c_int),
        "fair_sirt_autotune": ([h, vp, vp, i32, vp], C.c_int),
        "fair_sirt_prepare": ([h, C.c_char_p, P(Opts)], C.c_int),
        "fair_sirt_run_device": ([h, vp, vp, i32], C.c_int),
        "fair_sirt_run_device_timed": ([h, vp, vp, i32, P(C.c_float), P(C.c_float)], C.c_int),
        "fair_sirt_launches": ([h, i32, P(i64)], C.c_int),
        "fair_spmv_device": ([h, i32, vp, vp], C.c_int),
        "fair_matvecmul_noalloc": ([h, vp, i64, vp], C.c_int),
        "fair_write_csr_file": ([C.c_char_p, i32, i32, i32, vp, vp, vp], C.c_int),
        "fair_read_csr_file_sizes": ([C.c_char_p, P(i32), P(i32), P(i32)], C.c_int),
        "fair_read_csr_file": ([C.c_char_p, vp, vp, vp], C.c_int),
        "fair_store_matrix": ([h, C.c_char_p], C.c_int),
        "fair_read_csr_matrix": ([h, C.c_char_p], C.c_int),
        "fair_read_data_sizes": ([C.c_char_p, P(i32), P(i32), P(i32)], C.c_int),
        "fair_read_data": ([C.c_char_p, vp, vp, vp], C.c_int),
        "fair_read_ordering": ([C.c_char_p, P(i32), vp, i32], C.c_int),
        "fair_read_ref": ([C.c_char_p, i64, vp], C.c_int),
        "fair_write_values": ([C.c_char_p, vp, i64], C.c_int),
        "fair_phantom": ([C.c_char_p, i32, vp], C.c_int),
        "fair_phantom_device": ([C.c_char_p, i32, vp, vp], C.c_int),
        "fair_add_white_noise_device": ([vp, vp, vp, i64, d, vp], C.c_int),
        "fair_mf_create_parallel": ([P(h), P(Data), i32], C.c_int),
        "fair_mf_create_fan": ([P(h), P(Data), i32, i32], C.c_int),
        "fair_mf_destroy": ([h], C.c_int),
        "fair_mf_set_stream": ([h, vp], C.c_int),
        "fair_mf_info": ([h, P(i32), P(i32)], C.c_int),
        "fair_mf_project": ([h, vp, vp], C.c_int),
        "fair_mf_nnz": ([h, P(i64)], C.c_int),
        "fair_mf_backproject": ([h, vp, vp], C.c_int),
        "fair_mf_sirt": ([h, C.c_char_p, vp, i32, vp, P(Opts), vp], C.c_int),
        "fair_mf_sirt_prepare": ([h, C.c_char_p, P(Opts)], C.c_int),
        "fair_mf_sirt_run_device": ([h, vp, vp, i32], C.c_int),
        "fair_mf_sirt_run_device_timed": ([h, vp, vp, i32, P(C.c_float), P(C.c_float)], C.c_int),
        "fair_batch_create": ([P(h), i32], C.c_int),
        "fair_batch_destroy": ([h], C.c_int),
        "fair_batch_set_stream": ([h, vp], C.c_int),
        "fair_batch_set_layout": ([h, i32], C.c_int),
        "fair_batch_add": ([h, h, i32], C.c_int),
        "fair_batch_info": ([h, P(i32), P(i64), P(i64), P(i64), P(i64)], C.c_int),
        "fair_batch_problem_layout": ([h, i32, vp], C.c_int),
        "fair_batch_offsets": ([h, vp, vp], C.c_int),
        "fair_batch_pass_bytes": ([h, i32, P(i64), P(i64)], C.c_int),
        "fair_batch_sirt": ([h, C.c_char_p, vp, i32, vp, P(Opts), vp], C.c_int),
        "fair_batch_prepare": ([h, C.c_char_p, P(Opts)], C.c_int),
        "fair_batch_run_device": ([h, vp, vp, i32], C.c_int),
        "fair_batch_run_device_unbatched": ([h, vp, vp, i32], C.c_int),
        "fair_batch_launches": ([h, i32, P(i64)], C.c_int),
        "fair_batch_autotune": ([h, vp, vp, i32, vp], C.c_int),
        "fair_batch_set_config": ([h, vp], C.c_int),
        "fair_sirt_set_lanes": ([h, vp], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res


def check(status: int):
    if status != FAIR_OK:
        detail = lib().fair_last_error_detail()
        raise FairError(status, detail.decode() if detail else "")


def ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)
