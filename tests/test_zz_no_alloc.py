"""fair_matvecmul_noalloc: the product w = A*v without any GPU allocation.

Callers that cannot call cudaMalloc while they run -- a program that has
reserved the GPU's memory for its own pool, a real-time loop that cannot take
the device synchronisation of cudaMalloc/cudaFree, a job held to a fixed
memory budget on a shared GPU -- use this entry point instead of
fair_matvecmul. It stages the vectors in a fixed device array of the library,
so its result must equal fair_matvecmul's on consecutive calls (the array is
reused), and problems larger than the array must be refused.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT = 4194304  # FAIR_NOALLOC_MAX_ENTRIES (include/fair_gpu_ext.h)


def _entry(fair):
    f = fair.lib().fair_matvecmul_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    f.restype = C.c_int
    return f


def _call(f, A, v):
    m = A.m
    w = np.full(m, np.nan)
    v = np.ascontiguousarray(v, np.float64)
    st = f(A.handle, v.ctypes.data, v.size, w.ctypes.data)
    return st, w


def _close(w, ref, scale):
    # same tolerance as the product parity test: 1e-13 relative to |A||v|
    return np.max(np.abs(w - ref) / (scale + 1e-300)) < 1e-13


def test_noalloc_matches_matvecmul_on_consecutive_calls(fair):
    f = _entry(fair)
    rng = np.random.default_rng(0)
    th = np.pi * np.arange(90) / 90
    A = fair.paralleltomo(fair.Data(n=64, p=96, nth=90, theta=th))
    thf = 2 * np.pi * np.arange(120) / 120
    B = fair.fanlineartomo(fair.Data(n=48, p=73, nth=120, r=2.0, dw=73 / 48, sd=2.0, theta=thf))
    for M in (A, B, A):  # two calls in a row on one matrix, then another shape, then back
        for _ in range(2):
            v = rng.standard_normal(M.n)
            st, w = _call(f, M, v)
            assert st == 0, fair.lib().fair_last_error_detail()
            ref = M.matvecmul(v)
            scale = M.matvecmul(np.abs(v))
            assert _close(w, ref, scale)


def test_noalloc_size_errors(fair):
    f = _entry(fair)
    A = fair.paralleltomo(fair.Data(n=16, p=24, nth=8, theta=np.pi * np.arange(8) / 8))
    st, _ = _call(f, A, np.zeros(A.n + 1))
    assert st == 1  # "Vector input size incorrect."
    m = LIMIT  # n + m = LIMIT + 1: one entry over the array
    big = fair.CSRMatrix.construct(m, 1, np.zeros(0), np.zeros(m + 1, np.int32),
                                   np.zeros(0, np.int32))
    st, _ = _call(f, big, np.ones(1))
    assert st == 4
    assert b"FAIR_NOALLOC_MAX_ENTRIES" in fair.lib().fair_last_error_detail()
