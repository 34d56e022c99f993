"""fair_matvecmul_noalloc: the product w = A*v without any GPU allocation.

Callers that cannot call cudaMalloc while they run -- a program that has
reserved the GPU's memory for its own pool, a real-time loop that cannot take
the device synchronisation of cudaMalloc/cudaFree, a job held to a fixed
memory budget on a shared GPU -- use this entry point instead of
fair_matvecmul. It stages the vectors in a fixed device array of the library,
so its result must equal fair_matvecmul's on consecutive calls (the array is
reused), whatever value precision the handle is set to (the product is
computed in FP64), with no change in the GPU's free memory; n + m up to the
array's size must be accepted and larger problems refused.
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


def test_noalloc_computes_fp64_on_a_reduced_precision_handle(fair, oracle):
    """A handle set to q16 or f32 values still gets the FP64 product."""
    f = _entry(fair)
    n, nth, p = 40, 30, 58
    th = np.pi * np.arange(nth) / nth
    A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
    R = oracle.paralleltomo(n, nth, p, th)
    v = np.random.default_rng(4).standard_normal(A.n)
    ref = oracle.matvecmul(R, v)
    scale = oracle.matvecmul(R, np.abs(v))
    for prec in ("q16", "f32"):
        A.set_precision(prec)
        for _ in range(2):
            st, w = _call(f, A, v)
            assert st == 0
            assert _close(w, ref, scale)
    A.close()


def test_noalloc_accepts_the_largest_problem(fair):
    """n + m == FAIR_NOALLOC_MAX_ENTRIES exactly: accepted (an empty matrix
    of LIMIT - 1 rows and one column: w = 0)."""
    f = _entry(fair)
    m = LIMIT - 1
    edge = fair.CSRMatrix.construct(m, 1, np.zeros(0), np.zeros(m + 1, np.int32),
                                    np.zeros(0, np.int32))
    st, w = _call(f, edge, np.ones(1))
    assert st == 0
    assert not np.any(w)
    edge.close()


def test_noalloc_leaves_free_memory_unchanged(fair):
    """Around a call on a fresh handle whose work buffers were never grown
    (after one call elsewhere has loaded the kernels), the GPU's free memory
    does not change."""
    import torch
    f = _entry(fair)
    th = np.pi * np.arange(40) / 40
    A = fair.paralleltomo(fair.Data(n=48, p=70, nth=40, theta=th))
    assert _call(f, A, np.ones(A.n))[0] == 0  # warm: the product's kernels are loaded
    B = fair.paralleltomo(fair.Data(n=56, p=80, nth=36, theta=np.pi * np.arange(36) / 36))
    v = np.random.default_rng(2).standard_normal(B.n)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        st, w = _call(f, B, v)
        assert st == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert np.allclose(w, B.matvecmul(v), rtol=1e-13, atol=1e-13)
    A.close()
    B.close()
