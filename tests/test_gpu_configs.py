"""Parity with the oracle at the sizes the measured workloads run at.

The other GPU modules check every kernel and layout on small geometries;
this one checks the configurations the benchmark figures are quoted on, on
the layouts those figures use:

* parallel beam N=1024, 720 angles over [0, pi), 1448 bins (961,254,632
  nonzeros): the GPU matrix against the oracle's (IA, JA bit-exact, vA within
  1e-12 relative), then 3 Cimmino iterations on the layouts the autotuner
  picks and on pinned tiled / sliced / delta layouts: FP64 within 1e-10 of
  the oracle, the FP32 and 16-bit forms within 1e-5 of the oracle's FP64
  iterate;
* the tiled copy of A' with more than one block of angles (fan N=48 and
  parallel N=64, 720 angles): both pass-2 tiled codes in FP64 and q16;
* fan beam N=512, 720 angles over [0, 2pi), 725 bins (odd p: the ray angles
  of system_generation.f90:122), R = 2N: matrix bit-exact, then one sweep of
  random Kaczmarz with row-norm probabilities and one symmetric pair, bounds
  [0, 1], within 1e-10 (the same draws on both sides);
* parallel beam N=256, 360 angles over [0, pi), 362 bins: matrix, and the
  adjoint of 20 Cimmino steps for two right-hand sides against the oracle's
  FP64 adjoint. 363 bins (odd p) put a ray on the top edge at theta = pi/2
  whose direction has b = cos(pi/2) = 6e-17 != 0: the reference stops there
  with "++ Something went wrong" (system_generation.f90:478), and so do both
  the oracle and the GPU build, so this workload runs at 362 bins;
* the first 8 problems of the batch workload (seed 2) at their own sizes,
  through the tiled batch in FP32 (autotuned): within 1e-5 of the oracle's
  SART.

The oracle builds run on all host threads (identical to the serial builds,
tests/test_oracle_kat.py) and its SIRT iterations use the row-parallel
product and the race-free threaded transposed product.
"""
import ctypes as C
import math
import os

import numpy as np
import pytest

from conftest import rel_err

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

NT = os.cpu_count() or 1
MIXED_TOL = 1e-5  # reduced-precision forms against the FP64 oracle


def noisy(b, eta, seed):
    """b + e, e seeded Gaussian scaled to ||e|| = eta ||b|| (add_white_noise's scaling)."""
    e = np.random.default_rng(seed).standard_normal(b.size)
    return b + e * (eta * np.linalg.norm(b) / np.linalg.norm(e))


def compare_matrix(A, R):
    vA, IA, JA = A.arrays()
    assert (A.m, A.n) == (R.m, R.n)
    assert np.array_equal(IA, R.IA), "row offsets differ"
    assert np.array_equal(JA, R.JA), "column indices differ"
    rel = np.max(np.abs(vA - R.vA) / np.maximum(np.abs(R.vA), 1e-300)) if R.nnz else 0.0
    assert rel <= 1e-12, f"max relative vA difference {rel}"
    return rel


def set_layout(A, cfg):
    from fortran_airtools_gb300._clib import check, lib
    check(lib().fair_sirt_set_lanes(A.handle, (C.c_int32 * 4)(*cfg)))


# ------------------------------------------------------------ N=1024 parallel ----
@pytest.fixture(scope="module")
def c2(fair, oracle):
    n, nth, p = 1024, 720, 1448
    th = np.pi * np.arange(nth) / nth
    A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
    R = oracle.paralleltomo_mt(n, nth, p, th, NT)
    xt = fair.phantomgallery.gaussians(n, 20, seed=1)
    b = noisy(oracle.matvecmul(R, xt, nthreads=NT), 0.01, 1)
    xr = oracle.sirt("cimmino", R, b, 3, nthreads=NT)
    yield A, R, b, xr
    A.close()


def test_c2_matrix(c2):
    A, R, _, _ = c2
    assert R.nnz == 961254632
    compare_matrix(A, R)


def _autotuned(fair, A, b, prec):
    import torch
    from fortran_airtools_gb300._clib import check, lib
    L = lib()
    opts = fair.airms.options()
    check(L.fair_sirt_prepare(A.handle, b"cimmino", C.byref(opts)))
    d_b = torch.from_numpy(b).cuda()
    d_x = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    cfg = (C.c_int32 * 4)()
    check(L.fair_sirt_autotune(A.handle, d_b.data_ptr(), d_x.data_ptr(), 2, cfg))
    torch.cuda.synchronize()
    return tuple(cfg)


@pytest.mark.parametrize("prec,layouts", [
    ("f64", [None, (8, 1, 9, 5), (8, 8, 9, 13), (8, 8, 9, 10)]),
    ("f32", [None, (8, 8, 9, 10), (8, 8, 9, 13)]),
    ("f16", [None, (8, 8, 14, 14), (8, 8, 10, 10)]),
    ("q16", [None, (8, 8, 14, 14), (8, 8, 9, 11)]),
])
def test_c2_sirt(c2, fair, prec, layouts):
    """3 Cimmino iterations (reference defaults: relaxation 1, no bounds)."""
    A, R, b, xr = c2
    tol = 1e-10 if prec == "f64" else MIXED_TOL
    A.set_precision(prec)
    try:
        for cfg in layouts:
            if cfg is None:
                cfg = _autotuned(fair, A, b, prec)
            else:
                set_layout(A, cfg)
            x = fair.airms.sirt("cimmino", A, b, 3)
            err = rel_err(x, xr)
            print(f"N=1024 {prec} layouts {cfg}: rel err vs oracle {err:.3e}")
            assert err < tol, (prec, cfg, err)
    finally:
        A.set_precision("f64")


def test_c2_multi_angle_blocks_built(c2, fair):
    """At N=1024 the tiled copy of A' holds several blocks of angles."""
    A, _, b, _ = c2
    A.set_precision("q16")
    try:
        set_layout(A, (8, 8, 14, 14))
        fair.airms.sirt("cimmino", A, b, 1)
        info = A.tiled_info(transposed=True)
    finally:
        A.set_precision("f64")
    assert info["has"] and info["kind"] == 1 and info["angle_blocks"] > 1


# ------------------------------------------------- A' tiles, several angle blocks ----
@pytest.fixture(scope="module", params=["fan48", "par64"])
def blocks(request, fair, oracle):
    if request.param == "fan48":
        n, nth, p = 48, 720, 69
        th = 2 * np.pi * np.arange(nth) / nth
        A = fair.fanlineartomo(fair.Data(n=n, p=p, nth=nth, r=2.0, dw=p / n, sd=2.0, theta=th))
        R = oracle.fanlineartomo(n, nth, p, 2.0, p / n, 2.0, th)
    else:
        n, nth, p = 64, 720, 90  # odd p puts a ray on the top edge at theta = pi/2
        th = np.pi * np.arange(nth) / nth
        A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
        R = oracle.paralleltomo(n, nth, p, th)
    b = oracle.matvecmul(R, fair.phantomgallery.shepplogan(n))
    yield A, R, b
    A.close()


@pytest.mark.parametrize("prec", ["f64", "q16"])
@pytest.mark.parametrize("code", [10, 14])
def test_tiled_transpose_angle_blocks(blocks, fair, oracle, prec, code):
    A, R, b = blocks
    o = fair.airms.options(lbound=0.0, ubound=1.0)
    A.set_precision(prec)
    try:
        set_layout(A, (8, 8, 0, code))
        xt = fair.airms.sirt("sart", A, b, 15, opts=o)
        info = A.tiled_info(transposed=True)
        set_layout(A, (8, 8, 0, 0))
        xc = fair.airms.sirt("sart", A, b, 15, opts=o)
    finally:
        set_layout(A, (8, 8, 0, 0) if prec == "f64" else (8, 8, 1, 1))
        A.set_precision("f64")
    assert info["has"] and info["angle_blocks"] > 1, info
    assert rel_err(xt, xc) < (1e-12 if prec == "f64" else 2e-6)
    xr = oracle.sirt("sart", R, b, 15, opts=oracle.options(lbound=0.0, ubound=1.0))
    assert rel_err(xt, xr) < (1e-10 if prec == "f64" else 1e-4)


# ------------------------------------------------------------ N=512 fan beam ----
@pytest.fixture(scope="module")
def c5a(fair, oracle):
    n, nth, p = 512, 720, 725
    th = 2 * np.pi * np.arange(nth) / nth
    A = fair.fanlineartomo(fair.Data(n=n, p=p, nth=nth, r=2.0, dw=p / n, sd=2.0, theta=th))
    R = oracle.fanlineartomo_mt(n, nth, p, 2.0, p / n, 2.0, th, NT)
    xt = fair.phantomgallery.three_phases(n, seed=4)
    b = noisy(oracle.matvecmul(R, xt, nthreads=NT), 0.01, 4)
    yield A, R, b
    A.close()


def test_c5a_matrix(c5a):
    A, R, _ = c5a
    assert R.nnz == 124277580
    compare_matrix(A, R)


@pytest.mark.parametrize("method,K,rowprob", [("randkaczmarz", 1, True), ("symkaczmarz", 2, False)])
def test_c5a_kaczmarz(c5a, fair, oracle, method, K, rowprob):
    A, R, b = c5a
    o = fair.airms.options(lbound=0.0, ubound=1.0, rowprobability=rowprob)
    ro = oracle.options(lbound=0.0, ubound=1.0, rowprobability=rowprob)
    fair.airms.random_seed(4)
    oracle.random_seed(4)
    X = fair.airms.art(method, A, b, [K], opts=o)
    Xr = oracle.art(method, R, b, [K], opts=ro)
    err = rel_err(X[:, 0], Xr[:, 0])
    print(f"N=512 fan {method} K={K}: rel err vs oracle {err:.3e}")
    assert err < 1e-10


# ---------------------------------------------------- N=256 parallel, 362 bins ----
@pytest.fixture(scope="module")
def c4(fair, oracle):
    n, nth, p = 256, 360, 362
    th = np.pi * np.arange(nth) / nth
    A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
    R = oracle.paralleltomo_mt(n, nth, p, th, NT)
    X = np.stack([fair.phantomgallery.random_ellipses(n, seed=3 + s) for s in range(2)], 1)
    B = np.stack([noisy(oracle.matvecmul(R, X[:, c], nthreads=NT), 0.01, 3 + c)
                  for c in range(2)], 1)
    yield A, R, X, B
    A.close()


def test_c4_matrix_and_the_363_bin_stop(c4, fair, oracle):
    A, R, _, _ = c4
    compare_matrix(A, R)
    th = np.pi * np.arange(360) / 360
    with pytest.raises(oracle.OracleError) as eo:
        oracle.paralleltomo_mt(256, 360, 363, th, NT)
    assert eo.value.code == 3
    with pytest.raises(fair.FairError) as eg:
        fair.paralleltomo(fair.Data(n=256, p=363, nth=360, theta=th))
    assert eg.value.status == 3


def test_c4_adjoint(c4, fair, oracle):
    """x_K and the gradients of L = 0.5 ||x_K - x_true||^2 for two right-hand
    sides in one call, each against the oracle's FP64 adjoint (1e-10)."""
    A, R, X, B = c4
    K, lam = 20, 1.5
    ro = oracle.options(lbound=0.0)
    GX, refs = [], []
    for c in range(2):
        xk, _, _, _ = oracle.sirt_adjoint("cimmino", R, B[:, c], K, lam, np.zeros(R.n), opts=ro)
        GX.append(xk - X[:, c])
        refs.append(oracle.sirt_adjoint("cimmino", R, B[:, c], K, lam, GX[c], opts=ro))
    xK, gb, gx0, gl = fair.airms.sirt_adjoint("cimmino", A, B, K, np.full(2, lam),
                                              np.stack(GX, 1), opts=fair.airms.options(lbound=0.0))
    for c in range(2):
        rx, rb, rx0, rl = refs[c]
        assert rel_err(xK[:, c], rx) < 1e-10
        assert rel_err(gb[:, c], rb) < 1e-10
        assert rel_err(gx0[:, c], rx0) < 1e-10
        assert abs(gl[c] - rl) <= 1e-10 * abs(rl)


# ---------------------------------------------------------------- batch, seed 2 ----
def test_c3_first_problems_tiled_batch(fair, oracle):
    import torch
    nprob, K = 8, 10
    rng = np.random.default_rng(2)
    Ns = rng.choice(np.arange(64, 513, 32), 256)
    nths = rng.integers(90, 721, 256)
    cells = rng.integers(50, 401, 256)
    B = fair.Batch("f32", layout="tiled")
    Rs, bs = [], []
    for i in range(nprob):
        n, nth = int(Ns[i]), int(nths[i])
        p = int(math.ceil(1.42 * n))
        th = 2 * np.pi * np.arange(nth) / nth
        A = fair.fanlineartomo(fair.Data(n=n, p=p, nth=nth, r=2.0, dw=p / n, sd=2.0, theta=th))
        R = oracle.fanlineartomo_mt(n, nth, p, 2.0, p / n, 2.0, th, NT)
        x = fair.phantomgallery.grains(n, int(cells[i]), seed=1000 + i)
        b = noisy(oracle.matvecmul(R, x, nthreads=NT), 0.005, 1000 + i)
        B.add(A, take=True)
        A.close()
        Rs.append(R)
        bs.append(b)
    ball = np.concatenate(bs)
    o = fair.airms.options(lbound=0.0, ubound=1.0)
    B.prepare("sart", o)
    d_b = torch.from_numpy(ball).cuda()
    scratch = torch.zeros(B.info()["cols"], dtype=torch.float64, device="cuda")
    B.autotune(d_b.data_ptr(), scratch.data_ptr(), 2)
    torch.cuda.synchronize()
    X = B.sirt("sart", ball, K, opts=o)
    _, co = B.offsets()
    ro = oracle.options(lbound=0.0, ubound=1.0)
    for i, (R, b) in enumerate(zip(Rs, bs)):
        xr = oracle.sirt("sart", R, b, K, opts=ro, nthreads=NT)
        err = rel_err(X[co[i]:co[i + 1]], xr)
        print(f"batch problem {i} (N={int(Ns[i])}, {int(nths[i])} angles): rel err {err:.3e}")
        assert err < MIXED_TOL
    B.close()
