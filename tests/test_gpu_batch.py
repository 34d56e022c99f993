"""Batched SIRT/SART over problems of different sizes (include/fair_batch.h).

A batched iteration runs, problem by problem, the single-problem engine and
epilogue with the same lanes per row and groups per lane, so with the same
configuration the batch must reproduce fair_sirt on each problem bit for
bit (FP64 and the packed FP32 form); against the oracle the bars are the
single-problem ones (FP64 1e-10; f32 1e-5; f16 5e-3; q16 1e-4).
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

GEOMS = [  # (kind, N, nth, p)
    ("fan", 24, 40, 35), ("par", 32, 30, 46), ("fan", 40, 64, 57), ("par", 16, 20, 24),
    ("fan", 32, 50, 46),
]


def build(fair, oracle, kind, n, nth, p):
    if kind == "fan":
        th = 2 * np.pi * np.arange(nth) / nth
        A = fair.fanlineartomo(fair.Data(n=n, p=p, nth=nth, r=2.0, dw=p / n, sd=2.0, theta=th))
        R = oracle.fanlineartomo(n, nth, p, 2.0, p / n, 2.0, th)
    else:
        th = np.pi * np.arange(nth) / nth
        A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
        R = oracle.paralleltomo(n, nth, p, th)
    return A, R


@pytest.fixture(scope="module")
def problems(fair, oracle):
    out = []
    for i, g in enumerate(GEOMS):
        A, R = build(fair, oracle, *g)
        x = fair.phantomgallery.grains(g[1], 20 + 10 * i, seed=i)
        b = oracle.matvecmul(R, x)
        out.append((A, R, b))
    return out


def make_batch(fair, problems, prec, take=False):
    B = fair.Batch(prec)
    for A, _, _ in problems:
        B.add(A, take=take)
    return B


@pytest.mark.parametrize("method", ["sart", "cimmino"])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_batch_equals_single(problems, fair, oracle, prec, method):
    B = make_batch(fair, problems, prec)
    B.set_config([8, 8, 1, 1])  # the single-problem defaults
    o = fair.airms.options(lbound=0.0, ubound=1.0)
    ball = np.concatenate([b for _, _, b in problems])
    X = B.sirt(method, ball, 25, opts=o)
    ro, co = B.offsets()
    assert ro[-1] == ball.size
    for p, (A, R, b) in enumerate(problems):
        A.set_precision(prec)
        try:
            xs = fair.airms.sirt(method, A, b, 25, opts=o)
        finally:
            A.set_precision("f64")
        assert np.array_equal(X[co[p]:co[p + 1]], xs)
        xr = oracle.sirt(method, R, b, 25, opts=oracle.options(lbound=0.0, ubound=1.0))
        assert rel_err(X[co[p]:co[p + 1]], xr) < (1e-10 if prec == "f64" else 1e-5)
    B.close()


@pytest.mark.parametrize("prec,tol", [("f16", 5e-3), ("q16", 1e-4)])
def test_batch_16bit(problems, fair, oracle, prec, tol):
    B = make_batch(fair, problems, prec)
    ball = np.concatenate([b for _, _, b in problems])
    X = B.sirt("sart", ball, 30, opts=fair.airms.options(lbound=0.0, ubound=1.0))
    _, co = B.offsets()
    for p, (A, R, b) in enumerate(problems):
        xr = oracle.sirt("sart", R, b, 30, opts=oracle.options(lbound=0.0, ubound=1.0))
        assert rel_err(X[co[p]:co[p + 1]], xr) < tol
    B.close()


def test_device_api_graph_reuse_and_unbatched(problems, fair):
    import torch
    B = make_batch(fair, problems, "f32")
    ball = np.concatenate([b for _, _, b in problems])
    info = B.info()
    assert info["problems"] == len(problems) and info["nnz"] > 0 and info["device_bytes"] > 0
    o = fair.airms.options(lbound=0.0, ubound=1.0)
    ref = B.sirt("sart", ball, 12, opts=o)
    B.prepare("sart", o)
    stream = torch.cuda.Stream()
    B.set_stream(stream.cuda_stream)
    d_b = torch.from_numpy(ball).cuda()
    outs = []
    for K, batched in ((12, True), (12, True), (7, True), (12, False)):
        d_x = torch.zeros(info["cols"], dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        B.run_device(d_b.data_ptr(), d_x.data_ptr(), K, batched=batched)
        stream.synchronize()
        outs.append((K, d_x.cpu().numpy()))
    assert np.array_equal(outs[0][1], ref) and np.array_equal(outs[1][1], ref)
    assert np.array_equal(outs[3][1], ref)  # problem-by-problem launches, same numbers
    assert not np.array_equal(outs[2][1], ref)
    scratch = torch.zeros(info["cols"], dtype=torch.float64, device="cuda")
    cfg = B.autotune(d_b.data_ptr(), scratch.data_ptr())
    assert cfg[0] in (4, 8, 16, 32) and cfg[1] in (4, 8, 16, 32) and cfg[2] in (1, 2)
    x = B.sirt("sart", ball, 12, opts=o)
    assert rel_err(x, ref) < 1e-6
    B.close()


def single_code9(fair, A, b, prec, method, K, opts):
    """fair_sirt on the tiled copies (layout code 9 for both passes)."""
    from fortran_airtools_gb300._clib import check, lib
    A.set_precision(prec)
    try:
        check(lib().fair_sirt_set_lanes(A.handle, (C.c_int32 * 4)(8, 8, 9, 9)))
        return fair.airms.sirt(method, A, b, K, opts=opts)
    finally:
        default = (8, 8, 0, 0) if prec == "f64" else (8, 8, 1, 1)
        check(lib().fair_sirt_set_lanes(A.handle, (C.c_int32 * 4)(*default)))
        A.set_precision("f64")


@pytest.mark.parametrize("method", ["sart", "cimmino"])
@pytest.mark.parametrize("prec", ["f64", "f32", "f16", "q16"])
def test_tiled_batch_equals_single(problems, fair, oracle, prec, method):
    """layout 'tiled': every problem on its tiled copies of A and A' (two
    launches per pass for the whole batch); the same numbers as fair_sirt
    on the tiled copies, problem by problem, bit for bit."""
    B = fair.Batch(prec, layout="tiled")
    for A, _, _ in problems:
        B.add(A)
    info = B.info()
    o = fair.airms.options(lbound=0.0, ubound=1.0)
    ball = np.concatenate([b for _, _, b in problems])
    X = B.sirt(method, ball, 20, opts=o)
    _, co = B.offsets()
    tol = {"f64": 1e-10, "f32": 1e-5, "f16": 5e-3, "q16": 1e-4}[prec]
    for p, (A, R, b) in enumerate(problems):
        xs = single_code9(fair, A, b, prec, method, 20, o)
        assert np.array_equal(X[co[p]:co[p + 1]], xs)
        xr = oracle.sirt(method, R, b, 20, opts=oracle.options(lbound=0.0, ubound=1.0))
        assert rel_err(X[co[p]:co[p + 1]], xr) < tol
    from fortran_airtools_gb300._clib import check, lib
    n = C.c_int64()
    check(lib().fair_batch_launches(B.handle, 20, C.byref(n)))
    assert n.value == (0 if prec == "f64" else 1) + 2 * 2 * 20  # partials + row sums per pass
    assert info["device_bytes"] > 0
    B.close()


@pytest.mark.parametrize("prec", ["f64", "f32", "q16"])
def test_auto_layout(problems, fair, oracle, prec):
    """layout 'auto': per class of problems the faster of the packed streams
    and the tiled copies, with the fastest tile shape, timed on the class's
    first problem; a tiled problem equals fair_sirt on its tiled copies with
    the reported shape, bit for bit, and every problem meets its bar against
    the oracle."""
    from fortran_airtools_gb300._clib import check, lib
    B = fair.Batch(prec, layout="auto")
    for A, _, _ in problems:
        B.add(A)
    o = fair.airms.options(lbound=0.0, ubound=1.0)
    ball = np.concatenate([b for _, _, b in problems])
    X = B.sirt("sart", ball, 20, opts=o)
    _, co = B.offsets()
    tol = {"f64": 1e-10, "f32": 1e-5, "q16": 1e-4}[prec]
    for p, (A, R, b) in enumerate(problems):
        lay = B.problem_layout(p)
        if lay["tiled"]:
            assert lay["tile"] in (64, 96, 128) and lay["pixel_tile"] in (16, 32, 48)
            check(lib().fair_sirt_set_tiles(A.handle, (C.c_int32 * 3)(lay["tile"], lay["pixel_tile"],
                                                                       lay["cells"])))
            try:
                xs = single_code9(fair, A, b, prec, "sart", 20, o)
            finally:
                check(lib().fair_sirt_set_tiles(A.handle, (C.c_int32 * 3)(0, 0, 0)))
            assert np.array_equal(X[co[p]:co[p + 1]], xs)
        xr = oracle.sirt("sart", R, b, 20, opts=oracle.options(lbound=0.0, ubound=1.0))
        assert rel_err(X[co[p]:co[p + 1]], xr) < tol
    B.close()


def test_tiled_batch_mixed_and_device_api(problems, fair, oracle):
    """A problem whose columns are not an N x N image keeps the packed layout
    beside the tiled ones (three launches per pass); the device-resident
    graph, its reuse and the problem-by-problem launches give the same numbers."""
    import torch
    rng = np.random.default_rng(5)
    m, n, L = 60, 150, 10  # 150 columns: no square image, no tiled copy
    # banded rows of 10 consecutive columns that cover every column
    starts = np.minimum((np.arange(m) * 2.5).astype(np.int64), n - L)
    IA = np.arange(0, L * (m + 1), L, dtype=np.int64)
    JA = (starts[:, None] + np.arange(L)[None, :]).ravel().astype(np.int32) + 1
    vA = rng.random(IA[-1]) + 0.05
    odd = fair.CSRMatrix.construct(m, n, vA, IA.astype(np.int32), JA)
    Rodd = oracle.OracleCSR(m, n, IA, JA, vA)
    bodd = oracle.matvecmul(Rodd, rng.random(n))
    probs = [(A, R, b) for A, R, b in problems[:3]] + [(odd, Rodd, bodd)] + [problems[3]]
    B = fair.Batch("f32", layout="tiled")
    for A, _, _ in probs:
        B.add(A)
    from fortran_airtools_gb300._clib import check, lib
    cnt = C.c_int64()
    check(lib().fair_batch_launches(B.handle, 10, C.byref(cnt)))
    assert cnt.value == 1 + 2 * 3 * 10
    o = fair.airms.options(lbound=0.0, ubound=1.0)
    ball = np.concatenate([b for _, _, b in probs])
    ref = B.sirt("sart", ball, 10, opts=o)
    _, co = B.offsets()
    for p, (A, R, b) in enumerate(probs):
        xr = oracle.sirt("sart", R, b, 10, opts=oracle.options(lbound=0.0, ubound=1.0))
        assert rel_err(ref[co[p]:co[p + 1]], xr) < 1e-5
    B.prepare("sart", o)
    stream = torch.cuda.Stream()
    B.set_stream(stream.cuda_stream)
    d_b = torch.from_numpy(ball).cuda()
    for batched in (True, True, False):
        d_x = torch.zeros(B.info()["cols"], dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        B.run_device(d_b.data_ptr(), d_x.data_ptr(), 10, batched=batched)
        stream.synchronize()
        assert np.array_equal(d_x.cpu().numpy(), ref)
    B.close()
    odd.close()


def test_take_moves_matrix(fair, oracle):
    A, R = build(fair, oracle, "par", 16, 12, 24)
    B = fair.Batch("f64")
    B.add(A, take=True)
    with pytest.raises(fair.FairError):
        A.matvecmul(np.ones(R.n))
    b = oracle.matvecmul(R, np.linspace(0, 1, R.n))
    x = B.sirt("cimmino", b, 10)
    assert rel_err(x, oracle.sirt("cimmino", R, b, 10)) < 1e-10
    B.close()


def test_batch_errors(fair, oracle):
    from fortran_airtools_gb300._clib import lib
    with pytest.raises(ValueError):
        fair.Batch("f32", layout="rows")
    B = fair.Batch("f32")
    assert lib().fair_batch_set_layout(B.handle, 3) == 4  # FAIR_ERR_ARG
    Bt = fair.Batch("f64")
    At, _ = build(fair, oracle, "par", 16, 12, 24)
    Bt.add(At)
    assert lib().fair_batch_set_layout(Bt.handle, 1) == 9  # FAIR_ERR_STATE: after the first add
    Bt.close()
    At.close()
    with pytest.raises(fair.FairError):
        B.prepare("sart")  # empty batch
    with pytest.raises(fair.FairError):
        B.set_config([6, 8, 1, 1])
    rng = np.random.default_rng(5)
    m, n, per = 300, 5000, 60
    JA = np.concatenate([np.sort(rng.choice(n, per, replace=False)) + 1 for _ in range(m)])
    IA = np.arange(0, per * (m + 1), per, dtype=np.int32)
    A = fair.CSRMatrix.construct(m, n, rng.random(m * per) + 0.1, IA, JA.astype(np.int32))
    with pytest.raises(fair.FairError):
        B.add(A)  # no packed stream for random columns
    with pytest.raises(fair.FairError):
        fair.Batch("f32").prepare("landweber")
    B.close()
    A.close()
