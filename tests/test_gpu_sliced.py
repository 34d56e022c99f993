"""The sliced copy of the packed stream (layout codes 5-8): slices of
32/G rows with G = 1, 2, 4 or 8 lanes per row (G = 0: chosen per chunk of 32
rows), the groups of a slice interleaved by step, 2 or 4 steps of 32 slots in
flight per warp (codes 7, 8: with the gathers of x one step ahead). It holds
the same values as the CSR layout, so the two iterates differ only by
summation order: FP64 within 1e-12 of each other (and 1e-10 of the oracle),
the FP32-accumulating forms within 2e-6 of each other. The ragged matrix
mixes, inside one slice, empty rows, rows of 1-5 entries and rows spanning
hundreds of groups, and has chunks whose rows are all empty; padding slots
(holes) must add nothing."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL_SAME = {"f64": 1e-12, "f32": 2e-6, "f16": 2e-6, "q16": 2e-6}
TOL_ORACLE = {"f64": 1e-10, "f32": 1e-5, "f16": 5e-3, "q16": 1e-4}


def run(fair, A, b, prec, cfg, method, K, opts):
    from fortran_airtools_gb300._clib import check, lib
    A.set_precision(prec)
    try:
        check(lib().fair_sirt_set_lanes(A.handle, (C.c_int32 * 4)(*cfg)))
        return fair.airms.sirt(method, A, b, K, opts=opts)
    finally:
        default = (8, 8, 0, 0) if prec == "f64" else (8, 8, 1, 1)
        check(lib().fair_sirt_set_lanes(A.handle, (C.c_int32 * 4)(*default)))
        A.set_precision("f64")


def ragged_lengths(m):
    pattern = [0, 1, 2, 3, 4, 5, 7, 8, 124, 128, 129, 0, 0, 512, 513, 1000, 2000, 31, 32, 33,
               0, 127, 4, 4, 4, 60, 61, 62, 63, 64, 65, 256, 0, 1, 1, 1]
    lens = [pattern[i % len(pattern)] for i in range(m)]
    lens[64:128] = [0] * 64  # two chunks of empty rows
    return np.array(lens, dtype=np.int64)


@pytest.fixture(scope="module")
def ragged(fair, oracle):
    rng = np.random.default_rng(21)
    m, n = 900, 3001
    lens = ragged_lengths(m)
    IA = np.zeros(m + 1, dtype=np.int64)
    IA[1:] = np.cumsum(lens)
    JA = np.empty(IA[-1], dtype=np.int32)
    for i in range(m):
        c0 = (4 * i) % (n - lens[i] + 1)
        JA[IA[i]:IA[i + 1]] = np.arange(c0, c0 + lens[i]) + 1  # 1-based, consecutive columns
    vA = rng.random(IA[-1]) + 0.05
    A = fair.CSRMatrix.construct(m, n, vA, IA.astype(np.int32), JA)
    R = oracle.OracleCSR(m, n, IA, JA, vA)
    b = oracle.matvecmul(R, rng.random(n))
    yield A, R, b
    A.close()


@pytest.mark.parametrize("prec", ["f64", "f32", "f16", "q16"])
@pytest.mark.parametrize("code", [5, 6, 7, 8])
@pytest.mark.parametrize("G", [0, 1, 2, 4, 8])
def test_sliced_ragged_rows(ragged, fair, oracle, prec, code, G):
    A, R, b = ragged
    o = fair.airms.options(lbound=0.0)
    xs = run(fair, A, b, prec, (G, G, code, code), "cimmino", 15, o)
    assert A.packed_info()["has"] and A.packed_info()["sliced"]
    xc = run(fair, A, b, prec, (8, 8, 0, 0), "cimmino", 15, o)
    assert np.all(np.isfinite(xs))
    assert rel_err(xs, xc) < TOL_SAME[prec]
    xr = oracle.sirt("cimmino", R, b, 15, opts=oracle.options(lbound=0.0))
    assert rel_err(xs, xr) < TOL_ORACLE[prec]


@pytest.fixture(scope="module")
def par96(fair, oracle):
    n, nth, p = 96, 90, 136
    th = np.pi * np.arange(nth) / nth
    A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
    R = oracle.paralleltomo(n, nth, p, th)
    b = oracle.matvecmul(R, fair.phantomgallery.shepplogan(n))
    return A, R, b


@pytest.fixture(scope="module")
def fan64(fair, oracle):
    n, nth, p = 64, 120, 91
    th = 2 * np.pi * np.arange(nth) / nth
    A = fair.fanlineartomo(fair.Data(n=n, p=p, nth=nth, r=2.0, dw=p / n, sd=2.0, theta=th))
    R = oracle.fanlineartomo(n, nth, p, 2.0, p / n, 2.0, th)
    b = oracle.matvecmul(R, fair.phantomgallery.shepplogan(n))
    return A, R, b


@pytest.mark.parametrize("prec", ["f64", "f32", "f16", "q16"])
@pytest.mark.parametrize("cfg", [(1, 8, 5, 6), (8, 1, 6, 5), (2, 4, 6, 6), (4, 2, 5, 5), (0, 0, 6, 6),
                                 (8, 1, 7, 8), (1, 0, 8, 7), (8, 8, 11, 12), (8, 8, 12, 11)])
@pytest.mark.parametrize("case", ["par96", "fan64"])
def test_sliced_geometry(request, fair, oracle, case, prec, cfg):
    A, R, b = request.getfixturevalue(case)
    o = fair.airms.options(lbound=0.0, ubound=1.0)
    xs = run(fair, A, b, prec, cfg, "sart", 20, o)
    xc = run(fair, A, b, prec, (8, 8, 0, 0), "sart", 20, o)
    assert rel_err(xs, xc) < TOL_SAME[prec]
    xr = oracle.sirt("sart", R, b, 20, opts=oracle.options(lbound=0.0, ubound=1.0))
    assert rel_err(xs, xr) < TOL_ORACLE[prec]


def test_sliced_lanes_checked(par96, fair):
    """Codes 5-8 take 0 (per chunk), 1, 2, 4 or 8 lanes per row; codes 0-4
    and 9-14 take 4-32; codes past 14 are refused."""
    from fortran_airtools_gb300._clib import check, lib
    A = par96[0]
    for bad in [(16, 8, 5, 1), (8, 2, 1, 0), (8, 8, 15, 1), (3, 8, 6, 1), (1, 8, 9, 1), (8, 2, 11, 0)]:
        with pytest.raises(fair.FairError):
            check(lib().fair_sirt_set_lanes(A.handle, (C.c_int32 * 4)(*bad)))
    check(lib().fair_sirt_set_lanes(A.handle, (C.c_int32 * 4)(1, 32, 5, 0)))
    check(lib().fair_sirt_set_lanes(A.handle, (C.c_int32 * 4)(8, 8, 0, 0)))


@pytest.mark.parametrize("prec", ["f64", "f32", "f16", "q16"])
@pytest.mark.parametrize("code", [11, 12, 13])
def test_delta_ragged_rows(ragged, fair, oracle, prec, code):
    """The delta copy (codes 11, 12: one lane per row, 7-bit column steps from
    the row's previous entry) on rows of every length, empty rows included."""
    A, R, b = ragged
    o = fair.airms.options(lbound=0.0)
    xs = run(fair, A, b, prec, (8, 8, code, code), "cimmino", 15, o)
    xc = run(fair, A, b, prec, (8, 8, 0, 0), "cimmino", 15, o)
    assert np.all(np.isfinite(xs))
    assert rel_err(xs, xc) < TOL_SAME[prec]
    xr = oracle.sirt("cimmino", R, b, 15, opts=oracle.options(lbound=0.0))
    assert rel_err(xs, xr) < TOL_ORACLE[prec]


@pytest.mark.parametrize("prec", ["f64", "q16"])
def test_delta_side_table(par96, fair, oracle, prec):
    """Rows whose entries are shuffled have steps outside the 7-bit codes:
    their groups go to the side table; the iterate does not change."""
    A0, R, b = par96
    vA, IA, JA = A0.arrays()
    vA, JA = vA.copy(), JA.copy()
    rng = np.random.default_rng(12)
    for r in rng.choice(R.m, size=R.m // 40, replace=False):
        s, e = IA[r], IA[r + 1]
        perm = rng.permutation(e - s)
        vA[s:e], JA[s:e] = vA[s:e][perm], JA[s:e][perm]
    A = fair.CSRMatrix.construct(R.m, R.n, vA, IA, JA)
    Rs = oracle.OracleCSR(R.m, R.n, IA.astype(np.int64), JA.astype(np.int32), vA)
    o = fair.airms.options(lbound=0.0)
    xs = run(fair, A, b, prec, (8, 8, 12, 11), "cimmino", 12, o)
    xc = run(fair, A, b, prec, (8, 8, 0, 0), "cimmino", 12, o)
    assert rel_err(xs, xc) < TOL_SAME[prec]
    xr = oracle.sirt("cimmino", Rs, b, 12, opts=oracle.options(lbound=0.0))
    assert rel_err(xs, xr) < TOL_ORACLE[prec]
    A.close()
