"""Packed index stream of the reduced-precision SIRT passes (rows padded to
groups of 4 entries, one anchor column and three step codes per group).

The packed and unpacked layouts hold the same values, so their iterates may
differ only by the FP32 summation order (bar: 2e-6 relative after 30
iterations); groups whose steps have no code go through the escape table;
a matrix on which most groups would escape is left unpacked.
"""
import os

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def sirt_prec(fair, A, b, prec, method, K, packed, opts):
    os.environ["FAIR_PACKED"] = "1" if packed else "0"
    try:
        A.set_precision(prec)
        return fair.airms.sirt(method, A, b, K, opts=opts)
    finally:
        A.set_precision("f64")
        os.environ.pop("FAIR_PACKED", None)


@pytest.fixture(scope="module")
def par48(fair, oracle):
    n, nth, p = 48, 60, 68
    th = np.pi * np.arange(nth) / nth
    A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
    R = oracle.paralleltomo(n, nth, p, th)
    b = oracle.matvecmul(R, fair.phantomgallery.shepplogan(n))
    return A, R, b


@pytest.fixture(scope="module")
def fan40(fair, oracle):
    n, nth, p = 40, 72, 57
    th = 2 * np.pi * np.arange(nth) / nth
    A = fair.fanlineartomo(fair.Data(n=n, p=p, nth=nth, r=2.0, dw=p / n, sd=2.0, theta=th))
    R = oracle.fanlineartomo(n, nth, p, 2.0, p / n, 2.0, th)
    b = oracle.matvecmul(R, fair.phantomgallery.shepplogan(n))
    return A, R, b


@pytest.mark.parametrize("prec", ["f32", "f16", "q16"])
@pytest.mark.parametrize("method", ["cimmino", "sart"])
@pytest.mark.parametrize("case", ["par48", "fan40"])
def test_packed_equals_unpacked(request, fair, oracle, case, method, prec):
    A, R, b = request.getfixturevalue(case)
    o = fair.airms.options(lbound=0.0, ubound=1.0)
    xp = sirt_prec(fair, A, b, prec, method, 30, True, o)
    xu = sirt_prec(fair, A, b, prec, method, 30, False, o)
    assert rel_err(xp, xu) < 2e-6
    xr = oracle.sirt(method, R, b, 30, opts=oracle.options(lbound=0.0, ubound=1.0))
    tol = {"f32": 1e-5, "f16": 5e-3, "q16": 1e-4}[prec]
    assert rel_err(xp, xr) < tol
    # a ray moves to a 4- or 8-neighbour pixel: every step of A has a code;
    # in A' a pixel that leaves the fan for some angles jumps over them (the
    # odd-p fan case escapes about 3% of its groups)
    assert A.packed_info()["has"] and A.packed_info()["nesc"] == 0
    info = A.packed_info(transposed=True)
    assert info["has"] and info["nesc"] <= info["ngroups"] // 20
    # stride of a step across the image: N for A, the bins per angle for A'
    assert A.packed_info()["stride"] == int(round(np.sqrt(R.n)))
    assert A.packed_info(transposed=True)["stride"] == {"par48": 68, "fan40": 57}[case]


def test_packed_escape_table(par48, fair, oracle):
    """Rows whose entries are shuffled have steps with no code: their groups
    are stored in the escape table; the iterates do not change."""
    A0, R, b = par48
    vA, IA, JA = A0.arrays()
    vA, JA = vA.copy(), JA.copy()
    rng = np.random.default_rng(11)
    rows = rng.choice(R.m, size=R.m // 40, replace=False)
    for r in rows:
        s, e = IA[r], IA[r + 1]
        perm = rng.permutation(e - s)
        vA[s:e], JA[s:e] = vA[s:e][perm], JA[s:e][perm]
    A = fair.CSRMatrix.construct(R.m, R.n, vA, IA, JA)
    o = fair.airms.options(lbound=0.0)
    xp = sirt_prec(fair, A, b, "q16", "cimmino", 25, True, o)
    info = A.packed_info()
    assert info["has"] and info["nesc"] > 0
    xu = sirt_prec(fair, A, b, "q16", "cimmino", 25, False, o)
    assert rel_err(xp, xu) < 2e-6
    xr = oracle.sirt("cimmino", R, b, 25, opts=oracle.options(lbound=0.0))
    assert rel_err(xp, xr) < 1e-4
    A.close()


def test_packed_refused_for_random_columns(fair, oracle):
    """Random column indices: nearly every group would escape, so the matrix
    stays unpacked and the reduced form runs on the unpacked layout."""
    rng = np.random.default_rng(5)
    m, n, per = 600, 5000, 60  # n not a square: the only code is a plain 7-bit delta
    JA = np.concatenate([np.sort(rng.choice(n, per, replace=False)) + 1 for _ in range(m)])
    IA = np.arange(0, per * (m + 1), per, dtype=np.int32)
    vA = rng.random(m * per) + 0.1
    A = fair.CSRMatrix.construct(m, n, vA, IA, JA.astype(np.int32))
    R = oracle.OracleCSR(m, n, IA.astype(np.int64), JA.astype(np.int32), vA)
    b = oracle.matvecmul(R, rng.random(n))
    x = sirt_prec(fair, A, b, "f32", "cimmino", 20, True, fair.airms.options())
    assert not A.packed_info()["has"]
    xr = oracle.sirt("cimmino", R, b, 20)
    assert rel_err(x, xr) < 1e-5
    A.close()
