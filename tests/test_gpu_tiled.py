"""The tiled copies (layout codes 9, 10; 14: the 2-byte forms' 6-entry
records of tile-local index steps). Pass 1 reads A cut by 96 x 96 tiles of the
N x N image (each tile of x staged in shared memory); pass 2 reads A' cut by
32 x 32 pixel tiles times blocks of angles (each tile's window of residual
bins staged in shared memory); one partial sum per segment, the partials of a
row added in row order by a second kernel. The copy holds the same values as the
CSR layout, so the iterates differ only by summation order: FP64 within
1e-12 of the CSR iterate (and 1e-10 of the oracle), the FP32-accumulating
forms within 2e-6. Images of 3 x 3 tiles with partial edge tiles, a single
partial tile, a square matrix whose rows jump between tiles (its step
records and the delta copy of its transpose are refused: too many steps
outside the codes), and a matrix whose columns are not a square image (no
tiled copy: the pass falls back to the row layouts). Many angles (720) make
every tile hold thousands of chunks, so each warp streams several chunks per
work unit and the tiles' shortest segments form chunks of a single slot,
which the stream's lookahead must cross (a missed slot drops entries)."""
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


@pytest.fixture(scope="module")
def par260(fair, oracle):
    n, nth, p = 260, 40, 368
    th = np.pi * np.arange(nth) / nth
    A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
    R = oracle.paralleltomo(n, nth, p, th)
    b = oracle.matvecmul(R, fair.phantomgallery.shepplogan(n))
    return A, R, b


@pytest.fixture(scope="module")
def fan90(fair, oracle):
    n, nth, p = 90, 60, 127
    th = 2 * np.pi * np.arange(nth) / nth
    A = fair.fanlineartomo(fair.Data(n=n, p=p, nth=nth, r=2.0, dw=p / n, sd=2.0, theta=th))
    R = oracle.fanlineartomo(n, nth, p, 2.0, p / n, 2.0, th)
    b = oracle.matvecmul(R, fair.phantomgallery.shepplogan(n))
    return A, R, b


@pytest.fixture(scope="module")
def jumpy(fair, oracle):
    """Rows with sorted random columns of a 300 x 300 image: every row visits
    many tiles, several times over (one segment per run of entries in a tile)."""
    rng = np.random.default_rng(31)
    m, n = 700, 300 * 300
    lens = rng.integers(0, 400, m)
    lens[::50] = 0
    IA = np.zeros(m + 1, dtype=np.int64)
    IA[1:] = np.cumsum(lens)
    JA = np.concatenate([np.sort(rng.choice(n, L, replace=False)) + 1 for L in lens]).astype(np.int32)
    vA = rng.random(IA[-1]) + 0.05
    A = fair.CSRMatrix.construct(m, n, vA, IA.astype(np.int32), JA)
    R = oracle.OracleCSR(m, n, IA, JA, vA)
    b = oracle.matvecmul(R, rng.random(n))
    yield A, R, b
    A.close()


@pytest.mark.parametrize("prec", ["f64", "f32", "f16", "q16"])
@pytest.mark.parametrize("codes", [(9, 0), (10, 0), (14, 0), (0, 9), (9, 10), (14, 14)])
@pytest.mark.parametrize("case", ["par260", "fan90"])
def test_tiled_geometry(request, fair, oracle, case, prec, codes):
    A, R, b = request.getfixturevalue(case)
    o = fair.airms.options(lbound=0.0, ubound=1.0)
    xt = run(fair, A, b, prec, (8, 8) + codes, "sart", 15, o)
    xc = run(fair, A, b, prec, (8, 8, 0, 0), "sart", 15, o)
    assert rel_err(xt, xc) < TOL_SAME[prec]
    xr = oracle.sirt("sart", R, b, 15, opts=oracle.options(lbound=0.0, ubound=1.0))
    assert rel_err(xt, xr) < TOL_ORACLE[prec]


@pytest.mark.parametrize("prec", ["f64", "q16"])
@pytest.mark.parametrize("code", [10, 14])
def test_tiled_jumpy_rows(jumpy, fair, oracle, prec, code):
    A, R, b = jumpy
    o = fair.airms.options(lbound=0.0)
    xt = run(fair, A, b, prec, (8, 8, code, 12), "cimmino", 10, o)
    xc = run(fair, A, b, prec, (8, 8, 0, 0), "cimmino", 10, o)
    assert np.all(np.isfinite(xt))
    assert rel_err(xt, xc) < TOL_SAME[prec]
    xr = oracle.sirt("cimmino", R, b, 10, opts=oracle.options(lbound=0.0))
    assert rel_err(xt, xr) < TOL_ORACLE[prec]


def test_tiled_needs_a_square_image(fair, oracle):
    """n = 3001 columns: no tiled copy; code 9 runs on the row layouts."""
    rng = np.random.default_rng(8)
    m, n, per = 300, 3001, 40
    JA = np.concatenate([np.sort(rng.choice(n, per, replace=False)) + 1 for _ in range(m)])
    IA = np.arange(0, per * (m + 1), per, dtype=np.int32)
    vA = rng.random(m * per) + 0.1
    A = fair.CSRMatrix.construct(m, n, vA, IA, JA.astype(np.int32))
    R = oracle.OracleCSR(m, n, IA.astype(np.int64), JA.astype(np.int32), vA)
    b = oracle.matvecmul(R, rng.random(n))
    x = run(fair, A, b, "f32", (8, 8, 9, 1), "cimmino", 10, fair.airms.options())
    assert rel_err(x, oracle.sirt("cimmino", R, b, 10)) < 1e-5
    A.close()


@pytest.fixture(scope="module")
def par200(fair, oracle):
    n, nth, p = 200, 720, 284
    th = np.pi * np.arange(nth) / nth
    A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
    R = oracle.paralleltomo_mt(n, nth, p, th, 8)
    b = oracle.matvecmul(R, fair.phantomgallery.gaussians(n, 20, seed=1))
    yield A, R, b
    A.close()


@pytest.mark.parametrize("prec,codes", [("f64", (9, 0)), ("f64", (9, 9)), ("f32", (9, 14)),
                                        ("q16", (14, 14)), ("f16", (14, 0))])
def test_tiled_many_chunks_per_unit(par200, fair, oracle, prec, codes):
    A, R, b = par200
    xt = run(fair, A, b, prec, (8, 8) + codes, "cimmino", 5, fair.airms.options())
    xc = run(fair, A, b, prec, (8, 8, 0, 0), "cimmino", 5, fair.airms.options())
    assert rel_err(xt, xc) < TOL_SAME[prec]
    assert rel_err(xt, oracle.sirt("cimmino", R, b, 5, nthreads=8)) < (1e-10 if prec == "f64" else 1e-5)


@pytest.mark.parametrize("shape", [(64, 16, 6500), (128, 48, 13000), (40, 8, 2048)])
def test_tile_shapes(par200, fair, oracle, shape):
    """fair_sirt_set_tiles: other tile sides for A, pixel-tile sides and residual
    cells for A' (more angle blocks): the same iterates as the CSR layout."""
    from fortran_airtools_gb300._clib import check, lib
    A, R, b = par200
    L = lib()
    check(L.fair_sirt_set_tiles(A.handle, (C.c_int32 * 3)(*shape)))
    try:
        for prec, codes in (("f64", (9, 10)), ("q16", (14, 14))):
            A.set_precision(prec)
            check(L.fair_sirt_set_lanes(A.handle, (C.c_int32 * 4)(8, 8, *codes)))
            xt = fair.airms.sirt("cimmino", A, b, 5)
            ia, iat = A.tiled_info(), A.tiled_info(transposed=True)
            assert ia["has"] and ia["tile"] == shape[0]
            assert iat["has"] and iat["tile"] == shape[1]
            assert iat["angles_per_block"] * iat["window"] <= shape[2]
            check(L.fair_sirt_set_lanes(A.handle, (C.c_int32 * 4)(8, 8, 0, 0)))
            xc = fair.airms.sirt("cimmino", A, b, 5)
            assert rel_err(xt, xc) < TOL_SAME[prec]
    finally:
        check(L.fair_sirt_set_tiles(A.handle, (C.c_int32 * 3)(0, 0, 0)))
        check(L.fair_sirt_set_lanes(A.handle, (C.c_int32 * 4)(8, 8, 1, 1)))
        A.set_precision("f64")
        check(L.fair_sirt_set_lanes(A.handle, (C.c_int32 * 4)(8, 8, 0, 0)))
    with pytest.raises(fair.FairError):
        check(L.fair_sirt_set_tiles(A.handle, (C.c_int32 * 3)(200, 0, 0)))
