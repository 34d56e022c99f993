"""paralleltomo held in FP32 only (fair_paralleltomo_f32).

The matrix is traced by blocks of angles in FP64 and kept as FP32 values with
int32 columns and int64 row offsets; A' is assembled block by block. With the
same values and the same entry order as the FP64 handle's FP32 copy, the
results must equal that handle's in FP32 bit for bit: the structure, both
products, the row norms, and Cimmino SIRT on the CSR and tiled layouts
(its weights are the row norms). SART's column sums are added block by
block in FP64 (a different order), so SART agrees within FP32 rounding and
with the oracle within the FP32 bar. At N=2048 with 1440 angles and 2896 bins
(7.69e9 nonzeros: 64-bit row offsets past 2^31) the products and two
iterations agree with the matrix-free FP32 operator of the same geometry.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def structure(fair, A):
    from fortran_airtools_gb300._clib import check, lib, ptr
    m, n, nnz = A.info()
    IA = np.empty(m + 1, np.int64)
    JA = np.empty(nnz, np.int32)
    check(lib().fair_csr_download(A.handle, None, ptr(IA), ptr(JA)))
    return IA, JA


def set_layout(A, cfg):
    from fortran_airtools_gb300._clib import check, lib
    check(lib().fair_sirt_set_lanes(A.handle, (C.c_int32 * 4)(*cfg)))


@pytest.fixture(scope="module")
def pair(fair, oracle):
    n, nth, p = 64, 90, 90
    th = np.pi * np.arange(nth) / nth
    d = fair.Data(n=n, p=p, nth=nth, theta=th)
    A = fair.paralleltomo(d)
    A.set_precision("f32")
    H = fair.paralleltomo_f32(d, block_angles=7)
    R = oracle.paralleltomo(n, nth, p, th)
    b = oracle.matvecmul(R, fair.phantomgallery.shepplogan(n))
    yield A, H, R, b
    A.close()
    H.close()


def test_structure_and_products_equal(pair, fair):
    A, H, R, _ = pair
    assert H.info() == A.info()
    IA, JA = structure(fair, H)
    assert np.array_equal(IA, R.IA) and np.array_equal(JA, R.JA)
    rng = np.random.default_rng(1)
    x, y = rng.standard_normal(R.n), rng.standard_normal(R.m)
    assert np.array_equal(H.matvecmul(x), A.matvecmul(x))
    assert np.array_equal(H.transvecmul(y), A.transvecmul(y))
    for p in (1, 2):
        assert np.array_equal(H.row_norms(p), A.row_norms(p))
        assert rel_err(H.column_norms(p), A.column_norms(p)) < 1e-14


@pytest.mark.parametrize("cfg", [(8, 8, 0, 0), (8, 8, 9, 9), (8, 8, 1, 1), (8, 8, 9, 12), (8, 1, 10, 5)])
def test_cimmino_equals_fp64_handle_in_fp32(pair, fair, oracle, cfg):
    A, H, R, b = pair
    try:
        set_layout(A, cfg)
        set_layout(H, cfg)
        xa = fair.airms.sirt("cimmino", A, b, 10)
        xh = fair.airms.sirt("cimmino", H, b, 10)
    finally:
        set_layout(A, (8, 8, 1, 1))
        set_layout(H, (8, 8, 1, 1))
    assert np.array_equal(xh, xa)
    assert rel_err(xh, oracle.sirt("cimmino", R, b, 10)) < 1e-5


def test_sart_and_blocks(pair, fair, oracle):
    A, H, R, b = pair
    o = fair.airms.options(lbound=0.0, ubound=1.0)
    xa = fair.airms.sirt("sart", A, b, 10, opts=o)
    xh = fair.airms.sirt("sart", H, b, 10, opts=o)
    assert rel_err(xh, xa) < 1e-6
    assert rel_err(xh, oracle.sirt("sart", R, b, 10, opts=oracle.options(lbound=0.0, ubound=1.0))) < 1e-5
    th = np.pi * np.arange(90) / 90
    H1 = fair.paralleltomo_f32(fair.Data(n=64, p=90, nth=90, theta=th))  # blocks chosen by size
    y = np.random.default_rng(2).standard_normal(R.m)
    assert np.array_equal(H1.transvecmul(y), H.transvecmul(y))
    H1.close()


def test_fp64_entry_points_refuse(pair, fair):
    _, H, R, b = pair
    with pytest.raises(fair.FairError) as e:
        H.set_precision("f64")
    assert e.value.status == 9
    with pytest.raises(fair.FairError):
        H.arrays()  # vA has no FP64 copy
    with pytest.raises(fair.FairError):
        fair.airms.art("kaczmarz", H, b, [1])
    with pytest.raises(fair.FairError):
        fair.airms.normest(H)
    with pytest.raises(fair.FairError):
        H.rowvecmult(1, np.ones(R.n))
    with pytest.raises(fair.FairError):
        fair.Batch("f32").add(H)
    with pytest.raises(fair.FairError):
        fair.paralleltomo_f32(fair.Data(n=8, p=9, nth=3, theta=np.linspace(0.0, np.pi, 3)))


@pytest.mark.slow
def test_n2048_against_matrix_free(fair):
    """7.69e9 nonzeros: 64-bit row offsets past 2^31; FP32 products and two
    Cimmino iterations against the matrix-free FP32 pair of the same rays."""
    n, nth, p = 2048, 1440, 2896
    th = np.pi * np.arange(nth) / nth
    d = fair.Data(n=n, p=p, nth=nth, theta=th)
    H = fair.paralleltomo_f32(d)
    m, ncols, nnz = H.info()
    assert nnz > 2 ** 31
    M = fair.MatrixFree(d, "f32")
    assert M.nnz() == nnz
    x = fair.phantomgallery.gaussians(n, 20, seed=1)
    yh, ym = H.matvecmul(x), M.project(x)
    assert rel_err(yh, ym) < 1e-5
    assert rel_err(H.transvecmul(yh), M.backproject(yh)) < 1e-5
    xs = fair.airms.sirt("cimmino", H, ym, 2)
    xm = M.sirt("cimmino", ym, 2)
    assert rel_err(xs, xm) < 1e-5
    M.close()
    H.close()
