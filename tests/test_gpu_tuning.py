"""Lanes-per-row tuning of the SIRT passes (fair_sirt_set_lanes,
fair_sirt_autotune): every choice -- lanes per row, and 0 (the CSR) or 1-2
groups per lane on the packed stream, in every form including FP64 -- gives
the oracle's iterate within the precision's bar (3, 4: the fused 16-byte
records of the 2-byte forms, the packed stream elsewhere; 5, 6: the linear
walk of the stream), and the autotuner returns one of the supported choices."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def prob(fair, oracle):
    n, nth, p = 40, 50, 58
    th = np.pi * np.arange(nth) / nth
    A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
    R = oracle.paralleltomo(n, nth, p, th)
    b = oracle.matvecmul(R, fair.phantomgallery.shepplogan(n))
    return A, R, b


@pytest.mark.parametrize("prec,tol", [("f64", 1e-10), ("f32", 1e-5), ("f16", 5e-3), ("q16", 1e-4)])
@pytest.mark.parametrize("cfg", [(4, 32, 1, 2), (16, 4, 2, 1), (32, 16, 2, 2), (8, 8, 1, 1),
                                 (8, 4, 0, 2), (8, 8, 0, 0), (8, 4, 3, 4), (16, 32, 4, 3),
                                 (8, 8, 5, 6), (4, 2, 6, 5), (1, 1, 5, 5), (8, 1, 7, 8),
                                 (8, 1, 9, 5), (16, 8, 10, 3), (8, 8, 11, 12), (8, 8, 9, 12), (8, 8, 13, 13), (8, 8, 14, 12)])
def test_lanes_choice(prob, fair, oracle, prec, tol, cfg):
    from fortran_airtools_gb300._clib import check, lib
    A, R, b = prob
    A.set_precision(prec)
    try:
        check(lib().fair_sirt_set_lanes(A.handle, (C.c_int32 * 4)(*cfg)))
        x = fair.airms.sirt("sart", A, b, 20, opts=fair.airms.options(lbound=0.0))
    finally:
        check(lib().fair_sirt_set_lanes(A.handle, (C.c_int32 * 4)(8, 8, 1, 1)))
        A.set_precision("f64")
    xr = oracle.sirt("sart", R, b, 20, opts=oracle.options(lbound=0.0))
    assert rel_err(x, xr) < tol


def test_autotune(prob, fair, oracle):
    import torch
    from fortran_airtools_gb300._clib import check, lib
    A, R, b = prob
    L = lib()
    opts = fair.airms.options()
    A.set_precision("f32")
    try:
        check(L.fair_sirt_prepare(A.handle, b"cimmino", C.byref(opts)))
        d_b = torch.from_numpy(b).cuda()
        d_x = torch.zeros(R.n, dtype=torch.float64, device="cuda")
        cfg = (C.c_int32 * 4)()
        check(L.fair_sirt_autotune(A.handle, d_b.data_ptr(), d_x.data_ptr(), 2, cfg))
        for lanes, code in ((cfg[0], cfg[2]), (cfg[1], cfg[3])):
            assert code in range(15)
            assert lanes in ((0, 1, 2, 4, 8) if 5 <= code <= 8 else (4, 8, 16, 32))
        x = fair.airms.sirt("cimmino", A, b, 15)
    finally:
        A.set_precision("f64")
    assert rel_err(x, oracle.sirt("cimmino", R, b, 15)) < 1e-5
    with pytest.raises(fair.FairError):
        check(L.fair_sirt_set_lanes(A.handle, (C.c_int32 * 4)(6, 8, 1, 1)))
