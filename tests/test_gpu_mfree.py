"""Matrix-free parallel-beam projector pair (include/fair_mf.h).

In FP64 the on-the-fly entries are the segment lengths of the stored
paralleltomo matrix up to rounding, so A x and A' y agree with the oracle's
stored products to 1e-12 relative, including axis-aligned rays on grid lines
(odd p at 0 and pi/2) where the column rule decides ties; SIRT on the pair
matches the oracle's SIRT to 1e-10 (FP64) and 1e-5 (FP32). The projector and
backprojector compute bit-identical entries, so <A x, y> = <x, A' y> up to
the summation order.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

CASES = [  # (N, nth, p, angles)
    (32, 36, 46, "open"),      # theta = pi k/36 + 0.013: no axis-aligned ray
    (24, 6, 23, "axis"),       # theta = 0 with odd p: vertical rays on grid lines (ties)
    (40, 30, 58, "even"),      # theta = pi k/30 with even p: at 0 and pi/2 through pixel centres
    (17, 12, 25, "open"),      # odd N
]


def theta(nth, kind):
    if kind == "axis":
        # sin(0) = 0 exactly; theta = pi/2 is left out: cos(pi/2) = 6e-17 tilts the
        # reference's ray across the grid line it lies on, a tilt below the
        # operator's 2^-40 resolution
        return np.array([0.0, 0.4, np.pi / 4, 1.2, 2.0, 2.8])[:nth]
    th = np.pi * np.arange(nth) / nth
    return th + 0.013 if kind == "open" else th


@pytest.mark.parametrize("case", CASES)
def test_fp64_products_match_stored(fair, oracle, case):
    n, nth, p, kind = case
    th = theta(nth, kind)
    M = fair.MatrixFree(fair.Data(n=n, p=p, nth=nth, theta=th), "f64")
    R = oracle.paralleltomo(n, nth, p, th)
    rng = np.random.default_rng(n)
    x, y = rng.random(R.n), rng.random(R.m)
    assert rel_err(M.project(x), oracle.matvecmul(R, x)) < 1e-12
    assert rel_err(M.backproject(y), oracle.transvecmul(R, y)) < 1e-12
    # the stored matrix's row sums (all entries, nothing dropped or added)
    assert rel_err(M.project(np.ones(R.n)), oracle.matvecmul(R, np.ones(R.n))) < 1e-12
    assert M.nnz() == R.nnz
    M.close()


@pytest.mark.parametrize("prec,tol", [("f64", 1e-13), ("f32", 2e-6)])
def test_adjoint_identity(fair, prec, tol):
    n, nth, p = 48, 60, 70
    M = fair.MatrixFree(fair.Data(n=n, p=p, nth=nth, theta=theta(nth, "open")), prec)
    rng = np.random.default_rng(1)
    for _ in range(3):
        x, y = rng.random(M.n), rng.random(M.m)
        lhs, rhs = M.project(x) @ y, x @ M.backproject(y)
        assert abs(lhs - rhs) <= tol * abs(lhs)
    M.close()


@pytest.mark.parametrize("method", ["sart", "cimmino"])
@pytest.mark.parametrize("prec,tol", [("f64", 1e-10), ("f32", 1e-5)])
def test_sirt_matches_oracle(fair, oracle, method, prec, tol):
    n, nth, p = 32, 40, 46
    th = theta(nth, "open")
    M = fair.MatrixFree(fair.Data(n=n, p=p, nth=nth, theta=th), prec)
    R = oracle.paralleltomo(n, nth, p, th)
    b = oracle.matvecmul(R, fair.phantomgallery.shepplogan(n))
    o = fair.airms.options(lbound=0.0, ubound=1.0)
    x = M.sirt(method, b, 30, opts=o)
    xr = oracle.sirt(method, R, b, 30, opts=oracle.options(lbound=0.0, ubound=1.0))
    assert rel_err(x, xr) < tol
    M.close()


def test_device_api(fair):
    import torch
    n, nth, p = 40, 36, 58
    M = fair.MatrixFree(fair.Data(n=n, p=p, nth=nth, theta=theta(nth, "open")), "f32")
    b = M.project(fair.phantomgallery.shepplogan(n))
    o = fair.airms.options(lbound=0.0)
    ref = M.sirt("sart", b, 10, opts=o)
    M.prepare("sart", o)
    stream = torch.cuda.Stream()
    M.set_stream(stream.cuda_stream)
    d_b = torch.from_numpy(b).cuda()
    d_x = torch.zeros(M.n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    M.run_device(d_b.data_ptr(), d_x.data_ptr(), 10)
    stream.synchronize()
    assert np.array_equal(d_x.cpu().numpy(), ref)
    d_x.zero_()
    torch.cuda.synchronize()
    t1, t2 = M.run_device_timed(d_b.data_ptr(), d_x.data_ptr(), 10)
    assert t1 > 0 and t2 > 0
    assert np.array_equal(d_x.cpu().numpy(), ref)
    M.close()


def test_errors(fair):
    th = np.zeros(4)
    with pytest.raises(fair.FairError):
        fair.MatrixFree(fair.Data(n=8, p=1, nth=4, theta=th), "f32")
    with pytest.raises(fair.FairError):
        fair.MatrixFree(fair.Data(n=8, p=10, nth=4, theta=th), "f16")
    M = fair.MatrixFree(fair.Data(n=8, p=10, nth=4, theta=th), "f32")
    with pytest.raises(fair.FairError):
        M.prepare("landweber")
    M.close()


@pytest.mark.parametrize("n,p", [(16, 23), (16, 24), (17, 25)])
def test_axis_aligned_fp32_matches_fp64(fair, n, p):
    """Rays at theta = 0, pi/2, pi, 3pi/2 are axis-aligned (their fixed-point
    normal has a zero component): a ray on a grid line keeps the pixels on one
    side, decided on the exact distance in both precisions, so the FP32
    entries are the FP64 ones up to FP32 rounding (no pixel counted twice or
    dropped) and the FP32 pair stays adjoint."""
    th = np.array([0.0, np.pi / 2, np.pi, 1.5 * np.pi, np.pi / 4, 2.0])
    d = fair.Data(n=n, p=p, nth=len(th), theta=th)
    M64, M32 = fair.MatrixFree(d, "f64"), fair.MatrixFree(d, "f32")
    rng = np.random.default_rng(n + p)
    x, y = rng.random(n * n), rng.random(M64.m)
    for v in (np.ones(n * n), x):
        assert rel_err(M32.project(v), M64.project(v)) < 1e-6
    for w in (np.ones(M64.m), y):
        assert rel_err(M32.backproject(w), M64.backproject(w)) < 1e-6
    lhs, rhs = M32.project(x) @ y, x @ M32.backproject(y)
    assert abs(lhs - rhs) <= 2e-6 * abs(lhs)
    M64.close()
    M32.close()
