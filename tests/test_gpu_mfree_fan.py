"""Matrix-free fan-beam projector pair (fair_mf_create_fan, include/fair_mf.h).

Each ray of fanlineartomo (system_generation.f90:79-307) is the line from the
rotated source in the direction the reference computes; its entries are the
chords of the pixels it crosses, from the exact fixed-point distance. In FP64
A x and A' y agree with the oracle's stored fan matrix to 1e-12 relative (the
segment lengths up to rounding), the nonzero counts are equal, the projector
and backprojector are adjoint, and SIRT on the pair matches the oracle's SIRT
to 1e-10 (FP64) and 1e-5 (FP32). Known difference: with odd p the central
ray at theta = pi/2, pi, 3pi/2 lies on a grid line in exact arithmetic, and
the reference's rounding residue of cos/sin tilts it across that line (half
its pixels on each side); here it stays on one side.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

CASES = [  # (N, nth, p, theta, geometry_fix)
    (32, 36, 46, "open", 0),   # theta = 2 pi k/36 + 0.013, even p
    (24, 7, 35, "seven", 0),   # theta = 2 pi k/7: only theta = 0 is axis-aligned (odd p:
                               # the central ray on the grid line x = 0, a tie)
    (40, 30, 58, "plain", 0),  # theta = 2 pi k/30 (0, pi/2, pi, 3pi/2 included), even p
    (17, 12, 25, "open", 0),   # odd N, odd p (the reference's odd-p bin angles of :122)
    (26, 16, 37, "open", 1),   # odd p with the corrected angles
]


def theta(nth, kind):
    th = 2 * np.pi * np.arange(nth) / nth
    return th + 0.013 if kind == "open" else th


def fan(fair, oracle, n, nth, p, th, fix, prec="f64"):
    d = fair.Data(n=n, p=p, nth=nth, r=2.0, dw=p / n, sd=2.0, theta=th)
    M = fair.MatrixFree(d, prec, beam="fan", geometry_fix=fix)
    R = oracle.fanlineartomo(n, nth, p, 2.0, p / n, 2.0, th, geometry_fix=bool(fix))
    return M, R


@pytest.mark.parametrize("case", CASES)
def test_fp64_products_match_stored_fan(fair, oracle, case):
    n, nth, p, kind, fix = case
    M, R = fan(fair, oracle, n, nth, p, theta(nth, kind), fix)
    rng = np.random.default_rng(n)
    x, y = rng.random(R.n), rng.random(R.m)
    assert rel_err(M.project(x), oracle.matvecmul(R, x)) < 1e-12
    assert rel_err(M.backproject(y), oracle.transvecmul(R, y)) < 1e-12
    # every stored entry, nothing dropped or added
    assert rel_err(M.project(np.ones(R.n)), oracle.matvecmul(R, np.ones(R.n))) < 1e-12
    assert rel_err(M.backproject(np.ones(R.m)), oracle.transvecmul(R, np.ones(R.m))) < 1e-12
    assert M.nnz() == R.nnz
    M.close()


def test_fan_config1_geometry(fair, oracle):
    """Fan N=128, 360 angles, 181 bins: every ray agrees with the stored matrix
    but the odd-p central ray at theta = pi/2, pi and 3pi/2, which the
    reference's rounding tilts across the grid line it lies on."""
    n, nth, p = 128, 360, 181
    th = theta(nth, "plain")
    M, R = fan(fair, oracle, n, nth, p, th, 0)
    x = np.random.default_rng(5).random(R.n)
    y, yr = M.project(x), oracle.matvecmul(R, x)
    tilted = [i * p + (p - 1) // 2 for i in (90, 180, 270)]
    keep = np.ones(R.m, bool)
    keep[tilted] = False
    assert rel_err(y[keep], yr[keep]) < 1e-12
    # the tilted rays: the same total length, on one side of the grid line here
    ones = np.ones(R.n)
    assert rel_err(M.project(ones)[tilted], oracle.matvecmul(R, ones)[tilted]) < 1e-12
    M.close()


@pytest.mark.parametrize("prec,tol", [("f64", 1e-13), ("f32", 2e-6)])
def test_fan_adjoint_identity(fair, oracle, prec, tol):
    M, _ = fan(fair, oracle, 48, 60, 70, theta(60, "open"), 0, prec)
    rng = np.random.default_rng(1)
    for _ in range(3):
        x, y = rng.random(M.n), rng.random(M.m)
        lhs, rhs = M.project(x) @ y, x @ M.backproject(y)
        assert abs(lhs - rhs) <= tol * abs(lhs)
    M.close()


@pytest.mark.parametrize("method", ["sart", "cimmino"])
@pytest.mark.parametrize("prec,tol", [("f64", 1e-10), ("f32", 1e-5)])
def test_fan_sirt_matches_oracle(fair, oracle, method, prec, tol):
    n, nth, p = 32, 40, 46
    th = theta(nth, "open")
    M, R = fan(fair, oracle, n, nth, p, th, 0, prec)
    b = oracle.matvecmul(R, fair.phantomgallery.shepplogan(n))
    o = fair.airms.options(lbound=0.0, ubound=1.0)
    x = M.sirt(method, b, 30, opts=o)
    xr = oracle.sirt(method, R, b, 30, opts=oracle.options(lbound=0.0, ubound=1.0))
    assert rel_err(x, xr) < tol
    M.close()


def test_fan_beam_argument(fair):
    with pytest.raises(ValueError):
        fair.MatrixFree(fair.Data(n=8, p=10, nth=4, theta=np.zeros(4)), "f32", beam="cone")


@pytest.mark.parametrize("n,p", [(24, 35), (26, 36)])
def test_fan_fp32_matches_fp64(fair, n, p):
    """Fan beam at theta = 2 pi k/8 (axis-aligned central rays included): the
    FP32 entries are the FP64 ones up to FP32 rounding, and the FP32 pair is
    adjoint."""
    nth = 8
    th = theta(nth, "plain")
    d = fair.Data(n=n, p=p, nth=nth, r=2.0, dw=p / n, sd=2.0, theta=th)
    M64, M32 = fair.MatrixFree(d, "f64", beam="fan"), fair.MatrixFree(d, "f32", beam="fan")
    rng = np.random.default_rng(n)
    x, y = rng.random(n * n), rng.random(M64.m)
    for v in (np.ones(n * n), x):
        assert rel_err(M32.project(v), M64.project(v)) < 1e-6
    for w in (np.ones(M64.m), y):
        assert rel_err(M32.backproject(w), M64.backproject(w)) < 1e-6
    lhs, rhs = M32.project(x) @ y, x @ M32.backproject(y)
    assert abs(lhs - rhs) <= 2e-6 * abs(lhs)
    M64.close()
    M32.close()


def test_fan_close_source(fair, oracle):
    """Source 1.2 N from the centre (pixels up to ~36 degrees off the central
    ray): the backprojector searches the bin angles themselves, not their
    tangents; products equal the stored fan matrix's."""
    n, nth, p = 32, 24, 46
    th = theta(nth, "open")
    d = fair.Data(n=n, p=p, nth=nth, r=1.2, dw=p / n, sd=2.0, theta=th)
    M = fair.MatrixFree(d, "f64", beam="fan")
    R = oracle.fanlineartomo(n, nth, p, 1.2, p / n, 2.0, th)
    rng = np.random.default_rng(7)
    x, y = rng.random(R.n), rng.random(R.m)
    assert rel_err(M.project(x), oracle.matvecmul(R, x)) < 1e-12
    assert rel_err(M.backproject(y), oracle.transvecmul(R, y)) < 1e-12
    assert rel_err(M.backproject(np.ones(R.m)), oracle.transvecmul(R, np.ones(R.m))) < 1e-12
    M.close()
