"""GPU parity of the ray-traced system matrix with the oracle.

paralleltomo (system_generation.f90:309-492) and fanlineartomo (:79-307):
row offsets IA and column indices JA must be bit-exact, segment lengths vA
within 1e-12 relative (they are expected to be bit-exact as well).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

VA_RTOL = 1e-12


def _compare(F, O, A, R):
    vA, IA, JA = A.arrays()
    assert A.m == R.m and A.n == R.n
    assert np.array_equal(IA, R.IA), "row offsets differ"
    assert np.array_equal(JA, R.JA), "column indices differ"
    if R.nnz:
        rel = np.max(np.abs(vA - R.vA) / np.maximum(np.abs(R.vA), 1e-300))
        assert rel <= VA_RTOL, f"max relative vA difference {rel}"
    return vA


def _par(F, O, n, nth, p, theta):
    """Build on both sides; when the reference stops ('++ Something went
    wrong', a ray along the top edge), the GPU build must refuse as well."""
    try:
        R = O.paralleltomo(n, nth, p, theta)
    except O.OracleError as e:
        assert e.code == 3
        with pytest.raises(F.FairError) as ei:
            F.paralleltomo(F.Data(n=n, p=p, nth=nth, theta=theta))
        assert ei.value.status == 3
        return None, None
    A = F.paralleltomo(F.Data(n=n, p=p, nth=nth, theta=theta))
    return A, R


def test_parallel_main_exe_problem(fair, oracle):
    """main.exe -t: N=256, 400 angles over linspace(0,pi), p=1.5N (main.f90:191-205)."""
    th = oracle.linspace(0.0, np.pi, 400)
    A, R = _par(fair, oracle, 256, 400, 384, th)
    vA = _compare(fair, oracle, A, R)
    assert A.nnz == 33360464
    assert np.array_equal(vA, R.vA)


@pytest.mark.parametrize("n,nth,p", [(32, 37, 48), (32, 37, 31), (32, 37, 47), (31, 19, 45),
                                     (31, 19, 29), (17, 8, 16), (1, 3, 1), (2, 5, 3),
                                     (64, 90, 63), (64, 90, 91)])
def test_parallel_small(fair, oracle, n, nth, p):
    # angles include 0, pi/4 and pi/2 exactly: axis-aligned and diagonal rays,
    # NaN keys (odd p, ray on a grid line) and exact crossing ties
    th = np.concatenate([[0.0, np.pi / 4, np.pi / 2, 3 * np.pi / 4],
                         oracle.linspace(0.1, 3.0, nth - 4)]) if nth > 4 else \
        oracle.linspace(0.0, np.pi, nth)
    A, R = _par(fair, oracle, n, nth, p, th)
    if R is not None:
        _compare(fair, oracle, A, R)


@pytest.mark.parametrize("n,p", [(32, 31), (33, 33), (16, 15)])
def test_parallel_grid_line_rays(fair, oracle, n, p):
    """Odd p puts rays exactly on grid lines at theta = 0 (a = -0): the
    reference's quicksort then meets 0/0 keys; the exact path replays it."""
    th = np.array([0.0, 0.5, np.pi / 4])
    A, R = _par(fair, oracle, n, 3, p, th)
    assert R is not None
    _compare(fair, oracle, A, R)


def test_parallel_boundary_ray_excluded(fair, oracle):
    """A ray along the right edge is dropped (system_generation.f90:393-394)."""
    th = np.array([0.0, 0.3])
    A, R = _par(fair, oracle, 8, 2, 9, th)
    _compare(fair, oracle, A, R)
    IA = R.IA
    assert IA[9] - IA[8] == 0  # x0 = +4 = N/2 at theta = 0


def test_parallel_top_edge_ray_stops(fair, oracle):
    """A ray along the top edge with b != 0 produces column 0: the reference
    stops with '++ Something went wrong' (:478); both implementations refuse."""
    th = oracle.linspace(0.0, np.pi, 3)  # contains pi/2 exactly
    with pytest.raises(oracle.OracleError):
        oracle.paralleltomo(8, 3, 9, th)
    with pytest.raises(fair.FairError) as ei:
        fair.paralleltomo(fair.Data(n=8, p=9, nth=3, theta=th))
    assert ei.value.status == 3


@pytest.mark.parametrize("p,fix", [(181, False), (181, True), (182, False)])
def test_fan_config1(fair, oracle, p, fix):
    """Fan beam N=128, R=2N, 360 angles over [0, 2pi), unit bins (odd p keeps
    the reference's ray angles of system_generation.f90:122 unless fixed)."""
    n, nth = 128, 360
    th = 2 * np.pi * np.arange(nth) / nth
    d = fair.Data(n=n, p=p, nth=nth, r=2.0, dw=p / n, sd=2.0, theta=th)
    A = fair.fanlineartomo(d, geometry_fix=fix)
    R = oracle.fanlineartomo(n, nth, p, 2.0, p / n, 2.0, th, geometry_fix=fix)
    _compare(fair, oracle, A, R)
    if p == 181 and not fix:
        assert R.nnz == 3907192


@pytest.mark.parametrize("n,p", [(15, 21), (16, 21), (33, 40)])
def test_fan_small(fair, oracle, n, p):
    nth = 24
    th = np.concatenate([[0.0, np.pi / 2, np.pi, 1.5 * np.pi], 2 * np.pi * np.arange(1, nth - 3) / nth])
    d = fair.Data(n=n, p=p, nth=nth, r=1.5, dw=1.2, sd=2.5, theta=th)
    A = fair.fanlineartomo(d)
    R = oracle.fanlineartomo(n, nth, p, 1.5, 1.2, 2.5, th)
    _compare(fair, oracle, A, R)


def test_geometry_properties(fair, oracle):
    """Size-independent checks: columns in 1..N^2; at theta = 0 every ray that
    crosses the square has N unit segments, so the angle's lengths sum to N^2
    exactly; at other angles the unit-spaced chord sum is a midpoint rule for
    the area, within a few units of N^2; every row is shorter than 2N."""
    n, nth, p = 128, 30, 192
    th = oracle.linspace(0.0, np.pi, nth)
    A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
    vA, IA, JA = A.arrays()
    assert JA.min() >= 1 and JA.max() <= n * n
    assert np.diff(IA).max() <= 2 * n
    assert vA[IA[0]:IA[p]].sum() == n * n
    for i in range(nth):
        s = vA[IA[i * p]:IA[(i + 1) * p]].sum()
        assert abs(s - n * n) <= 4.0
