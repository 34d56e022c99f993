"""GPU parity of the level-scheduled Kaczmarz sweep (kaczmarz.cu) with the oracle.

The sweep gives every step the level 1 + the largest level of the earlier
steps that share a column with it, and runs the levels in order with the steps
of a level in parallel over a thread-block cluster. That is the sequence of
bounded projections of basic_sweep (AIRMs.f90:813-858), so the iterate must
equal the oracle's within 1e-10 relative for every order (natural, reversed,
permuted, sampled with repeats), cluster shape and level-table placement.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL64 = 1e-10


@pytest.fixture(scope="module")
def fan(fair, oracle):
    """Fan beam N=48, 120 angles, 69 bins (odd p), noisy Shepp-Logan data."""
    n, nth, p = 48, 120, 69
    th = 2 * np.pi * np.arange(nth) / nth
    A = fair.fanlineartomo(fair.Data(n=n, p=p, nth=nth, r=2.0, dw=p / n, sd=2.0, theta=th))
    R = oracle.fanlineartomo(n, nth, p, 2.0, p / n, 2.0, th)
    b = oracle.matvecmul(R, oracle.shepplogan(n))
    e = np.random.default_rng(3).standard_normal(b.size)
    bt = b + 0.01 * np.linalg.norm(b) / np.linalg.norm(e) * e
    return A, R, bt


def run_both(fair, oracle, A, R, b, method, K, **kw):
    fair.airms.random_seed(21)
    oracle.random_seed(21)
    X = fair.airms.art(method, A, b, K, opts=fair.airms.options(**kw))
    Xr = oracle.art(method, R, b, K, opts=oracle.options(**kw))
    return X, Xr


CASES = (("kaczmarz", [1, 3], dict(relaxpar=0.25, lbound=0.0, ubound=1.0)),
         ("symkaczmarz", [2], dict(relaxpar=0.5, lbound=0.0)),
         ("randkaczmarz", [2], dict(relaxpar=0.5, lbound=0.0, ubound=1.0)),
         ("randkaczmarz", [1], dict(relaxpar=1.0, rowprobability=True)))


@pytest.mark.parametrize("xmem", ["0", "1"])
@pytest.mark.parametrize("cluster", ["1", "2", "16"])
def test_level_sweep_orders(fan, fair, oracle, monkeypatch, cluster, xmem):
    """Natural, symmetric, permuted and sampled orders on one block and on
    clusters of 2 and up to 16 blocks, x in global memory or in (distributed)
    shared memory (random orders forced onto levels: by default a sweep drawn
    anew runs on the single-block kernel)."""
    monkeypatch.setenv("FAIR_SWEEP_CLUSTER", cluster)
    monkeypatch.setenv("FAIR_SWEEP_XMEM", xmem)
    monkeypatch.setenv("FAIR_SWEEP_LEVELS_ALWAYS", "1")
    A, R, b = fan
    for method, K, kw in CASES:
        X, Xr = run_both(fair, oracle, A, R, b, method, K, **kw)
        for l in range(len(K)):
            assert rel_err(X[:, l], Xr[:, l]) < TOL64, (method, kw)


@pytest.mark.parametrize("group", ["2", "8"])
def test_level_sweep_cooperative_grid(fan, fair, oracle, monkeypatch, group):
    """The level sweep on a cooperative grid of blocks (x in global memory, a
    software grid barrier between levels), as taken when a level holds more
    steps than one round of the cluster's warp groups."""
    monkeypatch.setenv("FAIR_SWEEP_GRID", "1")
    monkeypatch.setenv("FAIR_SWEEP_LEVELS_ALWAYS", "1")
    monkeypatch.setenv("FAIR_SWEEP_GROUP", group)
    A, R, b = fan
    for method, K, kw in CASES:
        X, Xr = run_both(fair, oracle, A, R, b, method, K, **kw)
        for l in range(len(K)):
            assert rel_err(X[:, l], Xr[:, l]) < TOL64, (method, kw)


def test_level_sweep_equals_single_block_kernel(fan, fair, oracle, monkeypatch):
    """The level sweep (default) and the single-block sweep on one problem."""
    A, R, b = fan
    kw = dict(relaxpar=0.25, lbound=0.0, ubound=1.0)
    Xl, Xr = run_both(fair, oracle, A, R, b, "symkaczmarz", [4], **kw)
    monkeypatch.setenv("FAIR_SWEEP_LEGACY", "1")
    Xs, _ = run_both(fair, oracle, A, R, b, "symkaczmarz", [4], **kw)
    assert rel_err(Xl, Xr) < TOL64
    assert rel_err(Xs, Xr) < TOL64
    assert rel_err(Xl, Xs) < TOL64


@pytest.mark.parametrize("cluster", ["8", "16"])
@pytest.mark.parametrize("group", ["1", "2", "4", "8"])
def test_level_sweep_long_rows_global_table(fair, oracle, monkeypatch, group, cluster):
    """Parallel beam N=256 (65,536 columns: the level table lives in global
    memory, its levels computed on a 16-block cluster or on one block; diagonal
    rays of up to ~360 entries run past the registers of one warp), each step
    on a group of 1, 2, 4 or 8 warps."""
    monkeypatch.setenv("FAIR_SWEEP_LEVELS_ALWAYS", "1")
    monkeypatch.setenv("FAIR_SWEEP_GROUP", group)
    monkeypatch.setenv("FAIR_SWEEP_CLUSTER", cluster)
    n, nth, p = 256, 12, 362
    th = oracle.linspace(0.0, np.pi, nth)
    A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
    R = oracle.paralleltomo(n, nth, p, th)
    assert int(np.diff(R.IA).max()) > 256
    b = oracle.matvecmul(R, oracle.shepplogan(n))
    for method, K, kw in CASES[:3]:
        X, Xr = run_both(fair, oracle, A, R, b, method, K, **kw)
        assert rel_err(X, Xr) < TOL64, method


def test_level_sweep_sampled_rows_repeat(fair, oracle, monkeypatch):
    """Random Kaczmarz with row probabilities on few rows: the same row is
    drawn many times in a sweep, each draw a step of its own level."""
    monkeypatch.setenv("FAIR_SWEEP_LEVELS_ALWAYS", "1")
    n, nth, p = 24, 6, 34
    th = oracle.linspace(0.0, np.pi, nth)
    A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
    R = oracle.paralleltomo(n, nth, p, th)
    b = oracle.matvecmul(R, oracle.shepplogan(n))
    X, Xr = run_both(fair, oracle, A, R, b, "randkaczmarz", [3], relaxpar=0.7,
                     rowprobability=True, lbound=0.0)
    assert rel_err(X, Xr) < TOL64


def test_level_sweep_twin_art(fan, fair, oracle):
    """twin_art sweeps x forwards and y backwards with the same order: both
    level schedules are built once and reused."""
    A, R, b = fan
    for rule in ("errorgauge", "mutualstep"):
        g = fair.airms.twin_art("symkaczmarz", rule, A, b, [8],
                                opts=fair.airms.options(relaxpar=0.5, lbound=0.0))
        r = oracle.twin_art("symkaczmarz", rule, R, b, [8],
                            opts=oracle.options(relaxpar=0.5, lbound=0.0))
        assert g[1] == r[1]
        assert rel_err(g[0], r[0]) < TOL64


def test_level_sweep_row_repeating_a_column(fan, fair, oracle):
    """A matrix whose rows repeat a column (constructed, not traced): the
    set-up detects it and the single-block kernel applies such a row's updates
    one after the other, as add_mult_row does."""
    _, R0, b = fan
    IA, JA, vA = R0.IA.copy(), R0.JA.copy(), R0.vA.copy()
    rows = [i for i in range(R0.m) if IA[i + 1] - IA[i] >= 4][::50]
    for i in rows:
        JA[IA[i] + 2] = JA[IA[i]]  # the row's first column again
    R = oracle.OracleCSR(R0.m, R0.n, IA, JA, vA)
    A = fair.CSRMatrix.construct(R0.m, R0.n, vA, IA, JA)
    for method, kw in (("kaczmarz", dict(relaxpar=0.25, lbound=0.0, ubound=1.0)),
                       ("symkaczmarz", dict(relaxpar=0.5)),
                       ("randkaczmarz", dict(relaxpar=0.5, lbound=0.0)),
                       ("randkaczmarz", dict(relaxpar=0.5, rowprobability=True))):
        X, Xr = run_both(fair, oracle, A, R, b, method, [2], **kw)
        assert rel_err(X, Xr) < TOL64, (method, kw)
