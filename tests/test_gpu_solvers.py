"""GPU parity of the AIR iterations (AIRMs.f90) with the oracle.

FP64 iterates must agree within 1e-10 relative; the reduced-precision SIRT
forms are checked against the FP64 oracle with the tolerances written below.
Random draws (scramble, row sampling, normest start vector) come from the
same seeded stream on both sides.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL64 = 1e-10


@pytest.fixture(scope="module")
def par(fair, oracle):
    n, nth, p = 64, 90, 96
    th = oracle.linspace(0.0, np.pi, nth)
    A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
    R = oracle.paralleltomo(n, nth, p, th)
    x = oracle.shepplogan(n)
    b = oracle.matvecmul(R, x)
    oracle.random_seed(11)
    bt, _ = oracle.add_white_noise(b, 0.01)
    return A, R, x, bt


@pytest.fixture(scope="module")
def fan1(fair, oracle):
    """Fan-beam N=128, 360 angles, 181 unit bins, R=2N (odd p, reference angles)."""
    n, nth, p = 128, 360, 181
    th = 2 * np.pi * np.arange(nth) / nth
    A = fair.fanlineartomo(fair.Data(n=n, p=p, nth=nth, r=2.0, dw=p / n, sd=2.0, theta=th))
    R = oracle.fanlineartomo(n, nth, p, 2.0, p / n, 2.0, th)
    x = oracle.shepplogan(n)
    b = oracle.matvecmul(R, x)
    oracle.random_seed(0)
    bt, _ = oracle.add_white_noise(b, 0.01)
    return A, R, x, bt


@pytest.mark.parametrize("method", ["cimmino", "sart"])
@pytest.mark.parametrize("bounds", [(None, None), (0.0, None), (0.0, 1.0), (None, 0.5)])
def test_sirt(par, fair, oracle, method, bounds):
    A, R, _, b = par
    lb, ub = bounds
    relax = 1.0 if method == "sart" else 1.5
    o = fair.airms.options(relaxpar=relax, lbound=lb, ubound=ub)
    ro = oracle.options(relaxpar=relax, lbound=lb, ubound=ub)
    x = fair.airms.sirt(method, A, b, 20, opts=o)
    xr = oracle.sirt(method, R, b, 20, opts=ro)
    assert rel_err(x, xr) < TOL64


def test_rows_by_group_equals_chunked(par, fair, monkeypatch):
    """A matrix with few 32-row chunks (8,640 rays, 4,096 pixels) runs its FP64
    CSR passes a group of rows per warp; the chunked engine
    (FAIR_ROWS_BY_GROUP=0) has the same arithmetic per row: the same bits."""
    A, R, _, b = par
    o = fair.airms.options(relaxpar=1.5, lbound=0.0)
    x1 = fair.airms.sirt("cimmino", A, b, 10, opts=o)
    monkeypatch.setenv("FAIR_ROWS_BY_GROUP", "0")
    x2 = fair.airms.sirt("cimmino", A, b, 10, opts=o)
    assert np.array_equal(x1, x2)


def test_fp64_csr_many_rows(fair, oracle):
    """Parallel N=96, 720 angles, 136 bins: 97,920 rays, enough 32-row chunks
    for the chunked engine on A (A' still a group of rows per warp)."""
    n, nth, p = 96, 720, 136
    th = np.pi * np.arange(nth) / nth
    A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
    R = oracle.paralleltomo(n, nth, p, th)
    b = oracle.matvecmul(R, oracle.shepplogan(n))
    for method in ("cimmino", "sart"):
        x = fair.airms.sirt(method, A, b, 5, opts=fair.airms.options(lbound=0.0))
        xr = oracle.sirt(method, R, b, 5, opts=oracle.options(lbound=0.0))
        assert rel_err(x, xr) < TOL64
    A.close()


def test_sirt_x0_and_defaults(par, fair, oracle):
    A, R, _, b = par
    x0 = np.full(R.n, 0.1)
    assert rel_err(fair.airms.sirt("cimmino", A, b, [3, 7], x0=x0),
                   oracle.sirt("cimmino", R, b, 7, x0=x0)) < TOL64
    with pytest.raises(fair.FairError) as ei:
        fair.airms.sirt("landweber", A, b, 3)
    assert ei.value.status == 2


def test_cimmino_config1(fan1, fair, oracle):
    """Cimmino, 100 iterations, L=0, lambda = 1.9/||M^(1/2) A||^2 (power iteration)."""
    A, R, _, b = fan1
    nr = oracle.row_norms(R, 2)
    Mh = np.where(nr > 0, 1.0 / np.sqrt(R.m * nr * nr + (nr == 0)), 0.0)
    # sigma_max of M^(-1/2) A by power iteration on the oracle (host numpy)
    import scipy.sparse as sp
    S = sp.csr_matrix((R.vA, R.JA - 1, R.IA), shape=(R.m, R.n))
    B = sp.diags(Mh) @ S
    v = np.random.default_rng(0).uniform(size=R.n)
    for _ in range(200):
        v = B.T @ (B @ v)
        v /= np.linalg.norm(v)
    sig2 = np.linalg.norm(B @ v) ** 2
    lam = 1.9 / sig2
    o = fair.airms.options(relaxpar=lam, lbound=0.0)
    ro = oracle.options(relaxpar=lam, lbound=0.0)
    x = fair.airms.sirt("cimmino", A, b, 100, opts=o)
    xr = oracle.sirt("cimmino", R, b, 100, opts=ro)
    assert rel_err(x, xr) < TOL64


def test_normest_and_gradient_descent(par, fair, oracle):
    A, R, _, b = par
    fair.airms.random_seed(5)
    oracle.random_seed(5)
    s_gpu = fair.airms.normest(A)
    v0 = oracle.random_number(R.n)
    s_ref = oracle.normest(R, v0)
    assert abs(s_gpu - s_ref) <= TOL64 * s_ref
    fair.airms.random_seed(6)
    oracle.random_seed(6)
    for opts in (None, (0.0, None), (0.0, 1.0)):
        o = ro = None
        if opts is not None:
            o = fair.airms.options(lbound=opts[0], ubound=opts[1])
            ro = oracle.options(lbound=opts[0], ubound=opts[1])
        x, it = fair.airms.gradient_descent(A, b, max_iter=40, opts=o)
        xr, itr = oracle.gradient_descent(R, b, max_iter=40, opts=ro)
        assert it == itr
        assert rel_err(x, xr) < TOL64


def test_gradient_descent_tolerance_exit(par, fair, oracle):
    A, R, _, b = par
    fair.airms.random_seed(8)
    oracle.random_seed(8)
    x, it = fair.airms.gradient_descent(A, b, max_iter=500, tolerance=5e-2)
    xr, itr = oracle.gradient_descent(R, b, max_iter=500, tol=5e-2)
    assert it == itr < 500
    assert rel_err(x, xr) < TOL64


@pytest.mark.parametrize("method,K", [("kaczmarz", [1, 3]), ("symkaczmarz", [2, 4]),
                                      ("randkaczmarz", [2])])
@pytest.mark.parametrize("bounds", [(None, None), (0.0, 1.0), (0.0, None)])
def test_art(par, fair, oracle, method, K, bounds):
    A, R, _, b = par
    lb, ub = bounds
    o = fair.airms.options(relaxpar=0.25, lbound=lb, ubound=ub)
    ro = oracle.options(relaxpar=0.25, lbound=lb, ubound=ub)
    fair.airms.random_seed(9)
    oracle.random_seed(9)
    X = fair.airms.art(method, A, b, K, opts=o)
    Xr = oracle.art(method, R, b, K, opts=ro)
    for l in range(len(K)):
        assert rel_err(X[:, l], Xr[:, l]) < TOL64


def test_randkaczmarz_rowprob(par, fair, oracle):
    A, R, _, b = par
    o = fair.airms.options(relaxpar=0.5, rowprobability=True, lbound=0.0)
    ro = oracle.options(relaxpar=0.5, rowprobability=True, lbound=0.0)
    fair.airms.random_seed(10)
    oracle.random_seed(10)
    X = fair.airms.art("randkaczmarz", A, b, [1, 2], opts=o)
    Xr = oracle.art("randkaczmarz", R, b, [1, 2], opts=ro)
    assert rel_err(X, Xr) < TOL64


def test_art_order_damp_xref(par, fair, oracle):
    A, R, xt, b = par
    order = np.random.default_rng(1).permutation(R.m)[: R.m // 2].astype(np.int32) + 1
    o = fair.airms.options(relaxpar=1.0, damp=0.1)
    ro = oracle.options(relaxpar=1.0, damp=0.1)
    X = fair.airms.art("kaczmarz", A, b, [2], order=order, opts=o)
    Xr = oracle.art("kaczmarz", R, b, [2], order=order, opts=ro)
    assert rel_err(X, Xr) < TOL64
    # oracle stopping rule: returns the previous iterate once the error grows
    X = fair.airms.art("kaczmarz", A, b, [30], xref=xt)
    Xr = oracle.art("kaczmarz", R, b, [30], xref=xt)
    assert rel_err(X, Xr) < TOL64


@pytest.mark.parametrize("warps", ["1", "2", "4", "8"])
def test_art_sweep_warps(par, fair, oracle, monkeypatch, warps):
    """Every warps-per-row choice of the single-block sweep: the row sums of 1
    to 8 warps (exact integer sums of the lanes' FP64 partials) against the
    oracle."""
    monkeypatch.setenv("FAIR_SWEEP_LEGACY", "1")
    monkeypatch.setenv("FAIR_SWEEP_WARPS", warps)
    A, R, _, b = par
    o = fair.airms.options(relaxpar=0.25, lbound=0.0, ubound=1.0)
    ro = oracle.options(relaxpar=0.25, lbound=0.0, ubound=1.0)
    X = fair.airms.art("kaczmarz", A, b, [2], opts=o)
    Xr = oracle.art("kaczmarz", R, b, [2], opts=ro)
    assert rel_err(X, Xr) < TOL64


@pytest.mark.parametrize("warps", ["window", "2", "8"])
def test_art_iterate_in_global_memory(fair, oracle, monkeypatch, warps):
    """N=192 (36,864 unknowns: more than one block's shared memory holds): the
    windowed sweep keeps each window's columns in slots, the single-block
    sweep gathers the iterate from global memory."""
    if warps != "window":
        monkeypatch.setenv("FAIR_SWEEP_LEGACY", "1")
        monkeypatch.setenv("FAIR_SWEEP_WARPS", warps)
    n, nth, p = 192, 24, 272
    th = oracle.linspace(0.0, np.pi, nth)
    A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
    R = oracle.paralleltomo(n, nth, p, th)
    b = oracle.matvecmul(R, oracle.shepplogan(n))
    o = fair.airms.options(relaxpar=0.5, lbound=0.0)
    ro = oracle.options(relaxpar=0.5, lbound=0.0)
    X = fair.airms.art("symkaczmarz", A, b, [2], opts=o)
    Xr = oracle.art("symkaczmarz", R, b, [2], opts=ro)
    assert rel_err(X, Xr) < TOL64


def test_art_nonfinite_b(par, fair, oracle):
    """NaN and +-Inf entries of b: the row sum is then the FP64 sum of the
    non-finite terms, and the box (MAX/MIN semantics: NaN loses) brings the
    iterate back to finite values as in the oracle."""
    A, R, _, b = par
    bb = b.copy()
    bb[5], bb[77], bb[300] = np.nan, np.inf, -np.inf
    o = fair.airms.options(relaxpar=0.25, lbound=0.0, ubound=1.0)
    ro = oracle.options(relaxpar=0.25, lbound=0.0, ubound=1.0)
    X = fair.airms.art("kaczmarz", A, bb, [1, 2], opts=o)
    Xr = oracle.art("kaczmarz", R, bb, [1, 2], opts=ro)
    assert np.all(np.isfinite(X)) and np.all(np.isfinite(Xr))
    assert rel_err(X, Xr) < TOL64


def test_art_errors(par, fair):
    A, R, _, b = par
    with pytest.raises(fair.FairError) as ei:
        fair.airms.art("symkaczmarz", A, b, [3])
    assert ei.value.status == 4
    with pytest.raises(fair.FairError) as ei:
        fair.airms.art("landweber", A, b, [3])
    assert ei.value.status == 2


def test_kaczmarz_config1(fan1, fair, oracle):
    """Kaczmarz, 10 natural-order sweeps, lambda = 0.25 (fan-beam N=128)."""
    A, R, _, b = fan1
    o = fair.airms.options(relaxpar=0.25)
    ro = oracle.options(relaxpar=0.25)
    X = fair.airms.art("kaczmarz", A, b, [10], opts=o)
    Xr = oracle.art("kaczmarz", R, b, [10], opts=ro)
    assert rel_err(X, Xr) < TOL64


@pytest.mark.parametrize("rule", ["errorgauge", "mutualstep"])
@pytest.mark.parametrize("method,K", [("kaczmarz", 12), ("symkaczmarz", 12)])
def test_twin_art(par, fair, oracle, rule, method, K):
    A, R, _, b = par
    o = fair.airms.options(relaxpar=0.5, lbound=0.0)
    ro = oracle.options(relaxpar=0.5, lbound=0.0)
    g = fair.airms.twin_art(method, rule, A, b, [K], opts=o)
    r = oracle.twin_art(method, rule, R, b, [K], opts=ro)
    assert g[1] == r[1], "final iteration differs"
    assert rel_err(g[0], r[0]) < TOL64
    assert rel_err(g[4], r[4]) < TOL64


@pytest.mark.parametrize("prec,tol", [("f32", 1e-5), ("f16", 5e-3), ("q16", 1e-5)])
def test_sirt_reduced_precision(par, fair, oracle, prec, tol):
    """FP32 / FP16-stored values with FP32 accumulation: error vs the FP64 oracle."""
    A, R, _, b = par
    o = fair.airms.options(relaxpar=1.0, lbound=0.0)
    ro = oracle.options(relaxpar=1.0, lbound=0.0)
    xr = oracle.sirt("sart", R, b, 50, opts=ro)
    A.set_precision(prec)
    try:
        x = fair.airms.sirt("sart", A, b, 50, opts=o)
    finally:
        A.set_precision("f64")
    assert rel_err(x, xr) < tol
