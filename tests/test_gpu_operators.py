"""GPU parity of the CSR operators (sparse_matrices.f90) with the oracle."""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def problem(fair, oracle):
    n, nth, p = 96, 120, 144
    th = oracle.linspace(0.0, np.pi, nth)
    A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
    R = oracle.paralleltomo(n, nth, p, th)
    return A, R


def test_matvecmul(problem, oracle):
    A, R = problem
    x = np.random.default_rng(0).standard_normal(R.n)
    w = A.matvecmul(x)
    ref = oracle.matvecmul(R, x)
    scale = oracle.matvecmul(R, np.abs(x)) + 1e-300
    assert np.max(np.abs(w - ref) / scale) < 1e-13


def test_transvecmul(problem, oracle):
    A, R = problem
    y = np.random.default_rng(1).standard_normal(R.m)
    w = A.transvecmul(y)
    ref = oracle.transvecmul(R, y)
    scale = oracle.transvecmul(R, np.abs(y)) + 1e-300
    assert np.max(np.abs(w - ref) / scale) < 1e-13


def test_adjoint_identity(problem):
    A, R = problem
    rng = np.random.default_rng(2)
    x, y = rng.standard_normal(R.n), rng.standard_normal(R.m)
    lhs = A.matvecmul(x) @ y
    rhs = x @ A.transvecmul(y)
    assert abs(lhs - rhs) <= 1e-12 * (abs(lhs) + 1)


def test_row_and_column_norms(problem, oracle):
    A, R = problem
    for p in (1, 2):
        assert rel_err(A.row_norms(p), oracle.row_norms(R, p)) < 1e-14
        assert rel_err(A.column_norms(p), oracle.column_norms(R, p)) < 1e-14


def test_transpose_matches_reorder(fair, oracle):
    n, nth, p = 48, 50, 72
    th = oracle.linspace(0.0, np.pi, nth)
    A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
    R = oracle.paralleltomo(n, nth, p, th)
    A.transpose()
    T = oracle.reorder(R)
    vA, IA, JA = A.arrays()
    assert (A.m, A.n) == (T.m, T.n)
    assert np.array_equal(IA, T.IA) and np.array_equal(JA, T.JA) and np.array_equal(vA, T.vA)
    A.transpose()
    vA2, IA2, JA2 = A.arrays()
    assert np.array_equal(IA2, R.IA) and np.array_equal(JA2, R.JA) and np.array_equal(vA2, R.vA)


def test_transpose_long_columns(fair, oracle):
    """Columns longer than the shared-memory sort capacity (4096 entries)."""
    m, n = 6000, 5
    rng = np.random.default_rng(3)
    IA = np.arange(m + 1, dtype=np.int32) * 2
    JA = np.stack([np.full(m, 1), rng.integers(2, n + 1, m)], 1).astype(np.int32).ravel()
    vA = rng.standard_normal(2 * m)
    A = fair.CSRMatrix.construct(m, n, vA, IA, JA)
    A.transpose()
    R = oracle.OracleCSR(m, n, IA.astype(np.int64), JA, vA)
    T = oracle.reorder(R)
    v2, I2, J2 = A.arrays()
    assert np.array_equal(I2, T.IA) and np.array_equal(J2, T.JA) and np.array_equal(v2, T.vA)


def test_rowvecmult_and_add_mult_row(problem, oracle):
    A, R = problem
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, R.n)
    for k in (1, 7, R.m // 2, R.m):
        assert abs(A.rowvecmult(k, x) - oracle.rowvecmult(R, k, x)) <= 1e-13 * (1 + abs(oracle.rowvecmult(R, k, x)))
        for lb, ub in ((None, None), (0.0, None), (None, 0.2), (-0.1, 0.1)):
            w1 = x.copy()
            w2 = x.copy()
            A.add_scalar_mult_row(k, 0.37, w1, lwrb=lb, upb=ub)
            oracle.add_mult_row(R, k, 0.37, w2, lwrb=lb, upb=ub)
            assert np.array_equal(w1, w2)


def test_multiply_by_scalar_and_roundtrip(fair, oracle):
    n, nth, p = 32, 20, 48
    th = oracle.linspace(0.0, np.pi, nth)
    R = oracle.paralleltomo(n, nth, p, th)
    A = fair.CSRMatrix.construct(R.m, R.n, R.vA, R.IA.astype(np.int32), R.JA)
    vA, IA, JA = A.arrays()
    assert np.array_equal(IA, R.IA) and np.array_equal(JA, R.JA) and np.array_equal(vA, R.vA)
    A.multiply_by_scalar(0.3)
    oracle.scalar_mult(R, 0.3)
    assert np.array_equal(A.arrays()[0], R.vA)


def test_size_errors(problem, fair):
    A, R = problem
    with pytest.raises(fair.FairError) as ei:
        A.matvecmul(np.zeros(R.n + 1))
    assert ei.value.status == 1 and "Vector input size incorrect." in str(ei.value)
    with pytest.raises(fair.FairError):
        A.transvecmul(np.zeros(R.n))
    with pytest.raises(fair.FairError):
        fair.CSRMatrix.construct(2, 2, [1.0], np.array([0, 1, 1], np.int32), np.array([3], np.int32))


@pytest.mark.parametrize("prec,tol", [("f32", 1e-6), ("f16", 2e-3), ("q16", 1e-4)])
def test_reduced_precision_products(problem, oracle, prec, tol):
    A, R = problem
    x = np.random.default_rng(5).uniform(0, 1, R.n)
    A.set_precision(prec)
    try:
        assert rel_err(A.matvecmul(x), oracle.matvecmul(R, x)) < tol
        y = np.random.default_rng(6).uniform(0, 1, R.m)
        assert rel_err(A.transvecmul(y), oracle.transvecmul(R, y)) < tol
    finally:
        A.set_precision("f64")
