"""GPU adjoint of K unrolled SIRT/SART steps (fair_sirt_adjoint).

Checked against the FP64 CPU adjoint of the oracle (1e-10 relative in FP64),
against central finite differences of the GPU forward (h = 1e-6, agreement
1e-6 relative), and through a torch.autograd.Function harness with
torch.autograd.gradcheck. The batched call (several right-hand sides sharing
the matrix) must equal the single-right-hand-side calls.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def prob(fair, oracle):
    n, nth, p = 32, 36, 46
    th = np.pi * np.arange(nth) / nth
    A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
    R = oracle.paralleltomo(n, nth, p, th)
    rng = np.random.default_rng(3)
    X = np.stack([fair.phantomgallery.random_ellipses(n, seed=s) for s in range(4)], 1)
    B = np.stack([oracle.matvecmul(R, X[:, c]) for c in range(4)], 1)
    B += 0.01 * rng.standard_normal(B.shape) * np.abs(B).mean()
    return A, R, X, B


@pytest.mark.parametrize("method", ["cimmino", "sart"])
def test_adjoint_matches_oracle_fp64(prob, fair, oracle, method):
    A, R, X, B = prob
    K = 20
    lam = 1.4 if method == "cimmino" else 0.9
    o = fair.airms.options(lbound=0.0)
    ro = oracle.options(lbound=0.0)
    xr, _, _, _ = oracle.sirt_adjoint(method, R, B[:, 0], K, lam, np.zeros(R.n), opts=ro)
    gx = xr - X[:, 0]  # dL/dx_K of L = 0.5 ||x_K - x_true||^2
    xK, gb, gx0, gl = fair.airms.sirt_adjoint(method, A, B[:, 0], K, lam, gx, opts=o)
    rx, rb, rx0, rl = oracle.sirt_adjoint(method, R, B[:, 0], K, lam, gx, opts=ro)
    assert rel_err(xK, rx) < 1e-10
    assert rel_err(gb, rb) < 1e-10
    assert rel_err(gx0, rx0) < 1e-10
    assert abs(gl - rl) <= 1e-10 * abs(rl)


def test_adjoint_batch_equals_single(prob, fair):
    A, R, X, B = prob
    K, lam = 12, np.array([1.0, 1.2, 1.4, 1.6])
    o = fair.airms.options(lbound=0.0, ubound=1.5)
    GX = np.random.default_rng(5).standard_normal((R.n, 4))
    X0 = np.full((R.n, 4), 0.02)
    xb, gbb, gxb, glb = fair.airms.sirt_adjoint("sart", A, B, K, lam, GX, x0=X0, opts=o)
    for c in range(4):
        xs, gbs, gxs, gls = fair.airms.sirt_adjoint("sart", A, B[:, c], K, lam[c], GX[:, c],
                                                    x0=X0[:, c], opts=o)
        assert rel_err(xb[:, c], xs) < 1e-12
        assert rel_err(gbb[:, c], gbs) < 1e-12
        assert rel_err(gxb[:, c], gxs) < 1e-12
        assert abs(glb[c] - gls) <= 1e-12 * abs(gls)


def test_adjoint_finite_differences(prob, fair):
    """Directional derivatives along random directions, central differences
    of the GPU forward with h = 1e-6: agreement 1e-6 relative."""
    A, R, X, B = prob
    K, lam, h = 20, 1.3, 1e-6
    b, xt = B[:, 1], X[:, 1]
    x0 = np.full(R.n, 0.05)

    def loss(bb, xx0, ll):
        x = fair.airms.sirt("cimmino", A, bb, K, x0=xx0, opts=fair.airms.options(relaxpar=ll, lbound=0.0))
        return 0.5 * np.sum((x - xt) ** 2), x

    _, xK = loss(b, x0, lam)
    _, gb, gx0, gl = fair.airms.sirt_adjoint("cimmino", A, b, K, lam, xK - xt, x0=x0,
                                             opts=fair.airms.options(lbound=0.0))
    rng = np.random.default_rng(7)
    db, dx = rng.standard_normal(R.m), rng.standard_normal(R.n)
    fd_b = (loss(b + h * db, x0, lam)[0] - loss(b - h * db, x0, lam)[0]) / (2 * h)
    fd_x = (loss(b, x0 + h * dx, lam)[0] - loss(b, x0 - h * dx, lam)[0]) / (2 * h)
    fd_l = (loss(b, x0, lam + h)[0] - loss(b, x0, lam - h)[0]) / (2 * h)
    assert abs(fd_b - gb @ db) <= 1e-6 * abs(fd_b)
    assert abs(fd_x - gx0 @ dx) <= 1e-6 * abs(fd_x)
    assert abs(fd_l - gl) <= 1e-6 * abs(fd_l)


def test_adjoint_fp32(prob, fair, oracle):
    A, R, X, B = prob
    K, lam = 20, 1.4
    ro = oracle.options(lbound=0.0)
    xr, _, _, _ = oracle.sirt_adjoint("cimmino", R, B[:, 2], K, lam, np.zeros(R.n), opts=ro)
    gx = xr - X[:, 2]
    rx, rb, rx0, rl = oracle.sirt_adjoint("cimmino", R, B[:, 2], K, lam, gx, opts=ro)
    A.set_precision("f32")
    try:
        xK, gb, gx0, gl = fair.airms.sirt_adjoint("cimmino", A, B[:, 2], K, lam, gx,
                                                  opts=fair.airms.options(lbound=0.0))
    finally:
        A.set_precision("f64")
    assert rel_err(xK, rx) < 1e-5
    assert rel_err(gb, rb) < 1e-4
    assert rel_err(gx0, rx0) < 1e-4
    assert abs(gl - rl) <= 1e-4 * abs(rl)


def test_torch_autograd_harness(fair, oracle):
    """torch.autograd.Function over the C-ABI (forward: fair_sirt; backward:
    fair_sirt_adjoint), checked by torch.autograd.gradcheck on a tiny problem."""
    torch = pytest.importorskip("torch")
    n, nth, p = 8, 6, 12
    th = np.pi * np.arange(nth) / nth + 0.1
    A = fair.paralleltomo(fair.Data(n=n, p=p, nth=nth, theta=th))
    K = 5

    class SirtK(torch.autograd.Function):
        @staticmethod
        def forward(ctx, b, x0, lam):
            bn, xn, ln = b.detach().numpy(), x0.detach().numpy(), float(lam.item())
            x = fair.airms.sirt("sart", A, bn, K, x0=xn, opts=fair.airms.options(relaxpar=ln))
            ctx.save_for_backward(b, x0, lam)
            return torch.from_numpy(x)

        @staticmethod
        def backward(ctx, g):
            b, x0, lam = ctx.saved_tensors
            _, gb, gx0, gl = fair.airms.sirt_adjoint("sart", A, b.numpy(), K, float(lam.item()),
                                                     g.numpy(), x0=x0.numpy())
            return torch.from_numpy(gb), torch.from_numpy(gx0), torch.tensor([gl], dtype=torch.float64)

    g = torch.Generator().manual_seed(0)
    b = torch.rand(A.m, dtype=torch.float64, generator=g, requires_grad=True)
    x0 = torch.rand(A.n, dtype=torch.float64, generator=g, requires_grad=True)
    lam = torch.tensor([0.8], dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(SirtK.apply, (b, x0, lam), eps=1e-6, atol=1e-7, rtol=1e-5)
