"""GPU: derivatives of linear_solve (lineax/_solve.py:151-317) against
PyTorch fp64 autograd of the same maps — torch.linalg.solve for square
systems, the pseudo-inverse torch.linalg.pinv for least-squares and
minimum-norm solves."""

import numpy as np
import pytest
import torch
from torch.autograd import forward_ad

import lineax_gb300 as lx

pytestmark = pytest.mark.gpu
TOL = 1e-9


def _pair(rng, shape, dev):
    t = torch.tensor(rng.standard_normal(shape), dtype=torch.float64, device=dev)
    return t.clone().requires_grad_(True), t.clone().requires_grad_(True)


def _close(a, b, tol=TOL):
    return float((a - b).abs().max()) <= tol * max(1.0, float(b.abs().max()))


@pytest.mark.parametrize("solver,m,n,tags", [
    (lx.LU(), 40, 40, ()),
    (lx.Cholesky(), 40, 40, (lx.positive_semidefinite_tag,)),
    (lx.QR(), 70, 30, ()),              # least squares: the (b - Ax) term
    (lx.QR(), 25, 60, ()),              # minimum norm: the y term
    (lx.Normal(lx.Cholesky()), 70, 30, ()),
])
def test_reverse_mode_matches_torch(dev, solver, m, n, tags):
    rng = np.random.default_rng(m * 100 + n)
    g = rng.standard_normal((m, n))
    if tags:
        g = g @ g.T / n + np.eye(m)
    elif m == n:
        g = g / np.sqrt(n) + 2 * np.eye(n)
    a = torch.tensor(g, dtype=torch.float64, device=dev)
    a1, a2 = a.clone().requires_grad_(True), a.clone().requires_grad_(True)
    b1, b2 = _pair(rng, (m,), dev)
    w = torch.tensor(rng.standard_normal(n), dtype=torch.float64, device=dev)
    x = lx.linear_solve(lx.MatrixLinearOperator(a1, tags), b1, solver).value
    (x * w).sum().backward()
    x_ref = (torch.linalg.solve(a2, b2) if m == n and not isinstance(solver, (lx.QR, lx.Normal))
             else torch.linalg.pinv(a2) @ b2)
    (x_ref * w).sum().backward()
    assert _close(x.detach(), x_ref.detach())
    assert _close(b1.grad, b2.grad), float((b1.grad - b2.grad).abs().max())
    assert _close(a1.grad, a2.grad), float((a1.grad - a2.grad).abs().max())


def test_forward_mode_matches_torch(dev):
    rng = np.random.default_rng(3)
    for m, n, solver in [(35, 35, lx.LU()), (60, 20, lx.QR()), (20, 45, lx.QR())]:
        g = rng.standard_normal((m, n)) + (2 * np.eye(n) if m == n else 0)
        a = torch.tensor(g, dtype=torch.float64, device=dev)
        b = torch.tensor(rng.standard_normal(m), dtype=torch.float64, device=dev)
        ta = torch.tensor(rng.standard_normal((m, n)), dtype=torch.float64, device=dev)
        tb = torch.tensor(rng.standard_normal(m), dtype=torch.float64, device=dev)
        with forward_ad.dual_level():
            ad = forward_ad.make_dual(a, ta)
            bd = forward_ad.make_dual(b, tb)
            x = lx.linear_solve(lx.MatrixLinearOperator(ad), bd, solver).value
            t = forward_ad.unpack_dual(x).tangent
        f = (lambda A, B: torch.linalg.solve(A, B)) if m == n else \
            (lambda A, B: torch.linalg.pinv(A) @ B)
        _, t_ref = torch.func.jvp(f, (a, b), (ta, tb))
        assert t is not None and _close(t, t_ref), (m, n, float((t - t_ref).abs().max()))


def test_function_operator_parameter_gradient(dev):
    """CG on theta * M (M the Poisson-like SPD matrix) as a FunctionLinearOperator
    closing over theta: x = M^-1 b / theta, so d sum(x) / d theta = -sum(x) / theta."""
    rng = np.random.default_rng(8)
    n = 50
    g = rng.standard_normal((n, n))
    mm = torch.tensor(g @ g.T / n + np.eye(n), dtype=torch.float64, device=dev)
    theta = torch.tensor(1.7, dtype=torch.float64, device=dev, requires_grad=True)
    b = torch.tensor(rng.standard_normal(n), dtype=torch.float64, device=dev,
                     requires_grad=True)
    op = lx.FunctionLinearOperator(lambda v: theta * (mm @ v),
                                   lx.ShapeDtypeStruct((n,), torch.float64),
                                   lx.positive_semidefinite_tag)
    x = lx.linear_solve(op, b, lx.CG(rtol=1e-13, atol=1e-13)).value
    x.sum().backward()
    xs = x.detach()
    assert abs(float(theta.grad) + float(xs.sum()) / 1.7) <= 1e-8 * max(1.0, float(xs.abs().sum()))
    bg = torch.linalg.solve(mm * 1.7, torch.ones(n, dtype=torch.float64, device=dev))
    assert _close(b.grad, bg, 1e-8)


def test_no_graph_without_grad(dev):
    a = torch.eye(4, dtype=torch.float64, device=dev) * 2
    x = lx.linear_solve(lx.MatrixLinearOperator(a), torch.ones(4, dtype=torch.float64,
                                                                 device=dev), lx.LU()).value
    assert not x.requires_grad and x.grad_fn is None
