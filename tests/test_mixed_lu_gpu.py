"""GPU: the FP32 LU with tensor-core (tcgen05 TF32) trailing updates, and
GMRES-IR with it as preconditioner, against the FP64 oracle."""

import numpy as np
import pytest
import torch

import lineax_gb300 as lx
from lineax_gb300 import mixed
from oracle import dense, krylov

pytestmark = pytest.mark.gpu


def haar(rng, n):
    q, r = np.linalg.qr(rng.standard_normal((n, n)))
    return q * np.sign(np.diag(r))


def conditioned(n, cond, seed):
    """A = U diag(sigma) Vᵀ, U and V Haar, sigma log-spaced with max/min = cond."""
    rng = np.random.default_rng(seed)
    u, v = haar(rng, n), haar(rng, n)
    s = np.logspace(0, -np.log10(cond), n)
    return (u * s) @ v.T


@pytest.mark.parametrize("precision,bound", [("tf32", 3e-2), ("3xtf32", 5e-5)])
@pytest.mark.parametrize("n", [64, 256, 600, 1024])
def test_tf32_lu_factorisation_residual(dev, n, precision, bound):
    """||P A - L U|| / ||A||: TF32 products leave a few units of sqrt(n) 2^-11;
    3xTF32 is at FP32 level."""
    a = conditioned(n, 1e2, n)
    f = mixed.lu_factor_tf32(torch.tensor(a, device=dev), precision)
    assert int(f.info) == 0
    lu = f.lu.double().cpu().numpy()
    piv = f.piv.cpu().numpy()
    l = np.tril(lu, -1) + np.eye(n)
    u = np.triu(lu)
    pa = a.copy()
    for k in range(n):
        pa[[k, piv[k]]] = pa[[piv[k], k]]
    rel = np.linalg.norm(pa - l @ u) / np.linalg.norm(a)
    assert rel < bound, rel


@pytest.mark.parametrize("n,cond", [(256, 1e2), (512, 1e6), (1024, 1e2), (1024, 1e6)])
def test_gmres_ir_reaches_fp64_backward_error(dev, n, cond):
    a = conditioned(n, cond, n + int(np.log10(cond)))
    rng = np.random.default_rng(7)
    b = rng.standard_normal((4, n))
    res = mixed.gmres_ir(torch.tensor(a, device=dev), torch.tensor(b, device=dev), tol=1e-12)
    assert res.converged and res.outer <= 6, (res.outer, res.berr)
    x = res.x.cpu().numpy()
    for c in range(4):
        assert res.berr[c] <= 1e-12
        assert dense.backward_error(a, x[c], b[c]) <= 1e-12
        assert dense.forward_error(x[c], dense.lu_linear_solve(a, b[c])) <= cond * 1e-13


def test_gmres_ir_through_linear_solve(dev):
    """lx.linear_solve(op, b, GMRES, options={"preconditioner": M}) with the TF32 LU
    as M matches the preconditioned GMRES restatement."""
    n = 256
    a = conditioned(n, 1e3, 3)
    b = np.random.default_rng(1).standard_normal(n)
    op = lx.MatrixLinearOperator(torch.tensor(a, device=dev))
    m = mixed.lu_preconditioner(op)
    sol = lx.linear_solve(op, torch.tensor(b, device=dev), lx.GMRES(rtol=1e-10, atol=1e-10),
                          options={"preconditioner": m})
    assert sol.result == lx.RESULTS.successful
    x = sol.value.cpu().numpy()
    assert dense.backward_error(a, x, b) <= 1e-12
    lu = m.factor.lu.cpu().numpy()
    piv = m.factor.piv.cpu().numpy()

    def pre(v):  # the FP32 factor applied in FP32, as on the device
        import scipy.linalg as sl
        return sl.lu_solve((lu, piv), v.astype(np.float32)).astype(np.float64)

    x_ref, r_ref, s_ref = krylov.gmres(lambda v: a @ v, b, rtol=1e-10, atol=1e-10, precond=pre)
    # FP32 preconditioner applies differ in rounding order: allow two restart cycles
    assert r_ref == 0 and abs(sol.stats["num_steps"] - s_ref) <= 2
