"""GPU parity: Householder QR (geqrf/ormqr) and the QR solver against SciPy
LAPACK (geqrf + ormqr + trsm), including the reference's 2×2 known answers."""

import json
import pathlib

import numpy as np
import pytest
import torch

import lineax_gb300 as lx
from lineax_gb300 import _dense
from oracle import dense

pytestmark = pytest.mark.gpu
GOLD = json.loads((pathlib.Path(__file__).parent / "golden" / "reference_kats.json").read_text())


def t(x, dev):
    return torch.tensor(np.asarray(x), dtype=torch.float64, device=dev)


@pytest.mark.parametrize("m,n", [(1, 1), (5, 3), (64, 64), (100, 33), (300, 100), (1000, 257),
                                 (2500, 96)])
def test_geqrf_matches_lapack(dev, m, n):
    rng = np.random.default_rng(m * 7 + n)
    a = rng.standard_normal((m, n))
    h, tau, _ = _dense.geqrf(t(a, dev))
    h_ref, tau_ref, _ = dense.qr_factor(a)   # h_ref: m×n geqrf output
    got = h.cpu().numpy().T                    # back to m×n
    np.testing.assert_allclose(tau.cpu().numpy(), tau_ref, rtol=1e-9, atol=1e-12)
    r, r_ref = np.triu(got[:n]), np.triu(h_ref[:n])
    np.testing.assert_allclose(r, r_ref, rtol=1e-9, atol=1e-10 * np.abs(r_ref).max())
    v, v_ref = np.tril(got, -1), np.tril(h_ref, -1)
    np.testing.assert_allclose(v, v_ref, rtol=1e-8, atol=1e-10)


@pytest.mark.parametrize("m,n,trans", [(300, 100, 1), (300, 100, 0), (2000, 600, 1),
                                       (2000, 600, 0)])
def test_ormqr_matches_lapack(dev, m, n, trans):
    rng = np.random.default_rng(m + n + trans)
    a = rng.standard_normal((m, n))
    c = rng.standard_normal((3, m))
    h, tau, tt = _dense.geqrf(t(a, dev))
    got = _dense.ormqr(h, tau, tt, t(c, dev), trans=bool(trans)).cpu().numpy()
    h_ref, tau_ref, _ = dense.qr_factor(a)
    ref = dense._ormqr(h_ref, tau_ref, np.asfortranarray(c.T), "L", "T" if trans else "N").T
    np.testing.assert_allclose(got, ref, rtol=1e-9, atol=1e-10)


@pytest.mark.parametrize("shape", [(50, 50), (200, 60), (40, 90), (1500, 300), (130, 700)])
def test_qr_solver_least_squares_and_min_norm(dev, shape):
    m, n = shape
    rng = np.random.default_rng(m * n)
    a = rng.standard_normal((m, n))
    b = rng.standard_normal(m)
    op = lx.MatrixLinearOperator(t(a, dev))
    sol = lx.linear_solve(op, t(b, dev), lx.QR())
    x = sol.value.cpu().numpy()
    ref = dense.qr_linear_solve(a, b)
    np.testing.assert_allclose(x, ref, rtol=1e-9, atol=1e-10 * max(1.0, np.abs(ref).max()))
    lstsq = np.linalg.lstsq(a, b, rcond=None)[0]
    np.testing.assert_allclose(x, lstsq, rtol=1e-8, atol=1e-9)


def test_qr_auto_for_nonsquare_and_transpose_state(dev):
    rng = np.random.default_rng(5)
    a = rng.standard_normal((80, 30))
    op = lx.MatrixLinearOperator(t(a, dev))
    solver = lx.AutoLinearSolver(well_posed=None)
    assert isinstance(solver.select_solver(op), lx.QR)
    b = rng.standard_normal(80)
    x = lx.linear_solve(op, t(b, dev), solver).value.cpu().numpy()
    np.testing.assert_allclose(x, np.linalg.lstsq(a, b, rcond=None)[0], rtol=1e-8, atol=1e-9)
    qr = lx.QR()
    st = qr.init(op, {})
    st_t, _ = qr.transpose(st, {})
    c = rng.standard_normal(30)
    xt, _, _ = qr.compute(st_t, t(c, dev), {})
    np.testing.assert_allclose(xt.cpu().numpy(), np.linalg.lstsq(a.T, c, rcond=None)[0],
                               rtol=1e-8, atol=1e-9)


@pytest.mark.parametrize("name", ["pytree_2x2", "mixed_dtypes_2x2"])
def test_reference_kat_qr(dev, name):
    k = GOLD[name]
    sol = lx.linear_solve(lx.MatrixLinearOperator(t(k["matrix"], dev)), t(k["vector"], dev),
                          lx.QR())
    np.testing.assert_allclose(sol.value.cpu().numpy(), k["solution"], rtol=1e-14)


@pytest.mark.parametrize("m,n,k", [(4096, 512, 1), (2048, 300, 3), (1024, 256, 2), (1024, 130, 1)])
def test_mixed_precision_least_squares(dev, m, n, k):
    """TF32 tensor-core QR + corrected semi-normal equations: the FP64
    least-squares solution (Gaussian tall matrices, kappa ~ 2-3; the
    refinement contracts by about kappa^2 u_TF32 per step) and a factor whose
    R reproduces AᵀA to TF32 accuracy."""
    from lineax_gb300 import mixed
    rng = np.random.default_rng(m + n)
    a = rng.standard_normal((m, n))
    b = rng.standard_normal((k, m))
    res = mixed.qr_lstsq(torch.tensor(a, device=dev), torch.tensor(b, device=dev))
    assert res.converged and res.iters <= 6, (res.iters, res.step)
    x = res.x.cpu().numpy()
    for c in range(k):
        x_ref = np.linalg.lstsq(a, b[c], rcond=None)[0]
        assert np.abs(x[c] - x_ref).max() <= 1e-10 * np.abs(x_ref).max()
    f = mixed.qr_factor_tf32(torch.tensor(a, device=dev))
    r = np.tril(f.rt.cpu().numpy()).T          # R (upper)
    ata = a.T @ a
    assert np.abs(r.T @ r - ata).max() <= 2e-3 * np.abs(ata).max()


def test_mixed_qr_through_linear_solve(dev):
    import lineax_gb300 as lx
    rng = np.random.default_rng(4)
    a = rng.standard_normal((2048, 256))
    b = rng.standard_normal(2048)
    sol = lx.linear_solve(lx.MatrixLinearOperator(torch.tensor(a, device=dev)),
                          torch.tensor(b, device=dev), lx.QR(precision="mixed"))
    x_ref = np.linalg.lstsq(a, b, rcond=None)[0]
    assert sol.result == lx.RESULTS.successful
    assert np.abs(sol.value.cpu().numpy() - x_ref).max() <= 1e-10 * np.abs(x_ref).max()


@pytest.mark.parametrize("n", [256, 1000, 2048])
def test_square_tf32_qr_with_q_and_gmres_ir(dev, n):
    """TF32 Householder QR that also forms Q (lxgb_geqrf_f32_tc_q): Q is
    orthogonal and Q R reproduces A to TF32 accuracy; R^{-1} Qᵀ as the
    GMRES-IR preconditioner recovers FP64 backward error on a square system
    (the serving path of QR requests)."""
    from lineax_gb300 import mixed
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n)) / np.sqrt(n) + np.eye(n)
    b = rng.standard_normal((3, n))
    qr = mixed.qr_square_tf32(t(a, dev))
    qt = qr.qt.double().cpu().numpy()
    rinv = qr.rinv.double().cpu().numpy()
    # TF32 products (u = 2^-11): orthogonality and the factorisation hold to
    # a small multiple of u
    assert np.abs(qt @ qt.T - np.eye(n)).max() <= 2e-2
    assert np.all(np.tril(rinv, -1) == 0)
    r = np.linalg.inv(rinv)
    assert np.abs(qt.T @ r - a).max() <= 2e-2 * np.abs(a).max()
    res = mixed.gmres_ir(t(a, dev), t(b, dev), tol=1e-12, restart=8, inner_max_steps=5,
                         arith="auto", qr=qr, fallback=False)
    assert res.converged, res.berr
    x = res.x.cpu().numpy()
    be = dense.backward_errors_exact(a, x, b)
    assert (be <= 1e-12 * (1 + 1e-4)).all(), be
    # backward error 1e-12 bounds the forward error by about cond(A) 1e-12
    bound = 4 * np.linalg.cond(a) * 1e-12
    for c in range(3):
        assert dense.forward_error(x[c], dense.qr_linear_solve(a, b[c])) <= bound
