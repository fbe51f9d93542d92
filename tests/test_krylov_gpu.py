"""GPU parity: CG, GMRES and BiCGStab (device Krylov engine) against the NumPy
restatements of lineax's loops, including the reference's failure case."""

import json
import pathlib

import numpy as np
import pytest
import torch

import lineax_gb300 as lx
from lineax_gb300 import _krylov
from oracle import dense, krylov

pytestmark = pytest.mark.gpu
GOLD = json.loads((pathlib.Path(__file__).parent / "golden" / "reference_kats.json").read_text())


def t(x, dev):
    return torch.tensor(np.asarray(x), dtype=torch.float64, device=dev)


def spd(rng, n, cond_shift=1.0):
    g = rng.standard_normal((n, n))
    return g @ g.T / n + cond_shift * np.eye(n)


def poisson2d(nx, ny):
    def one(m):
        return 2 * np.eye(m) - np.eye(m, k=1) - np.eye(m, k=-1)
    return np.kron(one(nx), np.eye(ny)) + np.kron(np.eye(nx), one(ny))


@pytest.mark.parametrize("n,tol", [(10, 1e-10), (60, 1e-10), (150, 1e-12)])
def test_cg_dense_matches_oracle(dev, n, tol):
    rng = np.random.default_rng(n)
    a = spd(rng, n, 0.1)
    b = rng.standard_normal(n)
    op = lx.MatrixLinearOperator(t(a, dev), lx.positive_semidefinite_tag)
    sol = lx.linear_solve(op, t(b, dev), lx.CG(rtol=tol, atol=tol))
    x_ref, res_ref, steps_ref = krylov.cg(lambda v: a @ v, b, rtol=tol, atol=tol)
    assert sol.result == res_ref == 0
    assert abs(sol.stats["num_steps"] - steps_ref) <= 1
    np.testing.assert_allclose(sol.value.cpu().numpy(), x_ref, rtol=1e-8, atol=1e-10)
    assert dense.backward_error(a, sol.value.cpu().numpy(), b) < 1e-9


def test_cg_nsd_and_max_steps_only(dev):
    """tests/test_solve.py::test_iterative_solver_max_steps_only (CG leg):
    NSD-tagged 1-D Poisson, rtol = atol = 0, max_steps = 2."""
    n = 100
    p = -2 * np.eye(n) + np.eye(n, k=1) + np.eye(n, k=-1)
    b = np.random.default_rng(0).standard_normal(n)
    op = lx.MatrixLinearOperator(t(p, dev), (lx.negative_semidefinite_tag, lx.symmetric_tag))
    sol = lx.linear_solve(op, t(b, dev), lx.CG(0.0, 0.0, max_steps=2))
    x_ref, res_ref, steps_ref = krylov.cg(lambda v: p @ v, b, rtol=0.0, atol=0.0, max_steps=2,
                                          nsd=True)
    assert sol.stats["num_steps"] == steps_ref == 2 and sol.result == res_ref
    np.testing.assert_allclose(sol.value.cpu().numpy(), x_ref, rtol=1e-10, atol=1e-12)


def test_cg_preconditioned(dev):
    rng = np.random.default_rng(4)
    n = 80
    a = spd(rng, n, 0.05) * np.outer(np.linspace(1, 5, n), np.linspace(1, 5, n))
    b = rng.standard_normal(n)
    m = np.diag(1.0 / np.diag(a))
    op = lx.MatrixLinearOperator(t(a, dev), lx.positive_semidefinite_tag)
    pre = lx.MatrixLinearOperator(t(m, dev), lx.positive_semidefinite_tag)
    sol = lx.linear_solve(op, t(b, dev), lx.CG(rtol=1e-10, atol=1e-10),
                          options={"preconditioner": pre})
    x_ref, res_ref, steps_ref = krylov.cg(lambda v: a @ v, b, rtol=1e-10, atol=1e-10,
                                          precond=lambda v: m @ v)
    assert sol.result == res_ref and abs(sol.stats["num_steps"] - steps_ref) <= 1
    np.testing.assert_allclose(sol.value.cpu().numpy(), x_ref, rtol=1e-7, atol=1e-9)


def test_cg_poisson_stencil_block(dev):
    """Matrix-free 5-point Poisson, 4 right-hand sides at once: each equals
    the oracle run alone, and the block equals the single-RHS runs bit for bit."""
    nx, ny, k = 24, 20, 4
    rng = np.random.default_rng(8)
    b = rng.standard_normal((k, nx * ny))
    a = poisson2d(nx, ny)
    op = lx.Poisson2DOperator(nx, ny)
    np.testing.assert_allclose(op.mv(t(b[0], dev)).cpu().numpy(), a @ b[0], rtol=1e-14)
    res = _krylov.cg_block(op, t(b, dev), rtol=1e-10, atol=1e-10)
    y = res.y.cpu().numpy()
    for c in range(k):
        x_ref, r_ref, s_ref = krylov.cg(lambda v: a @ v, b[c], rtol=1e-10, atol=1e-10)
        assert res.results[c] == r_ref and abs(res.steps[c] - s_ref) <= 1
        np.testing.assert_allclose(y[c], x_ref, rtol=1e-7, atol=1e-9)
        alone = _krylov.cg_block(op, t(b[c:c + 1], dev), rtol=1e-10, atol=1e-10)
        assert torch.equal(alone.y[0], res.y[c]) and alone.steps[0] == res.steps[c]


def test_gmres_large_dense_reference_pattern(dev):
    """tests/test_solve.py::test_gmres_large_dense: 100×100, restart=100, tol 1e-10."""
    rng = np.random.default_rng(1)
    a = rng.standard_normal((100, 100))
    xt = rng.standard_normal(100)
    b = a @ xt
    sol = lx.linear_solve(lx.MatrixLinearOperator(t(a, dev)), t(b, dev),
                          lx.GMRES(atol=1e-10, rtol=1e-10, restart=100))
    np.testing.assert_allclose(sol.value.cpu().numpy(), xt, rtol=1e-8, atol=1e-8)
    x_ref, res_ref, steps_ref = krylov.gmres(lambda v: a @ v, b, rtol=1e-10, atol=1e-10,
                                             restart=100)
    assert sol.result == res_ref == 0 and abs(sol.stats["num_steps"] - steps_ref) <= 1


@pytest.mark.parametrize("n,restart", [(30, 20), (200, 20), (64, 8)])
def test_gmres_matches_oracle(dev, n, restart):
    rng = np.random.default_rng(n + restart)
    a = rng.standard_normal((n, n)) / np.sqrt(n) + 1.5 * np.eye(n)
    b = rng.standard_normal(n)
    sol = lx.linear_solve(lx.MatrixLinearOperator(t(a, dev)), t(b, dev),
                          lx.GMRES(rtol=1e-10, atol=1e-10, restart=restart), throw=False)
    x_ref, res_ref, steps_ref = krylov.gmres(lambda v: a @ v, b, rtol=1e-10, atol=1e-10,
                                             restart=restart)
    assert sol.result == res_ref
    assert abs(sol.stats["num_steps"] - steps_ref) <= 1
    np.testing.assert_allclose(sol.value.cpu().numpy(), x_ref, rtol=1e-7, atol=1e-9)


def test_gmres_reference_failure_case(dev):
    """tests/test_singular.py::test_gmres_stagnation_or_breakdown: restart=2 on the
    literal 4×4 must report failure."""
    k = GOLD["gmres_fails_4x4"]
    a = np.array(k["matrix"])
    b = a @ np.array(k["true_x"])
    s = k["solver"]
    sol = lx.linear_solve(lx.MatrixLinearOperator(t(a, dev)), t(b, dev),
                          lx.GMRES(rtol=s["rtol"], atol=s["atol"], restart=s["restart"]),
                          throw=False)
    assert sol.result != lx.RESULTS.successful
    x_ref, res_ref, _ = krylov.gmres(lambda v: a @ v, b, rtol=s["rtol"], atol=s["atol"],
                                     restart=s["restart"])
    assert sol.result == krylov.finalize_result(x_ref, res_ref, b)


def test_gmres_preconditioned_block_equals_alone(dev):
    rng = np.random.default_rng(12)
    n, k = 120, 3
    a = rng.standard_normal((n, n)) / np.sqrt(n) + np.diag(np.linspace(1, 10, n))
    m = np.diag(1.0 / np.diag(a))
    b = rng.standard_normal((k, n))
    op = lx.MatrixLinearOperator(t(a, dev))
    pre = lx.MatrixLinearOperator(t(m, dev))
    res = _krylov.gmres_block(op, t(b, dev), rtol=1e-10, atol=1e-10, preconditioner=pre)
    for c in range(k):
        x_ref, r_ref, s_ref = krylov.gmres(lambda v: a @ v, b[c], rtol=1e-10, atol=1e-10,
                                           precond=lambda v: m @ v)
        assert res.results[c] == r_ref and abs(res.steps[c] - s_ref) <= 1
        np.testing.assert_allclose(res.y[c].cpu().numpy(), x_ref, rtol=1e-7, atol=1e-9)
        alone = _krylov.gmres_block(op, t(b[c:c + 1], dev), rtol=1e-10, atol=1e-10,
                                    preconditioner=pre)
        assert torch.equal(alone.y[0], res.y[c])


def test_cg_nonfinite_input_matches_reference(dev):
    """With a NaN right-hand side lineax's CG never enters its loop (gamma0 =
    NaN fails gamma > 0, cg.py:164) and returns the finite y0, so the result is
    `successful`; a LU solve of the same system reports nonfinite_input."""
    n = 5
    a = np.eye(n) * 2
    b = np.ones(n)
    b[2] = np.nan
    op = lx.MatrixLinearOperator(t(a, dev), lx.positive_semidefinite_tag)
    sol = lx.linear_solve(op, t(b, dev), lx.CG(rtol=1e-8, atol=1e-8), throw=False)
    x_ref, r_ref, s_ref = krylov.cg(lambda v: a @ v, b, rtol=1e-8, atol=1e-8)
    assert sol.result == krylov.finalize_result(x_ref, r_ref, b) == lx.RESULTS.successful
    assert sol.stats["num_steps"] == s_ref == 0
    sol = lx.linear_solve(lx.MatrixLinearOperator(t(a, dev)), t(b, dev), lx.LU(), throw=False)
    assert sol.result == lx.RESULTS.nonfinite_input


@pytest.mark.parametrize("nx,ny,k", [(48, 40, 4), (130, 70, 3)])
def test_cg_mixed_precision_poisson(dev, nx, ny, k):
    """FP32 iterations with FP64 residual replacement: every right-hand side
    ends on lineax's stopping test applied to the FP64 true residual, close to
    the FP64 restatement's solution, and independent of the other right-hand
    sides of the block."""
    rng = np.random.default_rng(nx + ny)
    b = rng.standard_normal((k, nx * ny))
    a = poisson2d(nx, ny)
    op = lx.Poisson2DOperator(nx, ny)
    res = _krylov.cg_poisson_mixed(op, t(b, dev), rtol=1e-10, atol=1e-10)
    y = res.y.cpu().numpy()
    for c in range(k):
        assert res.results[c] == 0
        r = b[c] - a @ y[c]
        assert np.all(np.abs(r) <= 1e-10 + 1e-10 * np.abs(b[c]))
        x_ref, r_ref, s_ref = krylov.cg(lambda v: a @ v, b[c], rtol=1e-10, atol=1e-10)
        np.testing.assert_allclose(y[c], x_ref, rtol=1e-6, atol=1e-8)
        assert res.steps[c] <= 2 * s_ref + 16
        alone = _krylov.cg_poisson_mixed(op, t(b[c:c + 1], dev), rtol=1e-10, atol=1e-10)
        assert torch.equal(alone.y[0], res.y[c]) and alone.steps[0] == res.steps[c]
    # through the solver API, and a max_steps cap
    sol = lx.linear_solve(op, t(b[0], dev), lx.CG(rtol=1e-10, atol=1e-10, precision="mixed"))
    assert sol.result == lx.RESULTS.successful
    capped = _krylov.cg_poisson_mixed(op, t(b, dev), rtol=1e-10, atol=1e-10, max_steps=16)
    assert all(s == 16 for s in capped.steps) and all(r_ == 1 for r_ in capped.results)


def nonsym(rng, n, shift=2.0):
    return rng.standard_normal((n, n)) / np.sqrt(n) + shift * np.eye(n)


@pytest.mark.parametrize("n,tol", [(10, 1e-10), (60, 1e-10), (150, 1e-12)])
def test_bicgstab_matches_oracle(dev, n, tol):
    rng = np.random.default_rng(100 + n)
    a = nonsym(rng, n)
    b = rng.standard_normal(n)
    op = lx.MatrixLinearOperator(t(a, dev))
    sol = lx.linear_solve(op, t(b, dev), lx.BiCGStab(rtol=tol, atol=tol))
    x_ref, res_ref, steps_ref = krylov.bicgstab(lambda v: a @ v, b, rtol=tol, atol=tol)
    assert sol.result == res_ref == 0
    assert abs(sol.stats["num_steps"] - steps_ref) <= 1
    np.testing.assert_allclose(sol.value.cpu().numpy(), x_ref, rtol=1e-8, atol=1e-10)
    assert dense.backward_error(a, sol.value.cpu().numpy(), b) < 1e-9


def test_bicgstab_max_steps_only(dev):
    """tests/test_solve.py::test_iterative_solver_max_steps_only (BiCGStab
    leg): NSD-tagged 1-D Poisson, rtol = atol = 0, max_steps = 2."""
    n = 100
    p = -2 * np.eye(n) + np.eye(n, k=1) + np.eye(n, k=-1)
    b = np.random.default_rng(0).standard_normal(n)
    op = lx.MatrixLinearOperator(t(p, dev), (lx.negative_semidefinite_tag, lx.symmetric_tag))
    sol = lx.linear_solve(op, t(b, dev), lx.BiCGStab(0.0, 0.0, max_steps=2))
    x_ref, res_ref, steps_ref = krylov.bicgstab(lambda v: p @ v, b, rtol=0.0, atol=0.0,
                                                max_steps=2)
    assert sol.stats["num_steps"] == steps_ref == 2 and sol.result == res_ref
    np.testing.assert_allclose(sol.value.cpu().numpy(), x_ref, rtol=1e-10, atol=1e-12)


def test_bicgstab_preconditioned_block_equals_alone(dev):
    rng = np.random.default_rng(14)
    n, k = 120, 3
    a = rng.standard_normal((n, n)) / np.sqrt(n) + np.diag(np.linspace(1, 10, n))
    m = np.diag(1.0 / np.diag(a))
    b = rng.standard_normal((k, n))
    op = lx.MatrixLinearOperator(t(a, dev))
    pre = lx.MatrixLinearOperator(t(m, dev))
    res = _krylov.bicgstab_block(op, t(b, dev), rtol=1e-10, atol=1e-10, preconditioner=pre)
    for c in range(k):
        x_ref, r_ref, s_ref = krylov.bicgstab(lambda v: a @ v, b[c], rtol=1e-10, atol=1e-10,
                                              precond=lambda v: m @ v)
        assert res.results[c] == r_ref and abs(res.steps[c] - s_ref) <= 1
        np.testing.assert_allclose(res.y[c].cpu().numpy(), x_ref, rtol=1e-7, atol=1e-9)
        alone = _krylov.bicgstab_block(op, t(b[c:c + 1], dev), rtol=1e-10, atol=1e-10,
                                       preconditioner=pre)
        assert torch.equal(alone.y[0], res.y[c]) and alone.steps[0] == res.steps[c]


def test_bicgstab_y0_and_transpose(dev):
    rng = np.random.default_rng(15)
    n = 80
    a = nonsym(rng, n)
    b = rng.standard_normal(n)
    y0 = rng.standard_normal(n)
    op = lx.MatrixLinearOperator(t(a, dev))
    sol = lx.linear_solve(op, t(b, dev), lx.BiCGStab(1e-11, 1e-11), options={"y0": t(y0, dev)})
    x_ref, r_ref, s_ref = krylov.bicgstab(lambda v: a @ v, b, rtol=1e-11, atol=1e-11, y0=y0)
    assert sol.result == r_ref == 0 and abs(sol.stats["num_steps"] - s_ref) <= 1
    np.testing.assert_allclose(sol.value.cpu().numpy(), x_ref, rtol=1e-8, atol=1e-10)
    solver = lx.BiCGStab(1e-11, 1e-11)
    state = solver.init(op, {})
    tstate, topts = solver.transpose(state, {})
    xt, rt, _ = solver.compute(tstate, t(b, dev), topts)
    assert rt == 0
    assert dense.backward_error(a.T, xt.cpu().numpy(), b) < 1e-9


def test_bicgstab_singular_reports_failure(dev):
    """A zero row (the reference's singular-matrix construction for Krylov
    solvers): the solve does not report success, as in the oracle."""
    rng = np.random.default_rng(16)
    n = 30
    a = nonsym(rng, n)
    a[7] = 0.0
    b = rng.standard_normal(n)
    op = lx.MatrixLinearOperator(t(a, dev))
    sol = lx.linear_solve(op, t(b, dev), lx.BiCGStab(1e-10, 1e-10), throw=False)
    x_ref, r_ref, _ = krylov.bicgstab(lambda v: a @ v, b, rtol=1e-10, atol=1e-10)
    assert krylov.finalize_result(x_ref, r_ref, b) != 0
    assert sol.result != lx.RESULTS.successful
