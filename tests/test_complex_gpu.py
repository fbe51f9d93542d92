"""GPU: complex128 operators and vectors through linear_solve, every solver,
against NumPy/LAPACK complex solutions (lineax runs its well-posed tests on
complex128 too: tests/test_well_posed.py:33-52, tolerance 1e-10 against the
true solution)."""

import numpy as np
import pytest
import torch

import lineax_gb300 as lx

pytestmark = pytest.mark.gpu
TOL = 1e-10


def c(x, dev):
    return torch.tensor(np.asarray(x), dtype=torch.complex128, device=dev)


def crandn(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def ferr(x, ref):
    x = x.cpu().numpy() if isinstance(x, torch.Tensor) else x
    return float(np.abs(x - ref).max() / max(np.abs(ref).max(), 1e-300))


def hpd(rng, n):
    g = crandn(rng, n, n)
    return g @ g.conj().T / n + np.eye(n)


@pytest.mark.parametrize("n", [1, 7, 64, 300])
def test_complex_lu(dev, n):
    rng = np.random.default_rng(n)
    a = crandn(rng, n, n) / np.sqrt(n) + 2 * np.eye(n)
    b = crandn(rng, n)
    sol = lx.linear_solve(lx.MatrixLinearOperator(c(a, dev)), c(b, dev), lx.LU())
    assert sol.value.dtype == torch.complex128
    assert ferr(sol.value, np.linalg.solve(a, b)) <= TOL
    # the returned state solves another right-hand side without refactorising
    b2 = crandn(rng, n)
    sol2 = lx.linear_solve(lx.MatrixLinearOperator(c(a, dev)), c(b2, dev), lx.LU(),
                           state=sol.state)
    assert ferr(sol2.value, np.linalg.solve(a, b2)) <= TOL


@pytest.mark.parametrize("nsd", [False, True])
def test_complex_cholesky_hermitian(dev, nsd):
    rng = np.random.default_rng(5)
    n = 96
    a = hpd(rng, n) * (-1 if nsd else 1)
    b = crandn(rng, n)
    tag = lx.negative_semidefinite_tag if nsd else lx.positive_semidefinite_tag
    op = lx.MatrixLinearOperator(c(a, dev), tag)
    sol = lx.linear_solve(op, c(b, dev), lx.Cholesky())
    assert ferr(sol.value, np.linalg.solve(a, b)) <= TOL
    # AutoLinearSolver picks Cholesky for the Hermitian definite operator
    auto = lx.linear_solve(op, c(b, dev))
    assert ferr(auto.value, np.linalg.solve(a, b)) <= TOL


@pytest.mark.parametrize("m,n", [(80, 80), (160, 50), (40, 90)])
def test_complex_qr(dev, m, n):
    rng = np.random.default_rng(m + n)
    a = crandn(rng, m, n)
    b = crandn(rng, m)
    sol = lx.linear_solve(lx.MatrixLinearOperator(c(a, dev)), c(b, dev), lx.QR())
    ref = np.linalg.lstsq(a, b, rcond=None)[0]   # least squares / minimum norm
    assert ferr(sol.value, ref) <= TOL


@pytest.mark.parametrize("lower,unit", [(True, False), (False, False), (True, True),
                                        (False, True)])
def test_complex_triangular(dev, lower, unit):
    rng = np.random.default_rng(11)
    n = 120
    t = crandn(rng, n, n) / np.sqrt(n)
    t = np.tril(t) if lower else np.triu(t)
    np.fill_diagonal(t, 1.0 if unit else 2.0 + crandn(rng, n))
    b = crandn(rng, n)
    tags = [lx.lower_triangular_tag if lower else lx.upper_triangular_tag]
    if unit:
        tags.append(lx.unit_diagonal_tag)
    op = lx.MatrixLinearOperator(c(t, dev), tags)
    sol = lx.linear_solve(op, c(b, dev), lx.Triangular())
    assert ferr(sol.value, np.linalg.solve(t, b)) <= TOL


def test_complex_diagonal(dev):
    rng = np.random.default_rng(2)
    d = crandn(rng, 50)
    b = crandn(rng, 50)
    op = lx.MatrixLinearOperator(c(np.diag(d), dev), lx.diagonal_tag)
    sol = lx.linear_solve(op, c(b, dev))      # AutoLinearSolver -> Diagonal
    assert ferr(sol.value, b / d) <= 1e-14


def test_complex_krylov(dev):
    rng = np.random.default_rng(9)
    n = 120
    a = hpd(rng, n)
    b = crandn(rng, n)
    ref = np.linalg.solve(a, b)
    op = lx.MatrixLinearOperator(c(a, dev), lx.positive_semidefinite_tag)
    cg = lx.linear_solve(op, c(b, dev), lx.CG(rtol=1e-13, atol=1e-13))
    assert ferr(cg.value, ref) <= 1e-9
    g = crandn(rng, n, n) / np.sqrt(n) + 3 * np.eye(n)
    ref_g = np.linalg.solve(g, b)
    gm = lx.linear_solve(lx.MatrixLinearOperator(c(g, dev)), c(b, dev),
                         lx.GMRES(rtol=1e-13, atol=1e-13, restart=40))
    assert ferr(gm.value, ref_g) <= 1e-9
    bi = lx.linear_solve(lx.MatrixLinearOperator(c(g, dev)), c(b, dev),
                         lx.BiCGStab(rtol=1e-13, atol=1e-13))
    assert ferr(bi.value, ref_g) <= 1e-9


def test_complex_normal_and_function_operator(dev):
    rng = np.random.default_rng(4)
    m, n = 150, 60
    a = crandn(rng, m, n)
    b = crandn(rng, m)
    ref = np.linalg.lstsq(a, b, rcond=None)[0]
    sol = lx.linear_solve(lx.MatrixLinearOperator(c(a, dev)), c(b, dev), lx.Normal(lx.Cholesky()))
    assert ferr(sol.value, ref) <= 1e-9
    # a FunctionLinearOperator over complex vectors: materialised (batched)
    # for LU, applied through its real form for GMRES
    sq = crandn(rng, n, n) / np.sqrt(n) + 3 * np.eye(n)
    at = c(sq, dev)
    fop = lx.FunctionLinearOperator(lambda x: at @ x,
                                    lx.ShapeDtypeStruct((n,), torch.complex128))
    assert torch.allclose(lx.materialise(fop).as_matrix(), at)
    bb = crandn(rng, n)
    ref2 = np.linalg.solve(sq, bb)
    assert ferr(lx.linear_solve(fop, c(bb, dev), lx.LU()).value, ref2) <= TOL
    assert ferr(lx.linear_solve(fop, c(bb, dev), lx.GMRES(rtol=1e-13, atol=1e-13)).value,
                ref2) <= 1e-9
    # MatrixLinearOperator.mv on complex vectors
    x = crandn(rng, n)
    assert ferr(lx.MatrixLinearOperator(at).mv(c(x, dev)), sq @ x) <= 1e-13


def test_complex_singular_reports(dev):
    a = np.zeros((4, 4), dtype=np.complex128)
    a[0, 0] = 1.0
    sol = lx.linear_solve(lx.MatrixLinearOperator(c(a, dev)), c(np.ones(4), dev), lx.LU(),
                          throw=False)
    assert sol.result == lx.RESULTS.singular
