"""CPU: the oracle against the reference's own known answers (tests/golden)
and the C getf2 twin against SciPy's LAPACK."""

import json
import pathlib

import numpy as np
import pytest

from oracle import dense, krylov
from oracle.build import getf2_batched

GOLD = json.loads((pathlib.Path(__file__).parent / "golden" / "reference_kats.json").read_text())


@pytest.mark.parametrize("name", ["pytree_2x2", "mixed_dtypes_2x2"])
def test_oracle_lu_qr_kats(name):
    k = GOLD[name]
    a, b, x = np.array(k["matrix"]), np.array(k["vector"]), np.array(k["solution"])
    np.testing.assert_allclose(dense.lu_linear_solve(a, b), x, rtol=1e-14)
    np.testing.assert_allclose(dense.qr_linear_solve(a, b), x, rtol=1e-14)


def test_oracle_triangular_kat():
    k = GOLD["triangular_2x2"]
    a, b, x = np.array(k["matrix"]), np.array(k["vector"]), np.array(k["solution"])
    np.testing.assert_allclose(dense.triangular_solve(a, b, lower=True, unit_diagonal=False), x)


def test_oracle_gmres_reports_failure_on_reference_4x4():
    k = GOLD["gmres_fails_4x4"]
    a = np.array(k["matrix"])
    b = a @ np.array(k["true_x"])
    s = k["solver"]
    x, result, _ = krylov.gmres(lambda v: a @ v, b, rtol=s["rtol"], atol=s["atol"],
                                restart=s["restart"])
    assert krylov.finalize_result(x, result, b) != krylov.SUCCESSFUL


def test_oracle_nonfinite_input_kat():
    k = GOLD["nonfinite_input"]
    d = np.array(k["diagonal"])
    for v in k["vectors"]:
        v = np.array(v)
        x = v / d
        assert krylov.finalize_result(x, krylov.SUCCESSFUL, v) == 6


def test_getf2_twin_matches_lapack_pivots():
    rng = np.random.default_rng(1)
    for n in (1, 2, 7, 33, 128, 200):
        a = rng.standard_normal((n, n))
        lu, piv, info = getf2_batched(a)
        lu_ref, piv_ref = dense.lu_factor(a)
        assert info[0] == 0
        np.testing.assert_array_equal(piv[0], piv_ref)
        np.testing.assert_allclose(lu[0], lu_ref, rtol=0, atol=1e-11 * max(1, n))


def test_getf2_twin_zero_pivot_info():
    a = np.array([[0.0, 1.0], [0.0, 2.0]])
    _, piv, info = getf2_batched(a)
    assert info[0] == 1  # first column all zero: LAPACK reports info = 1


def test_oracle_cg_poisson_converges():
    n = 50
    p = -2 * np.eye(n) + np.eye(n, k=1) + np.eye(n, k=-1)
    a = -p  # positive definite
    b = np.random.default_rng(0).standard_normal(n)
    x, result, steps = krylov.cg(lambda v: a @ v, b, rtol=1e-10, atol=1e-10)
    assert result == krylov.SUCCESSFUL and steps <= n + 5
    assert dense.backward_error(a, x, b) < 1e-12


def test_oracle_gmres_dense_converges():
    rng = np.random.default_rng(0)
    a = rng.standard_normal((40, 40))
    xt = rng.standard_normal(40)
    b = a @ xt
    x, result, _ = krylov.gmres(lambda v: a @ v, b, rtol=1e-10, atol=1e-10, restart=40)
    assert result == krylov.SUCCESSFUL
    np.testing.assert_allclose(x, xt, rtol=1e-8, atol=1e-8)


def test_oracle_cg_max_steps_only_poisson():
    """tests/test_solve.py::test_iterative_solver_max_steps_only, CG leg."""
    n = 100
    p = -2 * np.eye(n) + np.eye(n, k=1) + np.eye(n, k=-1)
    b = np.random.default_rng(0).standard_normal(n)
    x, result, steps = krylov.cg(lambda v: p @ v, b, rtol=0.0, atol=0.0, max_steps=2, nsd=True)
    assert steps == 2 and result == krylov.SUCCESSFUL


def test_oracle_bicgstab_iterates_match_scipy():
    """The BiCGStab restatement against an independent implementation of the
    same published recurrence (SciPy's bicgstab, right-preconditioned): the
    iterate after k steps agrees (no stopping test involved: tolerances 0)."""
    from scipy.sparse.linalg import LinearOperator, bicgstab as sp_bicgstab

    rng = np.random.default_rng(5)
    n = 60
    a = rng.standard_normal((n, n)) / np.sqrt(n) + 3 * np.eye(n)
    b = rng.standard_normal(n)
    d = np.diag(a).copy()
    for k in (1, 3, 7):
        for pre in (None, lambda v: v / d):
            x, res, steps = krylov.bicgstab(lambda v: a @ v, b, rtol=0.0, atol=0.0, max_steps=k,
                                            precond=pre)
            m = None if pre is None else LinearOperator((n, n), matvec=pre)
            xs, _ = sp_bicgstab(a, b, x0=np.zeros(n), rtol=0.0, atol=0.0, maxiter=k, M=m)
            assert steps == k and res == krylov.SUCCESSFUL
            np.testing.assert_allclose(x, xs, rtol=1e-10, atol=1e-12)


def test_oracle_bicgstab_max_steps_only_poisson():
    """tests/test_solve.py::test_iterative_solver_max_steps_only, BiCGStab leg."""
    n = 100
    p = -2 * np.eye(n) + np.eye(n, k=1) + np.eye(n, k=-1)
    b = np.random.default_rng(0).standard_normal(n)
    x, result, steps = krylov.bicgstab(lambda v: p @ v, b, rtol=0.0, atol=0.0, max_steps=2)
    assert steps == 2 and result == krylov.SUCCESSFUL and np.all(np.isfinite(x))


def test_oracle_bicgstab_converges_and_flags_singular():
    rng = np.random.default_rng(1)
    n = 40
    a = rng.standard_normal((n, n)) / np.sqrt(n) + 2 * np.eye(n)
    xt = rng.standard_normal(n)
    x, result, _ = krylov.bicgstab(lambda v: a @ v, a @ xt, rtol=1e-10, atol=1e-10)
    assert result == krylov.SUCCESSFUL
    np.testing.assert_allclose(x, xt, rtol=1e-8, atol=1e-8)
    a[3] = 0.0  # a zero row, as the reference's singular-matrix tests build
    b = rng.standard_normal(n)
    x, result, _ = krylov.bicgstab(lambda v: a @ v, b, rtol=1e-10, atol=1e-10)
    assert krylov.finalize_result(x, result, b) != krylov.SUCCESSFUL


@pytest.mark.parametrize("name", ["nonsquare_wide_2x3", "nonsquare_tall_3x2"])
def test_oracle_nonsquare_kats(name):
    """tests/test_singular.py::test_nonsquare_pytree_operator1/2: QR and
    Normal(Cholesky()) return the least-squares / minimum-norm solution."""
    k = GOLD[name]
    a = np.array(k["matrix"])
    b = np.array(k["vector"])
    expect = np.linalg.lstsq(a, b, rcond=None)[0]
    np.testing.assert_allclose(dense.qr_linear_solve(a, b), expect, rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(dense.normal_linear_solve(a, b), expect, rtol=1e-10, atol=1e-12)


def test_oracle_cg_iterates_match_scipy():
    """The CG restatement against SciPy's independent implementation of the
    same preconditioned recurrence: equal iterates for k < stabilise_every
    steps (lineax replaces the residual at step 10; tolerances 0)."""
    from scipy.sparse.linalg import LinearOperator, cg as sp_cg

    rng = np.random.default_rng(7)
    n = 60
    g = rng.standard_normal((n, n))
    a = g @ g.T / n + 0.5 * np.eye(n)
    b = rng.standard_normal(n)
    d = np.diag(a).copy()
    for k in (1, 4, 9):
        for pre in (None, lambda v: v / d):
            x, res, steps = krylov.cg(lambda v: a @ v, b, rtol=0.0, atol=0.0, max_steps=k,
                                      precond=pre)
            m = None if pre is None else LinearOperator((n, n), matvec=pre)
            xs, _ = sp_cg(a, b, x0=np.zeros(n), rtol=0.0, atol=0.0, maxiter=k, M=m)
            assert steps == k and res == krylov.SUCCESSFUL
            np.testing.assert_allclose(x, xs, rtol=1e-10, atol=1e-12)


def test_oracle_gmres_cycle_matches_scipy():
    """One restart cycle of the GMRES restatement (after lineax's dummy first
    pass) gives the Krylov minimiser that SciPy's GMRES returns after one
    cycle of the same length."""
    from scipy.sparse.linalg import gmres as sp_gmres

    rng = np.random.default_rng(8)
    n = 50
    a = rng.standard_normal((n, n)) / np.sqrt(n) + 2 * np.eye(n)
    b = rng.standard_normal(n)
    for k in (3, 8, 20):
        x, res, steps = krylov.gmres(lambda v: a @ v, b, rtol=0.0, atol=0.0, max_steps=2,
                                     restart=k)
        xs, _ = sp_gmres(a, b, x0=np.zeros(n), rtol=0.0, atol=0.0, restart=k, maxiter=1)
        assert steps == 2 and res == krylov.SUCCESSFUL
        np.testing.assert_allclose(x, xs, rtol=1e-9, atol=1e-11)


def test_residual_exact_against_rational_arithmetic():
    """oracle.dense.residual_exact: B - X Aᵀ to within 2^-70 of |X||A|ᵀ,
    checked against exact rational arithmetic on a small case with a wide
    dynamic range (products that cancel in FP64)."""
    from fractions import Fraction

    rng = np.random.default_rng(5)
    n, k = 24, 3
    a = rng.standard_normal((n, n)) * np.exp2(rng.integers(-30, 30, (n, n)))
    x = rng.standard_normal((k, n))
    b = x @ a.T  # b close to A x, so the residual is all cancellation
    r = dense.residual_exact(a, x, b)
    scale = np.abs(x) @ np.abs(a).T
    for c in range(k):
        for i in range(n):
            exact = Fraction(b[c, i]) - sum(Fraction(a[i, j]) * Fraction(x[c, j])
                                            for j in range(n))
            assert abs(Fraction(r[c, i]) - exact) <= Fraction(scale[c, i]) / 2 ** 70
    be = dense.backward_errors_exact(a, x, b)
    assert be.shape == (k,) and (be >= 0).all() and (be < 1e-15).all()
