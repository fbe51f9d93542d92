"""GPU parity: LU, Cholesky, Triangular and Diagonal solves through the C ABI
against the CPU oracle (SciPy LAPACK and the bit-exact getf2 twin)."""

import json
import pathlib

import numpy as np
import pytest
import torch

import lineax_gb300 as lx
from lineax_gb300 import _dense, batched
from oracle import dense
from oracle.build import getf2_batched

pytestmark = pytest.mark.gpu
GOLD = json.loads((pathlib.Path(__file__).parent / "golden" / "reference_kats.json").read_text())
TOL = 1e-12  # normwise backward error bound for every FP64 solve


def t(x, dev):
    return torch.tensor(np.asarray(x), dtype=torch.float64, device=dev)


@pytest.mark.parametrize("n", [1, 2, 3, 17, 32, 64, 100, 128, 168, 169, 200, 333, 512])
def test_getrf_bit_exact_vs_getf2_twin(dev, n):
    """The plain FP64 LU equals the getf2 recurrence bit for bit, on both the
    shared-memory path (n <= 168) and the blocked path."""
    rng = np.random.default_rng(n)
    batch = 3 if n <= 168 else 1
    a = rng.standard_normal((batch, n, n)) / np.sqrt(n) + np.eye(n)
    lu, piv, info = _dense.lu_factor_batched(t(a, dev))
    lu_ref, piv_ref, info_ref = getf2_batched(a)
    np.testing.assert_array_equal(piv.cpu().numpy(), piv_ref)
    np.testing.assert_array_equal(info.cpu().numpy(), info_ref)
    assert np.array_equal(lu.cpu().numpy(), lu_ref), np.max(np.abs(lu.cpu().numpy() - lu_ref))


@pytest.mark.parametrize("n,batch", [(128, 64), (33, 5), (167, 7), (168, 76)])
def test_getrf_pair_cluster_bit_exact(dev, n, batch):
    """With the switch on, batches of at most half the SM count run on two-CTA
    clusters (columns split by parity between the CTAs): factors, pivots and
    info equal the getf2 twin bit for bit, and equal the one-CTA kernel's."""
    from lineax_gb300 import _ffi

    rng = np.random.default_rng(n * 1000 + batch)
    a = rng.standard_normal((batch, n, n)) / np.sqrt(n) + np.eye(n)
    lu1, piv1, info1 = _dense.lu_factor_batched(t(a, dev))
    try:
        _ffi.call("lxgb_getrf_set_pair", 1)
        lu, piv, info = _dense.lu_factor_batched(t(a, dev))
    finally:
        _ffi.call("lxgb_getrf_set_pair", 0)
    lu_ref, piv_ref, info_ref = getf2_batched(a)
    np.testing.assert_array_equal(piv.cpu().numpy(), piv_ref)
    np.testing.assert_array_equal(info.cpu().numpy(), info_ref)
    assert np.array_equal(lu.cpu().numpy(), lu_ref)
    assert torch.equal(lu1, lu) and torch.equal(piv1, piv) and torch.equal(info1, info)


def test_getrf_pair_cluster_singular_and_nan(dev):
    """Zero pivots found by either CTA of the pair (info = the first one) and a
    column of NaNs, against the getf2 twin, on both kernels."""
    from lineax_gb300 import _ffi

    rng = np.random.default_rng(5)
    n = 64
    a = rng.standard_normal((4, n, n)) + np.eye(n)
    a[0, :, 10] = 0.0                   # zero column owned by CTA 0 (even)
    a[1, :, 37] = 0.0                   # zero column owned by CTA 1 (odd)
    a[2, :, 5] = 0.0
    a[2, :, 20] = 0.0                   # two zero columns: info is the first
    a[3, :, 12] = np.nan
    lu_ref, piv_ref, info_ref = getf2_batched(a)
    assert list(info_ref[:3]) == [11, 38, 6]
    for pair in (1, 0):
        try:
            _ffi.call("lxgb_getrf_set_pair", pair)
            lu, piv, info = _dense.lu_factor_batched(t(a, dev))
        finally:
            _ffi.call("lxgb_getrf_set_pair", 0)
        np.testing.assert_array_equal(info.cpu().numpy(), info_ref)
        np.testing.assert_array_equal(piv.cpu().numpy(), piv_ref)
        got = lu.cpu().numpy()
        assert np.array_equal(np.isnan(got), np.isnan(lu_ref))
        assert np.array_equal(np.nan_to_num(got), np.nan_to_num(lu_ref))


def test_getrf_pivots_match_lapack_config1(dev):
    """64 systems, n = 128, A = G/sqrt(n) + I: pivots equal LAPACK dgetrf's."""
    rng = np.random.default_rng(2024)
    n = 128
    a = rng.standard_normal((64, n, n)) / np.sqrt(n) + np.eye(n)
    _, piv, _ = _dense.lu_factor_batched(t(a, dev))
    piv = piv.cpu().numpy()
    for s in range(64):
        np.testing.assert_array_equal(piv[s], dense.lu_factor(a[s])[1])


def test_getrf_zero_pivot_info(dev):
    a = np.array([[[0.0, 1.0, 2.0], [0.0, 3.0, 4.0], [0.0, 5.0, 7.0]]])
    _, _, info = _dense.lu_factor_batched(t(a, dev))
    assert int(info[0]) == 1


@pytest.mark.parametrize("n,nrhs,trans", [(5, 1, 0), (64, 3, 1), (128, 1, 0), (300, 2, 1),
                                          (777, 4, 0), (33, 9, 0), (160, 11, 1), (168, 2, 0)])
def test_lu_solve_backward_error(dev, n, nrhs, trans):
    rng = np.random.default_rng(7 + n)
    a = rng.standard_normal((n, n)) / np.sqrt(n) + np.eye(n)
    b = rng.standard_normal((nrhs, n))
    lu, piv = _dense.lu_factor(t(a, dev))
    x = _dense.lu_solve(lu, piv, t(b, dev), trans=trans).cpu().numpy()
    at = a.T if trans else a
    for k in range(nrhs):
        ref = dense.lu_linear_solve(a, b[k], transpose=bool(trans))
        assert dense.backward_error(at, x[k], b[k]) <= TOL
        assert dense.forward_error(x[k], ref) <= 1e-10


def test_lu_batched_config1(dev):
    rng = np.random.default_rng(11)
    n = 128
    a = rng.standard_normal((64, n, n)) / np.sqrt(n) + np.eye(n)
    b = rng.standard_normal((64, n))
    x, info = batched.lu_solve_batched(t(a, dev), t(b, dev))
    x = x.cpu().numpy()
    assert int(info.abs().sum()) == 0
    for s in range(64):
        assert dense.backward_error(a[s], x[s], b[s]) <= TOL


@pytest.mark.parametrize("name", ["pytree_2x2", "mixed_dtypes_2x2"])
def test_reference_kat_lu_and_auto(dev, name):
    k = GOLD[name]
    op = lx.MatrixLinearOperator(t(k["matrix"], dev))
    for solver in (lx.LU(), None):
        sol = lx.linear_solve(op, t(k["vector"], dev), solver)
        np.testing.assert_allclose(sol.value.cpu().numpy(), k["solution"], rtol=1e-14)


def test_reference_kat_triangular(dev):
    k = GOLD["triangular_2x2"]
    op = lx.MatrixLinearOperator(t(k["matrix"], dev), lx.lower_triangular_tag)
    sol = lx.linear_solve(op, t(k["vector"], dev), lx.Triangular())
    np.testing.assert_allclose(sol.value.cpu().numpy(), k["solution"], rtol=1e-14)


def test_reference_kat_nonfinite_input(dev):
    k = GOLD["nonfinite_input"]
    op = lx.MatrixLinearOperator(torch.diag(t(k["diagonal"], dev)), lx.diagonal_tag)
    for v in k["vectors"]:
        sol = lx.linear_solve(op, t(v, dev), throw=False)
        assert sol.result == lx.RESULTS.nonfinite_input


@pytest.mark.parametrize("lower", [True, False])
@pytest.mark.parametrize("unit", [True, False])
@pytest.mark.parametrize("trans", [False, True])
@pytest.mark.parametrize("n", [1, 31, 70, 257, 768, 1500])
def test_triangular_all_flags(dev, lower, unit, trans, n):
    rng = np.random.default_rng(n + 10 * lower + 100 * unit)
    m = rng.standard_normal((n, n)) / np.sqrt(n) + 2 * np.eye(n)
    m = np.tril(m) if lower else np.triu(m)
    b = rng.standard_normal(n)
    tags = [lx.lower_triangular_tag if lower else lx.upper_triangular_tag]
    if unit:
        tags.append(lx.unit_diagonal_tag)
    op = lx.MatrixLinearOperator(t(m, dev), tags)
    solver = lx.Triangular()
    state = solver.init(op, {})
    if trans:
        state, _ = solver.transpose(state, {})
    x, res, _ = solver.compute(state, t(b, dev), {})
    ref = dense.triangular_solve(m, b, lower=lower, unit_diagonal=unit, transpose=trans)
    np.testing.assert_allclose(x.cpu().numpy(), ref, rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("nsd", [False, True])
@pytest.mark.parametrize("n", [1, 5, 64, 160, 161, 300, 800, 1300])
def test_cholesky_solver(dev, n, nsd):
    rng = np.random.default_rng(n)
    g = rng.standard_normal((n, n))
    a = g @ g.T / n + 0.1 * np.eye(n)
    if nsd:
        a = -a
    b = rng.standard_normal(n)
    tag = lx.negative_semidefinite_tag if nsd else lx.positive_semidefinite_tag
    op = lx.MatrixLinearOperator(t(a, dev), tag)
    sol = lx.linear_solve(op, t(b, dev))  # Auto -> Cholesky (Diagonal when 1x1)
    expected = lx.Diagonal if n == 1 else lx.Cholesky
    assert isinstance(lx.AutoLinearSolver(well_posed=True).select_solver(op), expected)
    sol = lx.linear_solve(op, t(b, dev), lx.Cholesky())
    x = sol.value.cpu().numpy()
    assert dense.backward_error(a, x, b) <= TOL
    u = sol.state[0].cpu().numpy()
    u_ref = dense.cho_factor_upper(a, nsd)
    np.testing.assert_allclose(u, u_ref, rtol=1e-10, atol=1e-12)


def test_cholesky_not_pd_is_singular(dev):
    a = np.diag([1.0, -1.0, 2.0])
    op = lx.MatrixLinearOperator(t(a, dev), lx.positive_semidefinite_tag)
    sol = lx.linear_solve(op, t([1.0, 1.0, 1.0], dev), lx.Cholesky(), throw=False)
    assert sol.result == lx.RESULTS.singular
    with pytest.raises(lx.LinearSolveError):
        lx.linear_solve(op, t([1.0, 1.0, 1.0], dev), lx.Cholesky())


def test_lu_singular_reports_singular(dev):
    a = np.array([[1.0, 2.0], [2.0, 4.0]])
    op = lx.MatrixLinearOperator(t(a, dev))
    sol = lx.linear_solve(op, t([1.0, 1.0], dev), lx.LU(), throw=False)
    assert sol.result == lx.RESULTS.singular


def test_lu_state_reuse_and_transpose(dev):
    rng = np.random.default_rng(3)
    n = 50
    a = rng.standard_normal((n, n)) + n ** 0.5 * np.eye(n)
    op = lx.MatrixLinearOperator(t(a, dev))
    solver = lx.LU()
    state = solver.init(op, {})
    b1, b2 = rng.standard_normal(n), rng.standard_normal(n)
    x1 = lx.linear_solve(op, t(b1, dev), solver, state=state).value.cpu().numpy()
    x2 = lx.linear_solve(op, t(b2, dev), solver, state=state).value.cpu().numpy()
    assert dense.backward_error(a, x1, b1) <= TOL and dense.backward_error(a, x2, b2) <= TOL
    st_t, _ = solver.transpose(state, {})
    xt, _, _ = solver.compute(st_t, t(b1, dev), {})
    assert dense.backward_error(a.T, xt.cpu().numpy(), b1) <= TOL


def test_invert_reuses_factor(dev):
    rng = np.random.default_rng(5)
    n = 20
    a = rng.standard_normal((n, n)) + 5 * np.eye(n)
    inv = lx.invert(lx.MatrixLinearOperator(t(a, dev)), lx.LU())
    b = rng.standard_normal(n)
    x = inv.mv(t(b, dev)).cpu().numpy()
    assert dense.backward_error(a, x, b) <= TOL


def test_gemv_and_norms(dev):
    rng = np.random.default_rng(9)
    a = rng.standard_normal((37, 53))
    x = rng.standard_normal(53)
    y = lx.MatrixLinearOperator(t(a, dev)).mv(t(x, dev)).cpu().numpy()
    np.testing.assert_allclose(y, a @ x, rtol=1e-13, atol=1e-13)
    from lineax_gb300._blas import gemv

    yt = gemv(t(a, dev), t(y, dev), trans=True).cpu().numpy()
    np.testing.assert_allclose(yt, a.T @ y, rtol=1e-12, atol=1e-12)
    v = rng.standard_normal(100001)
    assert abs(float(lx.two_norm(t(v, dev))) - np.linalg.norm(v)) < 1e-10
    assert float(lx.max_norm(t(v, dev))) == np.max(np.abs(v))
    assert abs(float(lx.tree_dot(t(v, dev), t(v, dev))) - v @ v) < 1e-8
    v[77] = np.nan
    assert np.isnan(float(lx.max_norm(t(v, dev))))
