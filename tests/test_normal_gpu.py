"""GPU parity: the FP64 SYRK (Gram matrices), the multi-CTA Cholesky of one
large matrix, and the Normal solver (lineax/_solver/normal.py) against the
LAPACK oracle."""

import numpy as np
import pytest
import scipy.linalg
import torch

import lineax_gb300 as lx
from lineax_gb300 import _dense, _ffi
from oracle import dense

pytestmark = pytest.mark.gpu


def t(x, dev):
    return torch.tensor(np.asarray(x), dtype=torch.float64, device=dev)


@pytest.mark.parametrize("m,n", [(300, 130), (130, 300), (1000, 64), (64, 1000), (1, 1),
                                 (257, 257)])
def test_syrk_gram(dev, m, n):
    rng = np.random.default_rng(m * 7 + n)
    a = rng.standard_normal((m, n))
    for tall in (True, False):
        g = _dense.gram(t(a, dev), tall)
        ref = a.T @ a if tall else a @ a.T
        gh = g.cpu().numpy()
        assert np.array_equal(gh, gh.T)
        scale = np.abs(a).max() ** 2 * (m if tall else n)
        assert np.abs(gh - ref).max() <= 1e-14 * scale


def test_syrk_update_form(dev):
    """update = 1: C -= AᵀA on the upper triangle only, lower untouched."""
    rng = np.random.default_rng(3)
    k, n = 40, 150
    a = rng.standard_normal((k, n))
    c0 = rng.standard_normal((n, n))
    c = t(c0, dev)
    _ffi.call("lxgb_syrk_f64", 0, n, k, _ffi.ptr(t(a, dev)), n, 1, _ffi.ptr(c), n, 0,
              _ffi.stream_handle(dev))
    ch = c.cpu().numpy()
    ref = c0 - a.T @ a
    iu = np.triu_indices(n)
    il = np.tril_indices(n, -1)
    assert np.abs(ch[iu] - ref[iu]).max() <= 1e-12 * k
    assert np.array_equal(ch[il], c0[il])


def spd(rng, n):
    g = rng.standard_normal((n, n))
    return g @ g.T / n + 0.5 * np.eye(n)


@pytest.mark.parametrize("n", [161, 300, 517, 1024])
def test_potrf_many_ctas_same_bits_as_one_cta(dev, n):
    rng = np.random.default_rng(n)
    a = spd(rng, n)
    u_multi = t(a, dev)
    info = torch.empty(1, dtype=torch.int32, device=dev)
    _ffi.call("lxgb_potrf_f64", n, _ffi.ptr(u_multi), n, _ffi.ptr(info), _ffi.stream_handle(dev))
    u_one = t(a, dev)
    nvec = torch.tensor([n], dtype=torch.int32, device=dev)
    off = torch.zeros(1, dtype=torch.int64, device=dev)
    info1 = torch.empty(1, dtype=torch.int32, device=dev)
    _ffi.call("lxgb_potrf_ragged_f64", 1, n, _ffi.ptr(nvec), _ffi.ptr(off), _ffi.ptr(u_one),
              _ffi.ptr(info1), _ffi.stream_handle(dev))
    torch.cuda.synchronize()
    assert int(info.item()) == 0 and int(info1.item()) == 0
    assert torch.equal(u_multi, u_one)
    u_ref = dense.cho_factor_upper(a)
    assert np.abs(u_multi.cpu().numpy() - u_ref).max() <= 1e-12 * np.abs(u_ref).max()


@pytest.mark.parametrize("n,k", [(300, 10), (300, 200), (700, 65)])
def test_potrf_not_positive_definite_info(dev, n, k):
    """info = k+1 for the first leading minor that is not positive definite
    (LAPACK dpotrf's convention)."""
    rng = np.random.default_rng(k)
    a = spd(rng, n)
    a[k, k] = -1.0e3
    _, info_ref = scipy.linalg.lapack.dpotrf(a, lower=0)
    u = t(a, dev)
    info = torch.empty(1, dtype=torch.int32, device=dev)
    _ffi.call("lxgb_potrf_f64", n, _ffi.ptr(u), n, _ffi.ptr(info), _ffi.stream_handle(dev))
    torch.cuda.synchronize()
    assert int(info.item()) == info_ref == k + 1


@pytest.mark.parametrize("m,n", [(500, 120), (80, 200), (400, 400)])
def test_normal_cholesky_matches_oracle(dev, m, n):
    rng = np.random.default_rng(m + n)
    a = rng.standard_normal((m, n)) / np.sqrt(max(m, n)) + (np.eye(m, n) if m >= n else 0)
    if m < n:
        a = a + np.eye(m, n)
    b = rng.standard_normal(m)
    op = lx.MatrixLinearOperator(t(a, dev))
    sol = lx.linear_solve(op, t(b, dev), lx.Normal(lx.Cholesky()))
    assert sol.result == lx.RESULTS.successful
    x = sol.value.cpu().numpy()
    x_ref = dense.normal_linear_solve(a, b)
    # Two FP64 solves of the normal equations differ by up to ~kappa(A)^2 u
    # (normwise); the bound below is 20 kappa^2 u.
    bound = 20 * np.linalg.cond(a) ** 2 * np.finfo(np.float64).eps
    assert np.abs(x - x_ref).max() <= bound * np.abs(x_ref).max()
    x_ls = np.linalg.lstsq(a, b, rcond=None)[0]
    assert np.abs(x - x_ls).max() <= bound * np.abs(x_ls).max()


def test_normal_cg_tall_and_wide(dev):
    rng = np.random.default_rng(9)
    for m, n in ((300, 100), (100, 300)):
        a = rng.standard_normal((m, n)) / np.sqrt(max(m, n)) + np.eye(m, n)
        b = rng.standard_normal(m)
        op = lx.MatrixLinearOperator(t(a, dev))
        sol = lx.linear_solve(op, t(b, dev), lx.Normal(lx.CG(rtol=1e-12, atol=1e-12)))
        assert sol.result == lx.RESULTS.successful
        x_ls = np.linalg.lstsq(a, b, rcond=None)[0]
        np.testing.assert_allclose(sol.value.cpu().numpy(), x_ls, rtol=1e-7, atol=1e-9)


def test_normal_cg_max_steps_only(dev):
    """tests/test_solve.py::test_iterative_solver_max_steps_only (Normal(CG)
    leg): NSD-tagged 1-D Poisson, rtol = atol = 0, max_steps = 2."""
    n = 100
    p = -2 * np.eye(n) + np.eye(n, k=1) + np.eye(n, k=-1)
    b = np.random.default_rng(0).standard_normal(n)
    op = lx.MatrixLinearOperator(t(p, dev), (lx.negative_semidefinite_tag, lx.symmetric_tag))
    sol = lx.linear_solve(op, t(b, dev), lx.Normal(lx.CG(0.0, 0.0, max_steps=2)))
    assert sol.result == lx.RESULTS.successful
    assert sol.stats["num_steps"] == 2
    assert np.all(np.isfinite(sol.value.cpu().numpy()))


def test_normal_transpose_reuses_state(dev):
    rng = np.random.default_rng(11)
    m, n = 240, 90
    a = rng.standard_normal((m, n)) / np.sqrt(m) + np.eye(m, n)
    solver = lx.Normal(lx.Cholesky())
    op = lx.MatrixLinearOperator(t(a, dev))
    state = solver.init(op, {})
    tstate, topts = solver.transpose(state, {})
    c = rng.standard_normal(n)
    y, res, _ = solver.compute(tstate, t(c, dev), topts)
    assert res == lx.RESULTS.successful
    # Aᵀ y = c is wide: the minimum-norm solution
    y_ref = np.linalg.lstsq(a.T, c, rcond=None)[0]
    np.testing.assert_allclose(y.cpu().numpy(), y_ref, rtol=1e-9, atol=1e-11)


def test_normal_cg_with_preconditioner(dev):
    """normal.py:17-37: the outer preconditioner M enters the inner CG as
    M Mᵀ (tall) or Mᵀ M (wide, with y0 -> Mᵀ y0); the solution is the
    least-squares / minimum-norm one either way."""
    rng = np.random.default_rng(21)
    for m, n in ((240, 90), (90, 240)):
        a = rng.standard_normal((m, n)) / np.sqrt(max(m, n)) + np.eye(m, n)
        b = rng.standard_normal(m)
        if m >= n:  # a diagonal M of the unknowns' space
            pre = lx.MatrixLinearOperator(t(np.diag(1.0 / (1.0 + rng.random(n))), dev))
        else:       # a general M of the right-hand side's space
            pre = lx.MatrixLinearOperator(t(rng.standard_normal((m, m)) * 0.01 + np.eye(m), dev))
        opts = {"preconditioner": pre}
        if m < n:
            opts["y0"] = t(np.zeros(m), dev)
        op = lx.MatrixLinearOperator(t(a, dev))
        sol = lx.linear_solve(op, t(b, dev), lx.Normal(lx.CG(rtol=1e-12, atol=1e-12)),
                              options=opts)
        assert sol.result == lx.RESULTS.successful
        x_ls = np.linalg.lstsq(a, b, rcond=None)[0]
        np.testing.assert_allclose(sol.value.cpu().numpy(), x_ls, rtol=1e-7, atol=1e-9)
