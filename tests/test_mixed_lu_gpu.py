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
@pytest.mark.parametrize("n", [64, 256, 600, 1024, 2500])
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


def swaps_to_perm(piv):
    perm = np.arange(len(piv))
    for k, p in enumerate(piv):
        perm[[k, p]] = perm[[p, k]]
    return perm


@pytest.mark.parametrize("precision,ulp", [("tf32", 2.0 ** -11), ("3xtf32", 2.0 ** -22)])
@pytest.mark.parametrize("n", [256, 600, 1024])
def test_lu_inverse_factors(dev, n, precision, ulp):
    """L^{-1} L = I and U^{-1} U = I componentwise to the update's rounding:
    |X T - I| <= n u |X| |T| (TF32 u = 2^-11, 3xTF32 about 2^-22); perm
    composes the row interchanges."""
    a = conditioned(n, 1e2, n + 1)
    f = mixed.lu_factor_tf32(torch.tensor(a, device=dev), precision)
    inv = mixed.lu_inverse(f, precision)
    lu = f.lu.double().cpu().numpy()
    l = np.tril(lu, -1) + np.eye(n)
    u = np.triu(lu)
    linv = inv.linv.double().cpu().numpy()
    uinv = inv.uinv.double().cpu().numpy()
    assert np.all(np.triu(linv, 1) == 0) and np.all(np.diag(linv) == 1)
    assert np.all(np.tril(uinv, -1) == 0)
    for x, t in ((linv, l), (uinv, u)):
        scale = np.abs(x) @ np.abs(t)
        err = np.abs(x @ t - np.eye(n))
        assert np.all(err[scale == 0] == 0)
        assert np.max(err[scale > 0] / scale[scale > 0]) < n * ulp
    assert np.array_equal(inv.perm.cpu().numpy(), swaps_to_perm(f.piv.cpu().numpy()))


@pytest.mark.parametrize("arith,bound", [("df", 1e-13), ("fp32", 1e-5)])
@pytest.mark.parametrize("n,k", [(256, 1), (600, 16), (1024, 20)])
def test_inverse_preconditioner_apply(dev, n, k, arith, bound):
    """M x = U^{-1} (L^{-1} (P x)) against the same FP32 inverses applied in FP64."""
    a = conditioned(n, 1e6, n + 2)
    f = mixed.lu_factor_tf32(torch.tensor(a, device=dev), "3xtf32")
    inv = mixed.lu_inverse(f, "3xtf32")
    x = np.random.default_rng(n + k).standard_normal((k, n))
    m = mixed.InverseLUPreconditioner(f, inv, arith)
    y = m.mv_block(torch.tensor(x, device=dev)).cpu().numpy()
    linv = inv.linv.double().cpu().numpy()
    uinv = inv.uinv.double().cpu().numpy()
    perm = inv.perm.cpu().numpy()
    ref = (uinv @ (linv @ x[:, perm].T)).T
    scale = (np.abs(uinv) @ (np.abs(linv) @ np.abs(x[:, perm]).T)).T
    assert np.max(np.abs(y - ref) / scale) < bound


@pytest.mark.parametrize("m,n,k", [(300, 200, 5), (512, 512, 16), (129, 700, 20), (333, 800, 1),
                                   (200, 1000, 3), (64, 2048, 4)])
def test_double_float_gemv(dev, m, n, k):
    """A x and b - A x with A as an FP32 hi + lo pair: FP64-level accuracy in
    double-float, FP32-level on the hi part alone."""
    rng = np.random.default_rng(m + n + k)
    a = rng.standard_normal((m, n))
    x = rng.standard_normal((k, n))
    b = rng.standard_normal((k, m))
    at = torch.tensor(a, device=dev)
    sp = mixed.split_matrix(at)
    assert np.abs(sp.hi.double().cpu().numpy() + sp.lo.double().cpu().numpy() - a).max() \
        <= 2.0 ** -46 * np.abs(a).max()
    lib_y = torch.empty((k, m), dtype=torch.float64, device=dev)
    from lineax_gb300 import _ffi
    wb = int(_ffi.load().lxgb_gemv_df_workspace_size(n, k))
    work = torch.empty(wb // 8 + 1, dtype=torch.float64, device=dev)
    xt = torch.tensor(x, device=dev)
    bt = torch.tensor(b, device=dev)
    scale = np.abs(x) @ np.abs(a).T
    for mode, bound in ((1, 1e-14), (0, 1e-6)):
        lo = sp.lo if mode == 1 else None
        for with_b in (False, True):
            _ffi.call("lxgb_gemv_df", m, n, _ffi.ptr(sp.hi), _ffi.ptr(lo), n, k, _ffi.ptr(xt), n,
                      _ffi.ptr(bt if with_b else None), _ffi.ptr(lib_y), m, mode, _ffi.ptr(work),
                      work.numel() * 8, _ffi.stream_handle(dev))
            y = lib_y.cpu().numpy()
            ref = (b - x @ a.T) if with_b else x @ a.T
            assert np.max(np.abs(y - ref) / scale) < bound, (mode, with_b)


@pytest.mark.parametrize("n,cond,arith", [(256, 1e2, "df"), (512, 1e6, "df"), (1024, 1e2, "df"),
                                          (1024, 1e6, "df"), (512, 1e2, "fp32"),
                                          (512, 1e6, "auto"), (1024, 1e2, "auto"),
                                          (1024, 1e2, "ir")])
def test_gmres_ir_reaches_fp64_backward_error(dev, n, cond, arith):
    a = conditioned(n, cond, n + int(np.log10(cond)))
    rng = np.random.default_rng(7)
    b = rng.standard_normal((4, n))
    res = mixed.gmres_ir(torch.tensor(a, device=dev), torch.tensor(b, device=dev), tol=1e-12,
                         arith=arith)
    assert res.converged and not res.fallback and res.outer <= 6, (res.outer, res.berr)
    x = res.x.cpu().numpy()
    for c in range(4):
        assert res.berr[c] <= 1e-12
        assert dense.backward_error(a, x[c], b[c]) <= 1e-12
        # a backward error <= 1e-12 implies a forward error <= ~2 cond * 1e-12
        assert dense.forward_error(x[c], dense.lu_linear_solve(a, b[c])) <= 2 * cond * 1e-12


def test_gmres_ir_falls_back_to_fp64_when_it_stalls(dev):
    """cond 1e10 with log-spaced singular values leaves about a quarter of the
    directions below FP32 resolution: GMRES(20) stalls, and fallback=True
    returns the FP64 LU solution instead."""
    n = 512
    a = conditioned(n, 1e10, 99)
    b = np.random.default_rng(5).standard_normal((3, n))
    res = mixed.gmres_ir(torch.tensor(a, device=dev), torch.tensor(b, device=dev), tol=1e-12,
                         max_outer=4, inner_max_steps=10, fallback=True)
    assert res.fallback and res.converged, res.berr
    x = res.x.cpu().numpy()
    for c in range(3):
        assert dense.backward_error(a, x[c], b[c]) <= 1e-12


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

    def pre(v):  # the FP32 factor applied in FP64 (the device applies its inverses in double-float)
        import scipy.linalg as sl
        return sl.lu_solve((lu.astype(np.float64), piv), v)

    x_ref, r_ref, s_ref = krylov.gmres(lambda v: a @ v, b, rtol=1e-10, atol=1e-10, precond=pre)
    # The inverses carry FP32 rounding of their own: allow two restart cycles
    assert r_ref == 0 and abs(sol.stats["num_steps"] - s_ref) <= 2


@pytest.mark.parametrize("n,cond,precision,max_outer", [(1024, 1e2, "3xtf32", 20),
                                                        (512, 1e6, "tf32", 6),
                                                        (768, 1e6, "3xtf32", 20)])
def test_gmres_ir_single_call_equals_host_loop(dev, n, cond, precision, max_outer):
    """lxgb_gmres_ir_run (the refinement loop, its tier switch and the inner
    GMRES loop as conditional graph nodes on the device) issues the host
    loop's kernels in the host loop's order: the same solution bits, the same
    number of refinement steps and the same backward errors, whether the
    solve converges in the plain-refinement tier or moves on to GMRES."""
    a = torch.tensor(conditioned(n, cond, n + 5), device=dev)
    b = torch.tensor(np.random.default_rng(n).standard_normal((3, n)), device=dev)
    f = mixed.lu_factor_tf32(a, precision)
    inv = mixed.lu_inverse(f, precision)
    sp = mixed.split_matrix(a)
    kw = dict(tol=1e-12, restart=8, inner_max_steps=5, max_outer=max_outer, factor=f,
              inverse=inv, split=sp, precision=precision, arith="auto", fallback=False)
    host = mixed.gmres_ir(a, b, device_loop=False, **kw)
    devl = mixed.gmres_ir(a, b, device_loop=True, **kw)
    assert torch.equal(host.x, devl.x)
    assert host.outer == devl.outer and host.converged == devl.converged
    assert host.berr == devl.berr
    assert (max(host.inner_steps) > 0) == (max(devl.inner_steps) > 0)


@pytest.mark.parametrize("n", [256, 1000])
def test_gmres_ir_qr_single_call_equals_host_loop(dev, n):
    """The QR-preconditioned refinement (M = R^{-1} Qᵀ of the square TF32 QR,
    LXGB_OP_QR32) in one lxgb_gmres_ir_run call equals the host loop bit for
    bit, and reaches the FP64 backward error."""
    g = np.random.default_rng(n).standard_normal((n, n))
    a_h = g / np.sqrt(n) + np.eye(n)
    a = torch.tensor(a_h, device=dev)
    b_h = np.random.default_rng(n + 1).standard_normal((2, n))
    b = torch.tensor(b_h, device=dev)
    qr = mixed.qr_square_tf32(a)
    sp = mixed.split_matrix(a)
    kw = dict(tol=1e-12, restart=8, inner_max_steps=5, max_outer=20, split=sp, qr=qr,
              arith="auto", fallback=False)
    host = mixed.gmres_ir(a, b, device_loop=False, **kw)
    devl = mixed.gmres_ir(a, b, device_loop=True, **kw)
    assert devl.converged and torch.equal(host.x, devl.x)
    assert host.outer == devl.outer and host.berr == devl.berr
    be = dense.backward_errors_exact(a_h, devl.x.cpu().numpy(), b_h)
    assert (be <= 1e-12 * (1 + 1e-4)).all(), be


@pytest.mark.parametrize("n", [256, 1024, 2048])
def test_bf16_lu_factorisation_residual(dev, n):
    """BF16 tensor-core updates (8-bit significands, FP32 accumulation): the
    factor reproduces P A to a small multiple of u = 2^-8 (the TF32 test's
    bound, 3e-2, is about 60 of its u = 2^-11; measured here: 23 u at n = 2048)."""
    a = conditioned(n, 1e2, n + 3)
    f = mixed.lu_factor_tf32(torch.tensor(a, device=dev), "bf16")
    assert int(f.info) == 0
    lu = f.lu.double().cpu().numpy()
    piv = f.piv.cpu().numpy()
    l = np.tril(lu, -1) + np.eye(n)
    u = np.triu(lu)
    pa = a.copy()
    for k in range(n):
        pa[[k, piv[k]]] = pa[[piv[k], k]]
    rel = np.linalg.norm(pa - l @ u) / np.linalg.norm(a)
    assert rel < 64 * 2.0 ** -8, rel


@pytest.mark.parametrize("cond", [1e2, 1e6])
def test_gmres_ir_precision_ladder(dev, cond):
    """A factor that stalls moves up the ladder BF16 -> TF32 -> 3xTF32 before
    any FP64 fallback: at cond 1e2 and 1e6 the solve ends on a low-precision
    factor, at backward error <= 1e-12, and reports the tiers it tried."""
    n = 1024
    a = conditioned(n, cond, 77)
    b = np.random.default_rng(3).standard_normal((4, n))
    res = mixed.gmres_ir(torch.tensor(a, device=dev), torch.tensor(b, device=dev), tol=1e-12,
                         restart=8, inner_max_steps=5, precision="bf16", arith="auto",
                         fallback=True, escalate=True)
    assert res.converged and not res.fallback, res.tiers
    assert res.tiers[0][0] == "bf16" and res.tiers[-1][2]
    x = res.x.cpu().numpy()
    be = dense.backward_errors_exact(a, x, b)
    assert (be <= 1e-12 * (1 + 1e-4)).all(), be


def spd(n, seed):
    g = np.random.default_rng(seed).standard_normal((n, n))
    return g @ g.T / n + 1e-2 * np.eye(n)


@pytest.mark.parametrize("n", [64, 260, 1000, 2048])
def test_cholesky_factor_tf32(dev, n):
    """FP32 Cholesky with 3xTF32 tensor-core updates (lxgb_potrf_f32_tc) in the
    mixed-LU form: L'U' = A to FP32 level, no interchanges, A read from its
    upper triangle (the lower triangle is ignored), and its inverses
    (L'^{-1} by substitution, U'^{-1} = L'^{-T} D^{-2}) within n u |X||T|."""
    a = spd(n, n)
    a_upper = np.triu(a)                  # lower triangle absent: it is not read
    f = mixed.cholesky_factor_tf32(torch.tensor(a_upper, device=dev))
    assert int(f.info) == 0
    assert np.array_equal(f.piv.cpu().numpy(), np.arange(n))
    lu = f.lu.double().cpu().numpy()
    l = np.tril(lu, -1) + np.eye(n)
    u = np.triu(lu)
    rel = np.linalg.norm(a - l @ u) / np.linalg.norm(a)
    assert rel < 5e-5, rel
    # U' = D^2 L'^T exactly as formed: U'_ij = L'_ji * U'_jj... within FP32 rounding
    assert np.allclose(u, np.diag(np.diag(u)) @ l.T, rtol=1e-5, atol=0)
    inv = mixed.cholesky_inverse(f)
    linv = inv.linv.double().cpu().numpy()
    uinv = inv.uinv.double().cpu().numpy()
    assert np.all(np.triu(linv, 1) == 0) and np.all(np.tril(uinv, -1) == 0)
    for x, t in ((linv, l), (uinv, u)):
        scale = np.abs(x) @ np.abs(t)
        err = np.abs(x @ t - np.eye(n))
        assert np.max(err[scale > 0] / scale[scale > 0]) < n * 2.0 ** -21


def test_cholesky_factor_tf32_gmres_ir_and_indefinite(dev):
    n = 1500 - 1500 % 4
    a = spd(n, 3)
    b = np.random.default_rng(4).standard_normal((5, n))
    at = torch.tensor(a, device=dev)
    f = mixed.cholesky_factor_tf32(at)
    inv = mixed.cholesky_inverse(f)
    res = mixed.gmres_ir(at, torch.tensor(b, device=dev), tol=1e-12, factor=f, inverse=inv,
                         precision="3xtf32", arith="auto", fallback=True)
    assert res.converged and not res.fallback, (res.outer, res.berr)
    be = dense.backward_errors_exact(a, res.x.cpu().numpy(), b)
    assert (be <= 1e-12 * (1 + 1e-4)).all(), be
    # not positive definite: the first non-positive pivot is reported
    m = -np.eye(128)
    fm = mixed.cholesky_factor_tf32(torch.tensor(m, device=dev))
    assert int(fm.info) == 1
