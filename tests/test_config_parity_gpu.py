"""GPU parity at the benchmark configurations' full sizes.

Every solution produced here is checked on the host against the oracle:
backward errors from residuals without rounding error
(oracle.dense.residual_exact), forward errors against SciPy/LAPACK or the
statement-for-statement Krylov restatement.  The bar follows lineax's own
well-posed tests (tests/test_well_posed.py:34-52 compare with the true
solution at 1e-10); the mixed-precision paths additionally promise a normwise
backward error of 1e-12.

Tolerance of the 1e-12 checks: the kernels stop on their own estimate of the
backward error, whose denominator ||A||_inf is summed in FP32 (relative error
up to n * 2^-24 = 3e-5 at n = 512) — so a solution the kernel accepted at
0.99999e-12 may measure 1.00003e-12 here.  BERR_BAR = 1e-12 * (1 + 1e-4).
"""

import numpy as np
import pytest
import scipy.linalg as sl
import torch

import lineax_gb300 as lx
from lineax_gb300 import _krylov, batched, mixed, serve, workloads
from oracle import dense, krylov

pytestmark = pytest.mark.gpu
TOL = 1e-12
BERR_BAR = TOL * (1 + 1e-4)


def t(x, dev):
    return torch.tensor(np.asarray(x), dtype=torch.float64, device=dev)


# ---------------------------------------------------------------------------
# Configuration 2: 4096 ragged SPD systems, n log-uniform in [16, 512], 1-8
# right-hand sides, FP32 factor + FP64 refinement (the seeded batch the
# benchmark times).
# ---------------------------------------------------------------------------
def test_ragged_spd_4096_every_system(dev):
    wl = workloads.ragged_spd(0, 4096)
    rb = batched.RaggedBatch.from_packed(torch.from_numpy(wl.a).to(dev),
                                         torch.from_numpy(wl.b).to(dev), wl.n, wl.nrhs, dev)
    res = batched.spd_solve_ragged_mixed(rb, tol=TOL)
    torch.cuda.synchronize()
    info = res.info.cpu().numpy()
    assert (info == 0).all(), np.flatnonzero(info)
    x = res.x.cpu().numpy()
    worst, ao, bo = 0.0, 0, 0
    rng = np.random.default_rng(7)
    sample = set(rng.choice(4096, 64, replace=False).tolist()) | {0, 4095}
    for s, (n, k) in enumerate(zip(wl.n, wl.nrhs)):
        a = wl.a[ao: ao + n * n].reshape(n, n)
        b = wl.b[bo: bo + n * k].reshape(k, n)
        xs = x[bo: bo + n * k].reshape(k, n)
        be = dense.backward_errors_exact(a, xs, b)
        worst = max(worst, float(be.max()))
        assert (be <= BERR_BAR).all(), (s, n, k, be)
        if s in sample:
            x_ref = dense.cholesky_linear_solve(a, b.T).T
            for c in range(k):
                assert dense.forward_error(xs[c], x_ref[c]) <= 1e-9, (s, n, c)
        ao += n * n
        bo += n * k
    print(f"ragged 4096: worst exact backward error {worst:.3e}")


# ---------------------------------------------------------------------------
# Configuration 3: dense n = 8192, 16 right-hand sides, cond 1e2 / 1e6 / 1e10.
# ---------------------------------------------------------------------------
def _haar_conditioned(n, cond, seed, dev):
    g = torch.Generator(device=dev).manual_seed(seed)

    def haar():
        q, r = torch.linalg.qr(torch.randn(n, n, dtype=torch.float64, device=dev, generator=g))
        return q * torch.sign(torch.diagonal(r))

    u, v = haar(), haar()
    sig = torch.logspace(0, -float(np.log10(cond)), n, dtype=torch.float64, device=dev)
    return ((u * sig) @ v.T).contiguous()


@pytest.mark.parametrize("cond", [1e2, 1e6, 1e10])
def test_gmres_ir_n8192(dev, cond):
    n, k = 8192, 16
    a = _haar_conditioned(n, cond, 5, dev)
    b = torch.randn(k, n, dtype=torch.float64, device=dev,
                    generator=torch.Generator(device=dev).manual_seed(11))
    res = mixed.gmres_ir(a, b, tol=TOL, restart=8, max_outer=20, inner_max_steps=5,
                         precision="3xtf32", arith="auto", fallback=True)
    torch.cuda.synchronize()
    tier = "fp64_lu" if res.fallback else ("gmres" if any(res.inner_steps) else "ir")
    be = dense.backward_errors_exact(a.cpu().numpy(), res.x.cpu().numpy(), b.cpu().numpy())
    print(f"n=8192 cond={cond:.0e}: tier {tier}, outer {res.outer}, "
          f"inner {res.inner_steps}, exact backward error {be.max():.3e}")
    assert (be <= BERR_BAR).all(), be
    if cond <= 1e6:
        assert not res.fallback  # refinement alone recovers FP64 accuracy here


# ---------------------------------------------------------------------------
# Configuration 4a: least squares 16384 x 2048, b = A x* + 1e-3 noise.
# ---------------------------------------------------------------------------
def test_least_squares_16384x2048(dev):
    m, n = 16384, 2048
    rng = np.random.default_rng(44)
    a = rng.standard_normal((m, n)).astype(np.float32).astype(np.float64)
    xs = rng.standard_normal(n)
    b = a @ xs + 1e-3 * rng.standard_normal(m)
    x_ref = sl.lstsq(a, b, lapack_driver="gelsy", check_finite=False)[0]
    res = mixed.qr_lstsq(t(a, dev), t(b[None, :], dev))
    assert res.converged
    x = res.x.cpu().numpy()[0]
    assert dense.forward_error(x, x_ref) <= 1e-10
    sol = lx.linear_solve(lx.MatrixLinearOperator(t(a, dev)), t(b, dev), lx.QR())
    assert dense.forward_error(sol.value.cpu().numpy(), x_ref) <= 1e-10
    # the least-squares optimality condition Aᵀ r = 0 to FP64 accuracy
    r = dense.residual_exact(a, x[None, :], b[None, :])[0]
    assert np.abs(a.T @ r).max() <= 1e-10 * np.abs(a).sum(axis=0).max() * np.abs(r).max()


# ---------------------------------------------------------------------------
# Configuration 4b: CG on the 5-point Poisson operator, 2048² grid, 64
# right-hand sides, at a capped number of steps.
# ---------------------------------------------------------------------------
def _poisson_np(nx, ny):
    def mv(v):
        u = v.reshape(nx, ny)
        out = 4.0 * u
        out[1:, :] -= u[:-1, :]
        out[:-1, :] -= u[1:, :]
        out[:, 1:] -= u[:, :-1]
        out[:, :-1] -= u[:, 1:]
        return out.reshape(-1)
    return mv


def test_cg_poisson_2048_64rhs_capped(dev):
    nx = ny = 2048
    k, cap = 64, 30
    rng = np.random.default_rng(64)
    b = rng.standard_normal((k, nx * ny))
    op = lx.Poisson2DOperator(nx, ny)
    res = _krylov.cg_block(op, t(b, dev), rtol=1e-10, atol=1e-10, max_steps=cap)
    assert all(s == cap for s in res.steps)
    assert all(r == _krylov.MAX_STEPS_REACHED for r in res.results)
    mv = _poisson_np(nx, ny)
    y = res.y
    for c in (0, 37):
        x_ref, r_ref, s_ref = krylov.cg(mv, b[c], rtol=1e-10, atol=1e-10, max_steps=cap)
        assert s_ref == cap and r_ref == krylov.MAX_STEPS_REACHED
        yc = y[c].cpu().numpy()
        assert np.abs(yc - x_ref).max() <= 1e-10 * np.abs(x_ref).max()
    # the mixed-precision CG at the same cap: FP32 iterations track the FP64
    # iterates to FP32 accuracy
    mx = _krylov.cg_poisson_mixed(op, t(b, dev), rtol=1e-10, atol=1e-10, max_steps=32)
    assert all(s == 32 for s in mx.steps)
    x_ref, _, _ = krylov.cg(mv, b[0], rtol=1e-10, atol=1e-10, max_steps=32)
    assert np.abs(mx.y[0].cpu().numpy() - x_ref).max() <= 1e-4 * np.abs(x_ref).max()


# ---------------------------------------------------------------------------
# Configuration 5: the serving mix up to n = 4096, every completion against
# the oracle's solution.
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_serving_mix_against_oracle(dev, mode):
    reqs = serve.synthetic_requests(48, seed=21, nmax=4096, device=dev)
    srv = serve.SolveServer(dev, mode=mode)
    out = srv.run(reqs, realtime=False)
    assert len(out) == len(reqs)
    mats = {}
    for r in reqs:
        if r.a is not None:
            mats[r.op_id] = r.a.numpy()
    for c, r in zip(out, reqs):
        a = mats[r.op_id]
        b = r.b.numpy().reshape(r.nrhs, r.n)
        x = c.x.cpu().numpy()
        if r.kind == "cholesky":
            x_ref = dense.cholesky_linear_solve(a, b.T).T
        elif r.kind == "qr":
            x_ref = dense.qr_linear_solve(a, b.T) if r.nrhs == 1 else np.stack(
                [dense.qr_linear_solve(a, b[j]) for j in range(r.nrhs)])
            x_ref = x_ref.reshape(r.nrhs, r.n)
        else:
            x_ref = dense.lu_linear_solve(a, b.T).T
        be = dense.backward_errors_exact(a, x, b)
        assert (be <= BERR_BAR).all(), (r.rid, r.kind, r.n, c.route, be)
        for j in range(r.nrhs):
            assert dense.forward_error(x[j], x_ref[j]) <= 1e-9, (r.rid, r.kind, r.n, c.route)
