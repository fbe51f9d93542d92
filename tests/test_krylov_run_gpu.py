"""GPU: the single-call CG and GMRES entry points (lxgb_cg_run,
lxgb_gmres_run), whose loops run on the device under a CUDA graph's
conditional while node.  They issue the same kernels in the same order as
the host-driven loop, so solutions must be bit-identical to it, with the
same step counts and result codes, and match the NumPy restatements of
lineax's loops (lineax/_solver/cg.py:114-227, gmres.py:106-413)."""

import ctypes

import numpy as np
import pytest
import torch

import lineax_gb300 as lx
from lineax_gb300 import _ffi, _krylov
from oracle import krylov

pytestmark = pytest.mark.gpu


def t(x, dev):
    return torch.tensor(np.asarray(x), dtype=torch.float64, device=dev)


def spd(rng, n, shift):
    g = rng.standard_normal((n, n))
    return g @ g.T / n + shift * np.eye(n)


def same(run, block):
    assert run is not None
    assert run.steps == block.steps and run.results == block.results
    assert torch.equal(run.y, block.y)


@pytest.mark.parametrize("every", [10, 1, None, 3])
@pytest.mark.parametrize("precond", [False, True])
def test_cg_run_equals_host_loop_and_oracle(dev, every, precond):
    rng = np.random.default_rng(40 + (every or 0))
    n, k = 150, 3
    a = spd(rng, n, 0.05)
    b = rng.standard_normal((k, n))
    m = np.diag(1.0 / np.diag(a)) if precond else None
    op = lx.MatrixLinearOperator(t(a, dev), lx.positive_semidefinite_tag)
    pre = lx.MatrixLinearOperator(t(m, dev), lx.positive_semidefinite_tag) if precond else None
    kw = dict(rtol=1e-10, atol=1e-10, stabilise_every=every, preconditioner=pre)
    run = _krylov.cg_run(op, t(b, dev), **kw)
    block = _krylov.cg_block(op, t(b, dev), **kw)
    same(run, block)
    # step counts within one of the restatement; with a true-residual
    # replacement every third step (rounding of reductions differs) within two
    slack = 2 if every == 3 else 1
    for c in range(k):
        x_ref, r_ref, s_ref = krylov.cg(lambda v: a @ v, b[c], rtol=1e-10, atol=1e-10,
                                        stabilise_every=every,
                                        precond=(lambda v: m @ v) if precond else None)
        assert run.results[c] == r_ref and abs(run.steps[c] - s_ref) <= slack
        np.testing.assert_allclose(run.y[c].cpu().numpy(), x_ref, rtol=1e-7, atol=1e-9)


def test_cg_run_nsd_max_steps_and_y0(dev):
    """Negated operator (negative-definite input), a max_steps cap with
    rtol = atol = 0, and a start vector: all through lineax's CG."""
    n = 100
    p = -2 * np.eye(n) + np.eye(n, k=1) + np.eye(n, k=-1)
    b = np.random.default_rng(0).standard_normal(n)
    op = lx.MatrixLinearOperator(t(p, dev), (lx.negative_semidefinite_tag, lx.symmetric_tag))
    sol = lx.linear_solve(op, t(b, dev), lx.CG(0.0, 0.0, max_steps=7))
    x_ref, r_ref, s_ref = krylov.cg(lambda v: p @ v, b, rtol=0.0, atol=0.0, max_steps=7, nsd=True)
    assert sol.stats["num_steps"] == s_ref == 7 and sol.result == r_ref
    np.testing.assert_allclose(sol.value.cpu().numpy(), x_ref, rtol=1e-10, atol=1e-12)
    y0 = np.random.default_rng(1).standard_normal(n)
    neg = -lx.MatrixLinearOperator(t(p, dev), lx.negative_semidefinite_tag)
    run = _krylov.cg_run(neg, t(-b, dev), rtol=1e-11, atol=1e-11, y0=t(y0, dev))
    block = _krylov.cg_block(neg, t(-b, dev), rtol=1e-11, atol=1e-11, y0=t(y0, dev))
    same(run, block)


def test_cg_run_poisson_block(dev):
    nx, ny, k = 130, 70, 3
    rng = np.random.default_rng(5)
    b = rng.standard_normal((k, nx * ny))
    op = lx.Poisson2DOperator(nx, ny)
    run = _krylov.cg_run(op, t(b, dev), rtol=1e-8, atol=1e-8, max_steps=400)
    block = _krylov.cg_block(op, t(b, dev), rtol=1e-8, atol=1e-8, max_steps=400)
    same(run, block)


@pytest.mark.parametrize("restart,precond", [(20, False), (5, True), (30, False)])
def test_gmres_run_equals_host_loop_and_oracle(dev, restart, precond):
    rng = np.random.default_rng(70 + restart)
    n, k = 90, 3
    a = rng.standard_normal((n, n)) / np.sqrt(n) + 2.0 * np.eye(n)
    b = rng.standard_normal((k, n))
    m = np.diag(1.0 / np.diag(a)) if precond else None
    op = lx.MatrixLinearOperator(t(a, dev))
    pre = lx.MatrixLinearOperator(t(m, dev)) if precond else None
    kw = dict(rtol=1e-10, atol=1e-10, restart=restart, preconditioner=pre)
    run = _krylov.gmres_run(op, t(b, dev), **kw)
    block = _krylov.gmres_block(op, t(b, dev), **kw)
    same(run, block)
    for c in range(k):
        x_ref, r_ref, s_ref = krylov.gmres(lambda v: a @ v, b[c], rtol=1e-10, atol=1e-10,
                                           restart=restart,
                                           precond=(lambda v: m @ v) if precond else None)
        assert run.results[c] == r_ref and abs(run.steps[c] - s_ref) <= 1
        np.testing.assert_allclose(run.y[c].cpu().numpy(), x_ref, rtol=1e-7, atol=1e-9)


def test_gmres_run_reference_failure_case(dev):
    """tests/test_singular.py: GMRES(restart=2) on the literal 4x4 system
    must not report success — through linear_solve, i.e. the single call."""
    import json
    import pathlib

    gold = json.loads((pathlib.Path(__file__).parent / "golden" /
                       "reference_kats.json").read_text())
    kat = gold["gmres_fails_4x4"]
    a = np.array(kat["matrix"], dtype=np.float64)
    x_true = np.array(kat["true_x"], dtype=np.float64)
    b = a @ x_true
    solver = lx.GMRES(rtol=1e-10, atol=1e-10, restart=2)
    sol = lx.linear_solve(lx.MatrixLinearOperator(t(a, dev)), t(b, dev), solver, throw=False)
    x_ref, r_ref, _ = krylov.gmres(lambda v: a @ v, b, rtol=1e-10, atol=1e-10, restart=2)
    assert sol.result != lx.RESULTS.successful
    assert sol.result == krylov.finalize_result(x_ref, r_ref, b)


def test_run_rejects_bad_arguments(dev):
    """Argument errors come back as LXGB_INVALID_ARG before anything runs."""
    n, k = 8, 1
    a = t(np.eye(n), dev)
    b = t(np.ones((k, n)), dev)
    y = torch.empty_like(b)
    ints = torch.empty(k, dtype=torch.int32, device=dev)
    work = torch.empty(1 << 16, dtype=torch.float64, device=dev)
    bad = _ffi.LinearOperatorDesc(kind=_ffi.OP_POISSON5, n=n, nx=3, ny=3, scale=1.0)  # 9 != 8
    with pytest.raises(_ffi.LxgbError) as e:
        _ffi.call("lxgb_cg_run", k, n, ctypes.addressof(bad), None, _ffi.ptr(b), _ffi.ptr(y), 0,
                  1e-8, 1e-8, -1, 10, _ffi.ptr(ints), _ffi.ptr(ints), _ffi.ptr(work),
                  work.numel() * 8, _ffi.stream_handle(dev))
    assert e.value.status == 100
    good = _ffi.LinearOperatorDesc(kind=_ffi.OP_DENSE, n=n, a=a.data_ptr(), lda=n, scale=1.0)
    with pytest.raises(_ffi.LxgbError) as e:  # stabilise_every above the unrolled limit
        _ffi.call("lxgb_cg_run", k, n, ctypes.addressof(good), None, _ffi.ptr(b), _ffi.ptr(y),
                  0, 1e-8, 1e-8, -1, 65, _ffi.ptr(ints), _ffi.ptr(ints), _ffi.ptr(work),
                  work.numel() * 8, _ffi.stream_handle(dev))
    assert e.value.status == 100
