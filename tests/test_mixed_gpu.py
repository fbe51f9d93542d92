"""GPU parity: ragged batched Cholesky, plain FP64 and mixed precision
(FP32 factor + FP64 refinement), against the SciPy oracle."""

import numpy as np
import pytest
import torch

from lineax_gb300 import _ffi, batched
from oracle import dense

pytestmark = pytest.mark.gpu
TOL = 1e-12


def make_ragged(rng, ns, ks):
    mats, rhs = [], []
    for n, k in zip(ns, ks):
        g = rng.standard_normal((n, n))
        mats.append(g @ g.T / n + 1e-2 * np.eye(n))
        rhs.append(rng.standard_normal((k, n)))
    return mats, rhs


def to_batch(mats, rhs, dev):
    return batched.RaggedBatch.from_lists([torch.tensor(m) for m in mats],
                                          [torch.tensor(r) for r in rhs], device=dev)


@pytest.mark.parametrize("ns", [[16, 17, 33], [64, 128, 160], [161, 224, 225, 300, 512]])
def test_ragged_potrf_potrs_f64(dev, ns):
    rng = np.random.default_rng(sum(ns))
    ks = [1 + (i % 3) for i in range(len(ns))]
    mats, rhs = make_ragged(rng, ns, ks)
    rb = to_batch(mats, rhs, dev)
    u, info = batched.cholesky_factor_ragged(rb)
    assert int(info.abs().sum()) == 0
    x, _ = batched.cholesky_solve_ragged(rb, u)
    for s, (m, r) in enumerate(zip(mats, rhs)):
        us = u[rb.a_off_host[s]: rb.a_off_host[s] + ns[s] ** 2].view(ns[s], ns[s]).cpu().numpy()
        np.testing.assert_allclose(us, dense.cho_factor_upper(m), rtol=1e-9, atol=1e-11)
        xs = rb.system_b(x, s).cpu().numpy()
        for k in range(ks[s]):
            assert dense.backward_error(m, xs[k], r[k]) <= TOL


@pytest.mark.parametrize("ns", [[16, 17, 40, 100], [200, 224, 225, 256], [300, 400, 512]])
def test_mixed_reaches_fp64_backward_error(dev, ns):
    rng = np.random.default_rng(len(ns) * 1000 + ns[0])
    ks = [1 + (3 * i) % 8 for i in range(len(ns))]
    mats, rhs = make_ragged(rng, ns, ks)
    rb = to_batch(mats, rhs, dev)
    res = batched.spd_solve_ragged_mixed(rb, tol=TOL)
    info = res.info.cpu().numpy()
    iters = res.iters.cpu().numpy()
    berr = res.berr.cpu().numpy()
    assert (info == 0).all(), info
    assert (iters >= 2).all() and (iters <= 10).all(), iters
    for s, (m, r) in enumerate(zip(mats, rhs)):
        xs = rb.system_b(res.x, s).cpu().numpy()
        worst = 0.0
        for k in range(ks[s]):
            ref = dense.cholesky_linear_solve(m, r[k])
            be = dense.backward_error(m, xs[k], r[k])
            worst = max(worst, be)
            assert be <= TOL
            assert dense.forward_error(xs[k], ref) <= 1e-9
        assert berr[s] <= TOL and berr[s] >= 0.0
        assert worst <= 10 * max(berr[s], 1e-17)


def test_mixed_many_rhs_chunks(dev):
    rng = np.random.default_rng(3)
    mats, rhs = make_ragged(rng, [50, 250], [20, 17])
    rb = to_batch(mats, rhs, dev)
    res = batched.spd_solve_ragged_mixed(rb, tol=TOL)
    assert (res.info.cpu().numpy() == 0).all()
    for s, (m, r) in enumerate(zip(mats, rhs)):
        xs = rb.system_b(res.x, s).cpu().numpy()
        for k in range(r.shape[0]):
            assert dense.backward_error(m, xs[k], r[k]) <= TOL


def test_mixed_not_spd_reports_breakdown(dev):
    rng = np.random.default_rng(4)
    good = make_ragged(rng, [30], [1])
    bad = np.diag(np.concatenate([np.ones(10), [-1.0], np.ones(9)]))
    mats = [good[0][0], bad]
    rhs = [good[1][0], rng.standard_normal((1, 20))]
    rb = to_batch(mats, rhs, dev)
    res = batched.spd_solve_ragged_mixed(rb, tol=TOL)
    info = res.info.cpu().numpy()
    assert info[0] == 0 and info[1] == 11
    assert np.isnan(rb.system_b(res.x, 1).cpu().numpy()).all()


def test_mixed_result_independent_of_batch_mix(dev):
    """A system's result is the same alone and inside a larger ragged mix."""
    rng = np.random.default_rng(6)
    mats, rhs = make_ragged(rng, [37, 190, 300, 64], [2, 1, 3, 1])
    rb = to_batch(mats, rhs, dev)
    res_all = batched.spd_solve_ragged_mixed(rb, tol=TOL)
    for s in range(len(mats)):
        alone = to_batch([mats[s]], [rhs[s]], dev)
        res1 = batched.spd_solve_ragged_mixed(alone, tol=TOL)
        assert torch.equal(rb.system_b(res_all.x, s), alone.system_b(res1.x, 0))


def test_mixed_captured_graph_replay_matches_direct_call(dev):
    """The ragged solve captured in a CUDA graph and replayed gives the same
    bits as a direct call, and a replay after the right-hand sides change
    solves the new ones."""
    rng = np.random.default_rng(21)
    ns = [300, 17, 144, 65, 512, 33]
    mats, rhs = make_ragged(rng, ns, [1 + i % 3 for i in range(len(ns))])
    rb = to_batch(mats, rhs, dev)
    direct = batched.spd_solve_ragged_mixed(rb, 1e-12)
    g = batched.CapturedMixedSolve(rb, 1e-12)
    out = g.replay()
    torch.cuda.synchronize()
    assert torch.equal(out.x, direct.x) and torch.equal(out.iters, direct.iters)
    rb.b.mul_(2.0)
    out = g.replay()
    again = batched.spd_solve_ragged_mixed(rb, 1e-12)
    torch.cuda.synchronize()
    assert torch.equal(out.x, again.x)
    assert float(out.berr.max()) <= 1e-12


@pytest.mark.parametrize("chunks,buffers", [(1, 1), (3, 1), (8, 2), (1, 2)])
def test_host_solver_chunked_copies_match_device_solve(dev, chunks, buffers):
    """The host-buffer solver (copies overlapping solves: later chunks of a
    call, or the next call into the other buffer set) returns the same bits
    as one device-resident solve, and later calls with new data solve the new
    data."""
    rng = np.random.default_rng(33)
    ns = [512, 300, 200, 145, 144, 100, 64, 33, 17, 16, 250, 90]
    ks = [1 + (3 * i) % 8 for i in range(len(ns))]
    mats, rhs = make_ragged(rng, ns, ks)
    rb = to_batch(mats, rhs, dev)
    ref = batched.spd_solve_ragged_mixed(rb, tol=TOL)
    hs = batched.HostRaggedSPDSolver(ns, ks, TOL, device=dev, chunks=chunks, buffers=buffers)
    assert len(hs.chunks) == min(chunks, len(ns))
    a_h = rb.a.cpu().pin_memory()
    b_h = rb.b.cpu().pin_memory()
    x_h = torch.empty(rb.b.numel(), dtype=torch.float64).pin_memory()
    i_h = torch.empty(len(ns), dtype=torch.int32).pin_memory()
    it_h = torch.empty(len(ns), dtype=torch.int32).pin_memory()
    be_h = torch.empty(len(ns), dtype=torch.float64).pin_memory()
    hs(a_h, b_h, x_h, i_h, it_h, be_h)
    torch.cuda.synchronize()
    assert torch.equal(x_h, ref.x.cpu())
    assert torch.equal(i_h, ref.info.cpu()) and torch.equal(it_h, ref.iters.cpu())
    assert torch.equal(be_h, ref.berr.cpu())
    for scale in (-3.0, 0.5, 2.0):
        b_h.mul_(scale)
        hs(a_h, b_h, x_h, i_h, it_h, be_h)
        torch.cuda.synchronize()
        rb.b.mul_(scale)
        ref2 = batched.spd_solve_ragged_mixed(rb, tol=TOL)
        torch.cuda.synchronize()
        assert torch.equal(x_h, ref2.x.cpu())


def test_mixed_edge_cases(dev):
    """Empty systems, a system with no right-hand side, the largest order
    (1024), a non-finite matrix (breakdown reported, NaN solution) and a
    system above the caller's max_n (info = -2) in one ragged launch."""
    from lineax_gb300 import _ffi

    rng = np.random.default_rng(41)
    ns = [0, 33, 1024, 20, 50]
    ks = [0, 2, 1, 0, 3]
    mats, rhs = make_ragged(rng, ns, ks)
    mats[4] = mats[4].copy()
    mats[4][7, 7] = np.nan
    rb = to_batch(mats, rhs, dev)
    res = batched.spd_solve_ragged_mixed(rb, tol=TOL)
    torch.cuda.synchronize()
    info = res.info.cpu().numpy()
    berr = res.berr.cpu().numpy()
    assert info[0] == 0 and berr[0] == 0.0
    assert info[1] == 0 and info[2] == 0 and info[3] == 0
    assert berr[1] <= TOL and berr[2] <= TOL
    for s in (1, 2):
        xs = rb.system_b(res.x, s).cpu().numpy()
        for k in range(xs.shape[0]):
            assert dense.backward_error(mats[s], xs[k], rhs[s][k]) <= TOL
    assert info[4] > 0 and np.isnan(rb.system_b(res.x, 4).cpu().numpy()).all()
    # a caller-side max_n below a system's order: that system gets info -2
    out = batched.MixedResult(x=torch.empty_like(rb.b), info=torch.empty_like(res.info),
                              iters=torch.empty_like(res.iters), berr=torch.empty_like(res.berr))
    ws = batched.MixedWorkspace(rb.batch, 64, rb.max_nrhs, dev)
    _ffi.call("lxgb_posv_ragged_mixed", rb.batch, 64, rb.max_nrhs, _ffi.ptr(rb.n),
              _ffi.ptr(rb.nrhs), _ffi.ptr(rb.a_off), _ffi.ptr(rb.a), _ffi.ptr(rb.b_off),
              _ffi.ptr(rb.b), _ffi.ptr(out.x), TOL, 10, _ffi.ptr(out.info), _ffi.ptr(out.iters),
              _ffi.ptr(out.berr), _ffi.ptr(ws.buf), ws.nbytes, _ffi.stream_handle(dev))
    torch.cuda.synchronize()
    info2 = out.info.cpu().numpy()
    assert info2[2] == -2 and info2[1] == 0 and info2[3] == 0 and info2[0] == 0
    assert torch.equal(rb.system_b(out.x, 1), rb.system_b(res.x, 1))


def test_mixed_factors_store_then_load_same_bits(dev):
    """lxgb_posv_ragged_mixed_factors: a stored FP32 factor is the Cholesky
    factor to FP32 accuracy, and solving again from it (no factorisation)
    gives bit-identical solutions, iteration counts and backward errors."""
    rng = np.random.default_rng(31)
    ns, ks = [512, 300, 145, 144, 100, 16], [3, 8, 1, 2, 5, 4]
    mats, rhs = make_ragged(rng, ns, ks)
    rb = to_batch(mats, rhs, dev)
    plain = batched.spd_solve_ragged_mixed(rb, tol=TOL)
    store = [torch.empty((n, n), dtype=torch.float32, device=dev) for n in ns]
    plan = batched.FactorPlan([batched.FACTOR_STORE] * len(ns), store, dev)
    first = batched.spd_solve_ragged_mixed(rb, tol=TOL, factors=plan)
    # a mix of loads and fresh factorisations in one launch
    modes = [batched.FACTOR_LOAD, batched.FACTOR_COMPUTE, batched.FACTOR_LOAD,
             batched.FACTOR_LOAD, batched.FACTOR_COMPUTE, batched.FACTOR_LOAD]
    again = batched.spd_solve_ragged_mixed(
        rb, tol=TOL, factors=batched.FactorPlan(modes, [f if m else None for m, f in
                                                        zip(modes, store)], dev))
    torch.cuda.synchronize()
    for r in (first, again):
        assert torch.equal(r.x, plain.x) and torch.equal(r.iters, plain.iters)
        assert torch.equal(r.info, plain.info) and torch.equal(r.berr, plain.berr)
    for s, n in enumerate(ns):
        u = store[s].double().cpu().numpy()
        u_ref = dense.cho_factor_upper(mats[s])
        assert np.all(np.tril(u, -1) == 0)
        assert np.abs(u - u_ref).max() <= 1e-4 * np.abs(u_ref).max()


def test_mixed_factors_rejects_missing_pointers(dev):
    rng = np.random.default_rng(32)
    mats, rhs = make_ragged(rng, [20], [1])
    rb = to_batch(mats, rhs, dev)
    ws = batched.MixedWorkspace(rb.batch, rb.max_n, rb.max_nrhs, dev)
    out = torch.empty_like(rb.b)
    small = torch.empty(1, dtype=torch.int32, device=dev)
    with pytest.raises(_ffi.LxgbError) as e:
        _ffi.call("lxgb_posv_ragged_mixed_factors", rb.batch, rb.max_n, rb.max_nrhs,
                  _ffi.ptr(rb.n), _ffi.ptr(rb.nrhs), _ffi.ptr(rb.a_off), _ffi.ptr(rb.a),
                  _ffi.ptr(rb.b_off), _ffi.ptr(rb.b), _ffi.ptr(out), TOL, 10, _ffi.ptr(small),
                  _ffi.ptr(small), _ffi.ptr(out), 0, 0, _ffi.ptr(ws.buf), ws.nbytes,
                  _ffi.stream_handle(dev))
    assert e.value.status == 100


@pytest.mark.parametrize("ns", [[145, 200, 300, 512, 400, 64], [544, 160, 33]])
def test_mixed_tensor_core_update(dev, ns):
    """The large-system factor's trailing updates on the tcgen05 tensor cores
    (split TF32 products): every system reaches the 1e-12 backward error bar
    and agrees with the oracle's solution, as with the CUDA-core updates."""
    rng = np.random.default_rng(sum(ns) + 5)
    ks = [1 + (5 * i) % 8 for i in range(len(ns))]
    mats, rhs = make_ragged(rng, ns, ks)
    rb = to_batch(mats, rhs, dev)
    _ffi.call("lxgb_posv_mixed_set_tensor_cores", 1)
    try:
        res = batched.spd_solve_ragged_mixed(rb, tol=TOL)
        torch.cuda.synchronize()
    finally:
        _ffi.call("lxgb_posv_mixed_set_tensor_cores", 0)
    ref = batched.spd_solve_ragged_mixed(rb, tol=TOL)
    assert (res.info.cpu().numpy() == 0).all()
    assert (res.iters.cpu().numpy() <= ref.iters.cpu().numpy() + 1).all()
    for s, (m, r) in enumerate(zip(mats, rhs)):
        xs = rb.system_b(res.x, s).cpu().numpy()
        be = dense.backward_errors_exact(m, xs, r)
        assert (be <= TOL * (1 + 1e-4)).all(), (ns[s], be)
        x_ref = dense.cholesky_linear_solve(m, r.T).T
        for c in range(ks[s]):
            assert dense.forward_error(xs[c], x_ref[c]) <= 1e-9
