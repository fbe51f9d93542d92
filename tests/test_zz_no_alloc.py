"""GPU: the allocation-free mixed-precision SPD entry point.

lxgb_posv_ragged_mixed_noalloc serves callers that cannot allocate device
memory when they solve (an XLA FFI handler, a serving loop that forbids
allocation after start-up): its scratch is a fixed array inside the library.
This file is collected last so that a run stopping at the first failure has
already run every other test; it passes alone in a fresh process too.
"""

import numpy as np
import pytest
import torch

from lineax_gb300 import _ffi, batched
from oracle import dense

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _case(dev):
    rng = np.random.default_rng(99)
    ns = [512, 300, 225, 224, 100, 33, 16]
    ks = [3, 1, 8, 2, 5, 1, 4]
    mats, rhs = [], []
    for n, k in zip(ns, ks):
        g = rng.standard_normal((n, n))
        mats.append(g @ g.T / n + 1e-2 * np.eye(n))
        rhs.append(rng.standard_normal((k, n)))
    rb = batched.RaggedBatch.from_lists([torch.tensor(m) for m in mats],
                                        [torch.tensor(r) for r in rhs], device=dev)
    return rb, mats, rhs


def _noalloc(rb):
    dev = rb.a.device
    out = batched.MixedResult(
        x=torch.full_like(rb.b, float("nan")),
        info=torch.full((rb.batch,), 7, dtype=torch.int32, device=dev),
        iters=torch.zeros(rb.batch, dtype=torch.int32, device=dev),
        berr=torch.full((rb.batch,), float("nan"), dtype=torch.float64, device=dev),
    )
    _ffi.call("lxgb_posv_ragged_mixed_noalloc", rb.batch, rb.max_n, rb.max_nrhs,
              _ffi.ptr(rb.n), _ffi.ptr(rb.nrhs), _ffi.ptr(rb.a_off), _ffi.ptr(rb.a),
              _ffi.ptr(rb.b_off), _ffi.ptr(rb.b), _ffi.ptr(out.x), TOL, 10,
              _ffi.ptr(out.info), _ffi.ptr(out.iters), _ffi.ptr(out.berr),
              _ffi.stream_handle(dev))
    torch.cuda.synchronize()
    return out


def test_noalloc_matches_workspace_entry_twice(dev):
    rb, mats, rhs = _case(dev)
    ref = batched.spd_solve_ragged_mixed(rb, tol=TOL)
    torch.cuda.synchronize()
    for _ in range(2):  # two calls in a row: the shared scratch is reused
        got = _noalloc(rb)
        assert torch.equal(got.info, ref.info) and int(got.info.abs().sum()) == 0
        assert torch.equal(got.iters, ref.iters)
        x_ref = ref.x.cpu().numpy()
        x_got = got.x.cpu().numpy()
        for s in range(rb.batch):
            o, n, k = rb.b_off_host[s], rb.n_host[s], rb.nrhs_host[s]
            xs = x_got[o: o + n * k].reshape(k, n)
            xr = x_ref[o: o + n * k].reshape(k, n)
            for j in range(k):
                assert dense.backward_error(mats[s], xs[j], rhs[s][j]) <= TOL
                assert dense.forward_error(xs[j], xr[j]) <= 1e-10
        assert (got.berr.cpu().numpy() <= TOL).all()


def test_noalloc_rejects_oversize(dev):
    # Real device buffers of a small batch, so that the call could only ever
    # touch valid memory even if the size check moved after a launch.
    rb, _, _ = _case(dev)
    out_x = torch.zeros_like(rb.b)
    info = torch.zeros(rb.batch, dtype=torch.int32, device=dev)
    iters = torch.zeros(rb.batch, dtype=torch.int32, device=dev)
    berr = torch.zeros(rb.batch, dtype=torch.float64, device=dev)
    with pytest.raises(_ffi.LxgbError) as e:
        _ffi.call("lxgb_posv_ragged_mixed_noalloc", rb.batch, 4096, rb.max_nrhs,
                  _ffi.ptr(rb.n), _ffi.ptr(rb.nrhs), _ffi.ptr(rb.a_off), _ffi.ptr(rb.a),
                  _ffi.ptr(rb.b_off), _ffi.ptr(rb.b), _ffi.ptr(out_x), TOL, 10,
                  _ffi.ptr(info), _ffi.ptr(iters), _ffi.ptr(berr), _ffi.stream_handle(dev))
    assert e.value.status == 100
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0  # nothing was launched
