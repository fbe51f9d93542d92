"""Batched and ragged solves: the vmapped and ragged forms of lineax's LU and
Cholesky solves, and the mixed-precision SPD solve with FP64 refinement.

* ``lu_solve_batched(A, b)`` — equal-size batch, FP64 LU (the form
  ``jax.vmap(lambda A, b: lx.linear_solve(lx.MatrixLinearOperator(A), b,
  lx.LU()).value)`` evaluates).
* ``RaggedBatch`` — a ragged batch packed into one buffer with per-system
  offsets (the layout of the C ABI), built once from lists of tensors.
* ``cholesky_solve_ragged(batch)`` — plain FP64 potrf + potrs.
* ``spd_solve_ragged_mixed(batch, tol)`` — FP32 factor + FP64 iterative
  refinement to a normwise backward error <= tol, in one persistent launch.
"""

from __future__ import annotations

import dataclasses

import torch

from . import _dense, _ffi, autotune
from ._blas import as_device_f64


def lu_solve_batched(a: torch.Tensor, b: torch.Tensor, trans: int = 0):
    """x[i] = A[i]^{-1} b[i] (or A[i]^{-T} b[i]) for a (batch, n, n) FP64 stack.
    b is (batch, n) or (batch, nrhs, n).  Returns (x, info)."""
    lu, piv, info = _dense.lu_factor_batched(a)
    return _dense.lu_solve_batched(lu, piv, b, trans), info


@dataclasses.dataclass
class RaggedBatch:
    """Systems of different orders packed back to back.

    a: packed FP64 matrices (row-major), a_off[s] the start of system s.
    b: packed right-hand sides, system s holds nrhs[s] vectors of length n[s]
    from b_off[s].  n/nrhs/a_off/b_off live on the device; the host copies
    (n_host, nrhs_host) size launches.
    """

    a: torch.Tensor
    b: torch.Tensor
    n: torch.Tensor
    nrhs: torch.Tensor
    a_off: torch.Tensor
    b_off: torch.Tensor
    n_host: list
    nrhs_host: list
    a_off_host: list
    b_off_host: list

    @property
    def batch(self) -> int:
        return len(self.n_host)

    @property
    def max_n(self) -> int:
        return max(self.n_host) if self.n_host else 0

    @property
    def max_nrhs(self) -> int:
        return max(self.nrhs_host) if self.nrhs_host else 0

    @staticmethod
    def layout(n_list, nrhs_list):
        a_off, b_off, ao, bo = [], [], 0, 0
        for n, k in zip(n_list, nrhs_list):
            a_off.append(ao)
            b_off.append(bo)
            ao += n * n
            bo += n * k
        return a_off, b_off, ao, bo

    @classmethod
    def from_packed(cls, a, b, n_list, nrhs_list, device="cuda"):
        """Wrap already-packed device buffers (a: Σn², b: Σn·nrhs)."""
        a_off, b_off, ta, tb = cls.layout(n_list, nrhs_list)
        if a.numel() != ta or b.numel() != tb:
            raise ValueError("packed buffer sizes do not match the ragged layout")
        meta_i32 = torch.tensor([list(n_list), list(nrhs_list)], dtype=torch.int32)
        meta_i64 = torch.tensor([a_off, b_off], dtype=torch.int64)
        meta_i32 = meta_i32.to(device)
        meta_i64 = meta_i64.to(device)
        return cls(a, b, meta_i32[0], meta_i32[1], meta_i64[0], meta_i64[1], list(n_list),
                   list(nrhs_list), a_off, b_off)

    @classmethod
    def from_lists(cls, matrices, rhs, device="cuda"):
        """matrices[s]: (n, n); rhs[s]: (n,) or (nrhs, n)."""
        n_list = [int(m.shape[0]) for m in matrices]
        nrhs_list = [1 if r.ndim == 1 else int(r.shape[0]) for r in rhs]
        a = torch.cat([m.reshape(-1).to(torch.float64) for m in matrices]).to(device)
        b = torch.cat([r.reshape(-1).to(torch.float64) for r in rhs]).to(device)
        return cls.from_packed(a, b, n_list, nrhs_list, device)

    def system_b(self, x: torch.Tensor, s: int) -> torch.Tensor:
        """View of system s in a buffer with the layout of b: (nrhs, n)."""
        n, k, o = self.n_host[s], self.nrhs_host[s], self.b_off_host[s]
        return x[o : o + n * k].view(k, n)

    def system_a(self, s: int) -> torch.Tensor:
        n, o = self.n_host[s], self.a_off_host[s]
        return self.a[o : o + n * n].view(n, n)


def cholesky_factor_ragged(batch: RaggedBatch):
    """Plain FP64 upper Cholesky of every system (a copy of batch.a).
    Returns (factors packed like batch.a, info)."""
    u = as_device_f64(batch.a).clone()
    info = torch.empty(batch.batch, dtype=torch.int32, device=u.device)
    _ffi.call("lxgb_potrf_ragged_f64", batch.batch, batch.max_n, _ffi.ptr(batch.n),
              _ffi.ptr(batch.a_off), _ffi.ptr(u), _ffi.ptr(info), _ffi.stream_handle(u.device))
    return u, info


def cholesky_solve_ragged(batch: RaggedBatch, factors: torch.Tensor | None = None):
    """Plain FP64 Cholesky solve of a ragged batch (the FP64 GPU baseline).
    Returns (x packed like batch.b, info)."""
    if factors is None:
        factors, info = cholesky_factor_ragged(batch)
    else:
        info = torch.zeros(batch.batch, dtype=torch.int32, device=factors.device)
    x = as_device_f64(batch.b).clone()
    _ffi.call("lxgb_potrs_ragged_f64", batch.batch, batch.max_n, _ffi.ptr(batch.n),
              _ffi.ptr(batch.nrhs), _ffi.ptr(batch.a_off), _ffi.ptr(factors),
              _ffi.ptr(batch.b_off), _ffi.ptr(x), _ffi.stream_handle(x.device))
    return x, info


@dataclasses.dataclass
class MixedResult:
    x: torch.Tensor      # solutions, packed like batch.b
    info: torch.Tensor   # per system: 0 ok, k+1 FP32 breakdown, -1 not converged
    iters: torch.Tensor  # FP32 solves applied per system
    berr: torch.Tensor   # largest normwise backward error per system


class MixedWorkspace:
    """Caller-side scratch of lxgb_posv_ragged_mixed, reusable across calls
    (kept by the serving loop and by CUDA-graph captures)."""

    def __init__(self, batch: int, max_n: int, max_nrhs: int, device="cuda"):
        autotune.ensure_applied(device)
        nbytes = _ffi.load().lxgb_posv_ragged_mixed_workspace_size(batch, max_n, max_nrhs)
        self.nbytes = int(nbytes)
        # 256-byte alignment: torch's caching allocator returns 512-byte aligned blocks.
        self.buf = torch.empty(self.nbytes, dtype=torch.uint8, device=device)
        self.batch, self.max_n, self.max_nrhs = batch, max_n, max_nrhs

    def fits(self, batch: int, max_n: int, max_nrhs: int) -> bool:
        need = _ffi.load().lxgb_posv_ragged_mixed_workspace_size(batch, max_n, max_nrhs)
        return need <= self.nbytes


# fmode values of lxgb_posv_ragged_mixed_factors
FACTOR_COMPUTE, FACTOR_STORE, FACTOR_LOAD = 0, 1, 2


class FactorPlan:
    """Per-system factor handling of a mixed ragged solve: for each system
    FACTOR_COMPUTE (None), FACTOR_STORE (an empty n×n FP32 device tensor that
    receives the factor) or FACTOR_LOAD (a tensor holding a stored factor)."""

    def __init__(self, modes, tensors, device):
        ptrs = [0 if t is None else t.data_ptr() for t in tensors]
        for m, t in zip(modes, tensors):
            if m != FACTOR_COMPUTE and (t is None or t.dtype != torch.float32
                                        or not t.is_contiguous()):
                raise ValueError("stored factors are contiguous FP32 device tensors")
        self.tensors = list(tensors)  # keeps the factors alive while the call runs
        self.fmode = torch.tensor(list(modes), dtype=torch.int32).to(device, non_blocking=True)
        self.fptr = torch.tensor(ptrs, dtype=torch.int64).to(device, non_blocking=True)


def spd_solve_ragged_mixed(batch: RaggedBatch, tol: float = 1e-12, max_iter: int = 10,
                           workspace: MixedWorkspace | None = None,
                           out: MixedResult | None = None,
                           factors: FactorPlan | None = None) -> MixedResult:
    """FP32-factor / FP64-refined solve of every SPD system of the batch.
    With `factors`, systems store their FP32 factor for later calls or reuse
    a stored one instead of factoring (lxgb_posv_ragged_mixed_factors)."""
    dev = batch.a.device
    autotune.ensure_applied(dev)
    if workspace is None or not workspace.fits(batch.batch, batch.max_n, batch.max_nrhs):
        workspace = MixedWorkspace(batch.batch, batch.max_n, batch.max_nrhs, dev)
    if out is None:
        out = MixedResult(
            x=torch.empty_like(batch.b, dtype=torch.float64),
            info=torch.empty(batch.batch, dtype=torch.int32, device=dev),
            iters=torch.empty(batch.batch, dtype=torch.int32, device=dev),
            berr=torch.empty(batch.batch, dtype=torch.float64, device=dev),
        )
    common = (batch.batch, batch.max_n, batch.max_nrhs,
              _ffi.ptr(batch.n), _ffi.ptr(batch.nrhs), _ffi.ptr(batch.a_off),
              _ffi.ptr(batch.a), _ffi.ptr(batch.b_off), _ffi.ptr(batch.b), _ffi.ptr(out.x),
              float(tol), int(max_iter), _ffi.ptr(out.info), _ffi.ptr(out.iters),
              _ffi.ptr(out.berr))
    if factors is None:
        _ffi.call("lxgb_posv_ragged_mixed", *common, _ffi.ptr(workspace.buf), workspace.nbytes,
                  _ffi.stream_handle(dev))
    else:
        _ffi.call("lxgb_posv_ragged_mixed_factors", *common, _ffi.ptr(factors.fmode),
                  _ffi.ptr(factors.fptr), _ffi.ptr(workspace.buf), workspace.nbytes,
                  _ffi.stream_handle(dev))
    return out


class CapturedMixedSolve:
    """The mixed-precision ragged solve (queue reset + one persistent
    posv_mixed_kernel launch) captured once in a CUDA graph for a fixed batch,
    workspace and output, then replayed: repeated solves of a resident batch
    cost one graph launch.  The library holds no state between calls, so the
    captured launch reads whatever the batch's buffers hold at replay time."""

    def __init__(self, batch: RaggedBatch, tol: float = 1e-12, max_iter: int = 10,
                 workspace: MixedWorkspace | None = None, out: MixedResult | None = None):
        dev = batch.a.device
        if workspace is None:
            workspace = MixedWorkspace(batch.batch, batch.max_n, batch.max_nrhs, dev)
        self.batch, self.workspace = batch, workspace
        # first call outside the capture: sets the kernel's shared-memory limit
        self.out = spd_solve_ragged_mixed(batch, tol, max_iter, workspace, out)
        torch.cuda.synchronize(dev)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            spd_solve_ragged_mixed(batch, tol, max_iter, workspace, self.out)

    def replay(self) -> MixedResult:
        self.graph.replay()
        return self.out


def chunk_bounds(sizes, chunks: int) -> list:
    """Boundaries [0, b1, ..., len(sizes)] of at most `chunks` contiguous,
    non-empty ranges of about equal total size (a range closes once the
    running total reaches its share)."""
    nb = len(sizes)
    k = max(1, min(int(chunks), nb))
    total = float(sum(sizes)) or 1.0
    bounds, acc = [0], 0
    for s, sz in enumerate(sizes):
        acc += sz
        if len(bounds) < k and acc >= total * len(bounds) / k and s + 1 < nb:
            bounds.append(s + 1)
    bounds.append(nb)
    return bounds


class _HostSet:
    """One set of device buffers of HostRaggedSPDSolver (matrices, right-hand
    sides, results), cut into chunks."""

    def __init__(self, n_list, nrhs_list, chunks: int, device):
        a_off, b_off, ta, tb = RaggedBatch.layout(n_list, nrhs_list)
        nb = len(n_list)
        self.a_dev = torch.empty(ta, dtype=torch.float64, device=device)
        self.b_dev = torch.empty(tb, dtype=torch.float64, device=device)
        self.out = MixedResult(
            x=torch.empty(tb, dtype=torch.float64, device=device),
            info=torch.empty(nb, dtype=torch.int32, device=device),
            iters=torch.empty(nb, dtype=torch.int32, device=device),
            berr=torch.empty(nb, dtype=torch.float64, device=device),
        )
        bounds = chunk_bounds([n * n + n * r for n, r in zip(n_list, nrhs_list)], chunks)
        self.chunks = []
        for lo, hi in zip(bounds[:-1], bounds[1:]):
            a0, b0 = a_off[lo], b_off[lo]
            a1 = a_off[hi] if hi < nb else ta
            b1 = b_off[hi] if hi < nb else tb
            sub = RaggedBatch.from_packed(self.a_dev[a0:a1], self.b_dev[b0:b1],
                                          list(n_list[lo:hi]), list(nrhs_list[lo:hi]), device)
            res = MixedResult(x=self.out.x[b0:b1], info=self.out.info[lo:hi],
                              iters=self.out.iters[lo:hi], berr=self.out.berr[lo:hi])
            self.chunks.append((lo, hi, a0, a1, b0, b1, sub, res))
        self.copied = [torch.cuda.Event() for _ in self.chunks]
        self.released = torch.cuda.Event()   # the last solve that read this set
        self.used = False


class HostRaggedSPDSolver:
    """Solve ragged SPD batches whose data lives in host memory.

    Device buffers, metadata and the workspace are allocated once for a fixed
    layout (n_list, nrhs_list); each call copies the matrices and right-hand
    sides in from (pinned) host tensors, runs the mixed-precision solve, and
    copies solutions and per-system status back into host tensors.  Calls are
    asynchronous (stream-ordered on the caller's current stream): read the
    results, or change the host inputs, after synchronising.

    Overlap: host-to-device copies run on a side stream.  With `buffers` >= 2
    device buffer sets, calls rotate through them, so the copy of call k+1
    runs while call k is solved (a set is refilled once the solve that last
    read it has finished).  With `chunks` > 1 the systems of a call are also
    cut into contiguous ranges of about equal bytes, and the solve of chunk j
    waits only for chunk j's copy.  A system's result does not depend on
    either setting.
    """

    def __init__(self, n_list, nrhs_list, tol: float = 1e-12, max_iter: int = 10,
                 device="cuda", chunks: int = 1, buffers: int = 2):
        self.sets = [_HostSet(n_list, nrhs_list, chunks, device) for _ in range(max(1, buffers))]
        first = self.sets[0]
        self.out, self.chunks = first.out, first.chunks
        self.batch = RaggedBatch.from_packed(first.a_dev, first.b_dev, n_list, nrhs_list, device)
        self.tol, self.max_iter = tol, max_iter
        nb = len(n_list)
        self.h2d_bytes = (first.a_dev.numel() + first.b_dev.numel()) * 8
        self.d2h_bytes = first.b_dev.numel() * 8 + nb * (4 + 4 + 8)
        self.ws = MixedWorkspace(max(c[6].batch for c in first.chunks),
                                 max(c[6].max_n for c in first.chunks),
                                 max(c[6].max_nrhs for c in first.chunks), device)
        self.copy_stream = torch.cuda.Stream(device=device)
        self.calls = 0

    def __call__(self, a_host: torch.Tensor, b_host: torch.Tensor, x_host: torch.Tensor,
                 info_host: torch.Tensor, iters_host: torch.Tensor, berr_host: torch.Tensor):
        st = self.sets[self.calls % len(self.sets)]
        self.calls += 1
        main = torch.cuda.current_stream(st.a_dev.device)
        if st.used:
            self.copy_stream.wait_event(st.released)
        else:
            self.copy_stream.wait_stream(main)
            st.used = True
        with torch.cuda.stream(self.copy_stream):
            for (lo, hi, a0, a1, b0, b1, sub, res), ev in zip(st.chunks, st.copied):
                st.a_dev[a0:a1].copy_(a_host[a0:a1], non_blocking=True)
                st.b_dev[b0:b1].copy_(b_host[b0:b1], non_blocking=True)
                ev.record(self.copy_stream)
        for (lo, hi, a0, a1, b0, b1, sub, res), ev in zip(st.chunks, st.copied):
            main.wait_event(ev)
            spd_solve_ragged_mixed(sub, self.tol, self.max_iter, self.ws, res)
            x_host[b0:b1].copy_(res.x, non_blocking=True)
            info_host[lo:hi].copy_(res.info, non_blocking=True)
            iters_host[lo:hi].copy_(res.iters, non_blocking=True)
            berr_host[lo:hi].copy_(res.berr, non_blocking=True)
        st.released.record(main)
