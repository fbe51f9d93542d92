"""Continuous-batching solve server on one GPU.

Requests are dense square systems A X = B (1 to 16 right-hand sides) tagged
with the lineax solver the client asked for (LU, Cholesky or QR) and an
operator id; a request may omit A and reuse an operator the server has seen.
What a solver's `init` produces for an operator (its factor state, the
object lineax reuses when `linear_solve` is given `state`,
lineax/_solve.py:785-790) stays resident in device memory under an LRU
policy, so a request on a resident operator skips the factorisation.  Each
scheduling round admits the queued requests that have arrived, first come
first served, while their device footprint plus the resident operators fits
the HBM budget, and runs them grouped by route:

  chol_ragged  Cholesky requests with n <= 1024: one launch of the ragged
               mixed-precision SPD kernel (FP32 factor, FP64-accurate
               refinement) for the whole group, new operators storing their
               FP32 factor and resident ones loading it instead of factoring
               (lxgb_posv_ragged_mixed_factors); systems it does not solve to
               the tolerance are re-solved by FP64 LU.  FP64 mode: the ragged
               FP64 Cholesky for new operators, the resident FP64 factor's
               solve for the others.
  lu_small     LU requests with n <= 168: batched FP64 LU, one launch per
               distinct order (each system's arithmetic is the same as alone;
               right-hand-side blocks are zero padded, and each vector is
               solved independently).
  lu_mixed     LU requests with n >= 512 (MIXED_MIN_N; between 169 and 511
               the mixed server uses lu_f64, which is faster there): FP32 LU
               with 3xTF32 tensor-core
               updates, its triangular inverses, refinement to FP64 backward
               error (lineax_gb300.mixed: plain refinement, then GMRES-IR, then
               FP64 LU when refinement stalls); factor, inverses and the split
               A stay resident.
  chol_mixed   Cholesky requests with n > 1024: FP32 Cholesky with 3xTF32
               tensor-core updates (no pivoting, lower-triangle trailing
               updates), L'⁻¹ on the tensor cores and U'⁻¹ by a transposing
               copy, then the same refinement; an operator that is not
               positive definite in FP32 is factored by the mixed LU instead.
  qr_mixed     QR requests with n >= 512: FP32 Householder QR with TF32
               tensor-core updates and Q formed explicitly, R^{-1} on the
               tensor cores, GMRES-IR preconditioned by R^{-1} Qᵀ (FP64 QR
               when refinement stalls); Qᵀ, R^{-1} and the split A stay
               resident.
  qr_f64       QR requests with n < 512 (both modes) and every QR request in
               FP64 mode: FP64 Householder QR (lineax's QR solver), the
               factor resident.
  lu_f64 / chol_f64   LU above n = 168 (in mixed mode up to 511) and, in FP64
               mode, Cholesky above 1024 (multi-CTA FP64 factor): the plain
               FP64 GPU path with resident factors.

Serving is continuous: run() keeps admitting requests as they arrive and as
memory frees up while earlier work is still on the GPU.  Admitted work goes
to a pool of worker threads, each with its own CUDA stream (a ragged
Cholesky group or a small-LU group is one job, each large request is one
job), so requests overlap on the device; a job's device memory is released
back to the admission budget when it completes.  A resident operator made on
one worker's stream carries a CUDA event recorded after its factorisation;
a job on another stream waits on that event before it reads the operator and
marks the operator's tensors as used by its stream (record_stream), so
neither an unfinished factor nor freed memory is ever read.

mode="fp64" serves the same requests with the plain FP64 GPU path of this
library on one stream: the denominator of the mixed path's speed-up.  Every
completion carries its normwise backward error; a request's result does not
depend on what else was in its batch or on whether its operator was
resident.
"""

from __future__ import annotations

import collections
import concurrent.futures
import dataclasses
import threading
import time

import torch

from . import _blas, _dense, _ffi, batched, mixed

KINDS = ("lu", "cholesky", "qr")
SMALL_LU_MAX = 168      # one CTA per system, matrix in shared memory
RAGGED_CHOL_MAX = 1024  # the ragged mixed-precision Cholesky kernel's limit
# Below this order the FP64 LU and QR finish a request sooner than the mixed
# path's factor, inverses and refinement (measured on GB300 by order bucket:
# 169-255 LU 1.05 vs 1.85 ms, QR 2.7 vs 4.5 ms; 256-511 LU 2.05 vs 2.5 ms, QR
# 4.4 vs 4.6 ms; from 512 the mixed path wins), so the mixed server sends
# those requests to the FP64 routes.
MIXED_MIN_N = 512


@dataclasses.dataclass
class Request:
    rid: int
    kind: str                         # "lu", "cholesky" or "qr"
    b: torch.Tensor                   # (nrhs, n) FP64, host or device
    op_id: int                        # operator identity (reuse key)
    a: torch.Tensor | None = None     # (n, n) FP64; None: the registered operator op_id
    arrival: float = 0.0              # seconds after the start of the run

    @property
    def n(self) -> int:
        return int(self.b.shape[-1])

    @property
    def nrhs(self) -> int:
        return 1 if self.b.ndim == 1 else int(self.b.shape[0])


@dataclasses.dataclass
class Completion:
    rid: int
    x: torch.Tensor       # (nrhs, n) FP64 on the device
    berr: float           # max normwise backward error over the right-hand sides
    route: str
    fallback: bool        # re-solved by the FP64 path after refinement stalled
    reused: bool          # served from a resident factor
    finished: float = 0.0
    latency: float = 0.0


def route_of(kind: str, n: int, mode: str) -> str:
    if kind not in KINDS:
        raise ValueError(f"unknown request kind {kind!r}")
    if kind == "cholesky":
        if n <= RAGGED_CHOL_MAX:
            return "chol_ragged"
        return "chol_mixed" if mode == "mixed" else "chol_f64"
    if kind == "qr":
        return "qr_mixed" if (mode == "mixed" and n >= MIXED_MIN_N) else "qr_f64"
    if n <= SMALL_LU_MAX:
        return "lu_small"
    return "lu_mixed" if (mode == "mixed" and n >= MIXED_MIN_N) else "lu_f64"


def footprint(route: str, n: int, nrhs: int) -> int:
    """Device bytes a request holds while it is being served."""
    vec = 8 * 8 * n * max(nrhs, 1)  # b, x, residual and workspace vectors
    n4 = (n + 3) // 4 * 4
    if route == "chol_ragged":
        return resident_bytes(route, n) + 4 * n * n + vec   # + the packed copy of A
    if route == "lu_small":
        return 3 * 8 * SMALL_LU_MAX * SMALL_LU_MAX + vec
    if route in ("lu_f64", "chol_f64", "qr_f64"):
        return resident_bytes(route, n) + vec
    if route == "qr_mixed":
        return resident_bytes(route, n) + 20 * n4 * n4 + vec  # h, q, R, inversion work
    return resident_bytes(route, n) + 5 * 4 * 64 * n4 + vec


def resident_bytes(route: str, n: int) -> int:
    """Bytes of what stays resident for an operator between requests."""
    n4 = (n + 3) // 4 * 4
    if route in ("lu_mixed", "chol_mixed"):
        # A (FP64), FP32 factor, both triangular inverses, A as a hi + lo pair
        return 8 * n4 * n4 + 4 * n4 * n4 + 8 * n4 * n4 + 8 * n4 * n4
    if route == "qr_mixed":
        # A (FP64), A as a hi + lo pair, Qᵀ and R^{-1} (FP32)
        return 8 * n4 * n4 + 8 * n4 * n4 + 4 * n4 * n4 + 4 * n4 * n4
    if route == "chol_ragged":
        return 8 * n * n + 8 * n * n  # A and its factor (FP32 mixed, FP64 plain: the larger)
    if route in ("lu_f64", "chol_f64", "qr_f64"):
        return 2 * 8 * n * n + 8 * 32 * n  # A and its FP64 factor (+ QR's T blocks)
    return 8 * n * n          # the operator itself


class Scheduler:
    """First-come-first-served admission under a device-memory budget, with
    an LRU cache of resident operators charged against the same budget.  Host
    logic only: the server supplies what is resident and what it costs."""

    def __init__(self, budget_bytes: int, mode: str = "mixed"):
        self.budget = int(budget_bytes)
        self.mode = mode
        self.queue: collections.deque = collections.deque()
        self.resident: collections.OrderedDict = collections.OrderedDict()
        self.resident_total = 0
        self.inflight = 0          # bytes held by admitted, unfinished requests
        self.rejected: list = []
        self.lock = threading.RLock()

    def submit(self, req: Request) -> None:
        self.queue.append(req)

    def pending(self) -> int:
        return len(self.queue)

    def next_arrival(self):
        return self.queue[0].arrival if self.queue else None

    def _evict_for(self, need: int, pinned: set) -> None:
        for op_id in list(self.resident):
            if self.resident_total + self.inflight + need <= self.budget:
                return
            if op_id in pinned:
                continue
            nbytes, _ = self.resident.pop(op_id)
            self.resident_total -= nbytes

    def admit(self, now: float) -> list:
        """Requests that have arrived by `now`, in order, while they fit
        beside the resident operators and the work still in flight; their
        footprints stay charged until release()."""
        with self.lock:
            batch, used, pinned = [], 0, set()
            while self.queue and self.queue[0].arrival <= now:
                req = self.queue[0]
                route = route_of(req.kind, req.n, self.mode)
                need = footprint(route, req.n, req.nrhs)
                if req.op_id in self.resident:  # its resident part is already charged
                    need = max(need - self.resident[req.op_id][0], 0)
                self._evict_for(used + need, pinned | {req.op_id})
                if self.resident_total + self.inflight + used + need > self.budget:
                    if not batch and self.inflight == 0 and need > self.budget:
                        self.rejected.append(self.queue.popleft())  # can never fit
                        continue
                    break
                batch.append(self.queue.popleft())
                req._charge = need
                used += need
                pinned.add(req.op_id)
            self.inflight += used
            return batch

    def release(self, reqs) -> None:
        """Return the footprints of finished requests to the budget."""
        with self.lock:
            for r in reqs:
                self.inflight -= getattr(r, "_charge", 0)
                r._charge = 0

    def lookup(self, op_id):
        with self.lock:
            hit = self.resident.get(op_id)
            if hit is None:
                return None
            self.resident.move_to_end(op_id)
            return hit[1]

    def forget(self, op_id) -> None:
        """Drop a resident operator (its factor turned out unusable)."""
        with self.lock:
            hit = self.resident.pop(op_id, None)
            if hit is not None:
                self.resident_total -= hit[0]

    def remember(self, op_id, nbytes: int, payload) -> None:
        with self.lock:
            if op_id in self.resident:
                self.resident_total -= self.resident.pop(op_id)[0]
            self._evict_for(nbytes, {op_id})
            if self.resident_total + self.inflight + nbytes <= self.budget:
                self.resident[op_id] = (int(nbytes), payload)
                self.resident_total += int(nbytes)


def _check_pipeline(err) -> None:
    """Raise if a tensor-core pipeline wait of the request's factorisation
    gave up (the flag is read after the refinement has synchronised)."""
    if err is not None and int(err.item()) != 0:
        raise RuntimeError("tensor-core pipeline timed out while factoring a request")


def _pad_identity(a: torch.Tensor, n_to: int) -> torch.Tensor:
    n = a.shape[0]
    if n == n_to:
        return a.contiguous()
    out = torch.zeros((n_to, n_to), dtype=torch.float64, device=a.device)
    out[:n, :n] = a
    idx = torch.arange(n, n_to, device=a.device)
    out[idx, idx] = 1.0
    return out


def _berr(a: torch.Tensor, x: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """Per-vector normwise backward error (device), FP64 residual."""
    r = _blas.gemv(a, x, alpha=-1.0, beta=1.0, out=b.clone())
    anorm = mixed.norm_inf(a)
    return r.abs().amax(dim=1) / (anorm * x.abs().amax(dim=1) + b.abs().amax(dim=1))


class _Resident:
    """What stays on the device for an operator: `a` (the FP64 operator,
    padded where the route pads) and the route's factor tensors.  `ready`
    is a CUDA event recorded on the creating stream after the factorisation
    was issued."""

    def __init__(self, a: torch.Tensor, **parts):
        self.a = a
        self.parts = parts
        self.ready = None

    def __getattr__(self, name):
        parts = self.__dict__.get("parts", {})
        if name in parts:
            return parts[name]
        raise AttributeError(name)

    def tensors(self):
        out = [self.a]
        for v in self.parts.values():
            if isinstance(v, torch.Tensor):
                out.append(v)
            elif dataclasses.is_dataclass(v):
                out += [getattr(v, f.name) for f in dataclasses.fields(v)
                        if isinstance(getattr(v, f.name), torch.Tensor)]
            elif isinstance(v, tuple):
                out += [t for t in v if isinstance(t, torch.Tensor)]
        return out


class SolveServer:
    """Serve Requests on one GPU (see the module docstring)."""

    def __init__(self, device="cuda", mode: str = "mixed", hbm_budget: int = 64 << 30,
                 tol: float = 1e-12, precision: str = "3xtf32", streams: int | None = None):
        if mode not in ("mixed", "fp64"):
            raise ValueError("mode must be 'mixed' or 'fp64'")
        self.device = torch.device(device)
        if self.device.index is None:
            self.device = torch.device(self.device.type, torch.cuda.current_device())
        self.mode = mode
        self.tol = tol
        self.precision = precision
        self.streams = streams if streams is not None else (4 if mode == "mixed" else 1)
        self.sched = Scheduler(hbm_budget, mode)
        self.registry: dict = {}  # op_id -> host FP64 matrix (the client's copy)
        self._tls = threading.local()  # per worker thread: its stream and workspace

    def register(self, op_id, a_host: torch.Tensor) -> None:
        self.registry[op_id] = a_host

    # -- resident operators ----------------------------------------------------

    def _acquire(self, op_id):
        """The resident operator op_id, made safe to read on this thread's
        stream (waits for its factorisation, pins its memory), or None."""
        res = self.sched.lookup(op_id)
        if res is None:
            return None
        st = torch.cuda.current_stream(self.device)
        if res.ready is not None:
            st.wait_event(res.ready)
        for t in res.tensors():
            t.record_stream(st)
        return res

    def _publish(self, op_id, route: str, n: int, res: _Resident) -> None:
        """Make a new resident operator visible to other streams: record the
        event that orders its factorisation before any later reader."""
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(self.device))
        res.ready = ev
        self.sched.remember(op_id, resident_bytes(route, n), res)

    def _check_or_forget(self, err, op_id) -> None:
        """The request's pipeline flag (see _check_pipeline); on a timeout the
        factor it published is dropped, so later requests on the operator
        factor it again.  (A request that acquired it meanwhile still ends
        correct: its refinement falls back to FP64 when it stalls.)"""
        try:
            _check_pipeline(err)
        except RuntimeError:
            self.sched.forget(op_id)
            raise

    # -- execution ------------------------------------------------------------

    def _matrix(self, req: Request) -> torch.Tensor:
        a = req.a if req.a is not None else self.registry[req.op_id]
        if req.a is not None:
            self.registry.setdefault(req.op_id, req.a)
        return a.to(self.device, torch.float64, non_blocking=True)

    def _rhs(self, req: Request) -> torch.Tensor:
        b = req.b.reshape(req.nrhs, req.n)
        return b.to(self.device, torch.float64, non_blocking=True).contiguous()

    def _fp64_lu(self, a: torch.Tensor, b: torch.Tensor):
        lu, piv = _dense.lu_factor(a)
        return _dense.lu_solve(lu, piv, b), lu, piv

    def _run_chol(self, reqs: list) -> list:
        if self.mode == "fp64":
            return self._run_chol_f64(reqs)
        found = [self._acquire(r.op_id) for r in reqs]
        mats = [res.a if res is not None else self._matrix(r) for r, res in zip(reqs, found)]
        rhs = [self._rhs(r) for r in reqs]
        rb = batched.RaggedBatch.from_lists(mats, rhs, device=self.device)
        modes, ftens = [], []
        for res, r in zip(found, reqs):
            if res is not None:
                modes.append(batched.FACTOR_LOAD)
                ftens.append(res.factor)
            else:
                modes.append(batched.FACTOR_STORE)
                ftens.append(torch.empty((r.n, r.n), dtype=torch.float32, device=self.device))
        plan = batched.FactorPlan(modes, ftens, self.device)
        ws = getattr(self._tls, "ws", None)
        if ws is None or not ws.fits(rb.batch, rb.max_n, rb.max_nrhs):
            ws = batched.MixedWorkspace(rb.batch, rb.max_n, rb.max_nrhs, self.device)
            self._tls.ws = ws
        res_k = batched.spd_solve_ragged_mixed(rb, tol=self.tol, workspace=ws, factors=plan)
        info = res_k.info.cpu().tolist()
        berr = res_k.berr.cpu().tolist()
        out = []
        for s, req in enumerate(reqs):
            x = rb.system_b(res_k.x, s).clone()
            reused = found[s] is not None
            if info[s] != 0 or not berr[s] <= self.tol:
                x, _, _ = self._fp64_lu(mats[s], rhs[s])
                e = float(_berr(mats[s], x, rhs[s]).max())
                out.append(Completion(req.rid, x, e, "chol_ragged", True, reused))
                continue
            if not reused:
                self._publish(req.op_id, "chol_ragged", req.n,
                              _Resident(mats[s], factor=ftens[s]))
            out.append(Completion(req.rid, x, berr[s], "chol_ragged", False, reused))
        return out

    def _run_chol_f64(self, reqs: list) -> list:
        """Plain FP64: one ragged potrf launch for the new operators, then one
        ragged potrs launch for every request, resident operators with their
        stored FP64 factor (the same solve kernel either way)."""
        found = [self._acquire(r.op_id) for r in reqs]
        rhs = [self._rhs(r) for r in reqs]
        mats = [res.a if res is not None else self._matrix(r) for r, res in zip(reqs, found)]
        us = [res.u if res is not None else None for res in found]
        fallback = [False] * len(reqs)
        fresh = [s for s, res in enumerate(found) if res is None]
        if fresh:
            rbf = batched.RaggedBatch.from_lists([mats[s] for s in fresh],
                                                 [rhs[s] for s in fresh], device=self.device)
            u, info = batched.cholesky_factor_ragged(rbf)
            info = info.cpu().tolist()
            for j, s in enumerate(fresh):
                n, off = reqs[s].n, rbf.a_off_host[j]
                us[s] = u[off: off + n * n].view(n, n).clone()
                fallback[s] = info[j] != 0
        ok = [s for s in range(len(reqs)) if not fallback[s]]
        xs = [None] * len(reqs)
        if ok:
            rb = batched.RaggedBatch.from_lists([mats[s] for s in ok], [rhs[s] for s in ok],
                                                device=self.device)
            x, _ = batched.cholesky_solve_ragged(
                rb, torch.cat([us[s].reshape(-1) for s in ok]))
            for j, s in enumerate(ok):
                xs[s] = rb.system_b(x, j).clone()
                if found[s] is None:
                    self._publish(reqs[s].op_id, "chol_ragged", reqs[s].n,
                                  _Resident(mats[s], u=us[s]))
        for s in range(len(reqs)):
            if fallback[s]:
                xs[s], _, _ = self._fp64_lu(mats[s], rhs[s])
        errs = torch.stack([_berr(mats[s], xs[s], rhs[s]).max() for s in range(len(reqs))])
        errs = errs.cpu().tolist()
        return [Completion(r.rid, xs[s], errs[s], "chol_ragged", fallback[s],
                           found[s] is not None) for s, r in enumerate(reqs)]

    def _run_small(self, reqs: list) -> list:
        mats = [self._matrix(r) for r in reqs]
        rhs = [self._rhs(r) for r in reqs]
        xs = [None] * len(reqs)
        by_n = collections.defaultdict(list)
        for s, r in enumerate(reqs):
            by_n[r.n].append(s)
        for n, idx in by_n.items():  # one batched launch per order
            kmax = max(reqs[s].nrhs for s in idx)
            a = torch.stack([mats[s] for s in idx])
            b = torch.zeros((len(idx), kmax, n), dtype=torch.float64, device=self.device)
            for j, s in enumerate(idx):
                b[j, : reqs[s].nrhs] = rhs[s]
            lu, piv, _ = _dense.lu_factor_batched(a)
            x = _dense.lu_solve_batched(lu, piv, b)
            for j, s in enumerate(idx):
                xs[s] = x[j, : reqs[s].nrhs].contiguous()
        errs = torch.stack([_berr(mats[s], xs[s], rhs[s]).max() for s in range(len(reqs))])
        errs = errs.cpu().tolist()
        return [Completion(r.rid, xs[s], errs[s], "lu_small", False, False)
                for s, r in enumerate(reqs)]

    def _padded_rhs(self, req: Request, n4: int) -> torch.Tensor:
        b = self._rhs(req)
        if n4 == req.n:
            return b
        return torch.cat([b, torch.zeros((req.nrhs, n4 - req.n), dtype=torch.float64,
                                         device=b.device)], 1)

    def _run_mixed(self, req: Request) -> Completion:
        res = self._acquire(req.op_id)
        reused = res is not None
        n4 = (req.n + 3) // 4 * 4
        err = None
        if res is None:
            # one pipeline flag for the request, read after the refinement's
            # own synchronisation: the host keeps enqueueing meanwhile
            err = torch.zeros(1, dtype=torch.int32, device=self.device)
            ap = _pad_identity(self._matrix(req), n4)
            f = mixed.lu_factor_tf32(ap, self.precision, err=err)
            res = _Resident(ap, factor=f, inverse=mixed.lu_inverse(f, self.precision, err=err),
                            split=mixed.split_matrix(ap))
            self._publish(req.op_id, "lu_mixed", req.n, res)
        ir = mixed.gmres_ir(res.a, self._padded_rhs(req, n4), tol=self.tol, max_outer=20,
                            inner_max_steps=5, restart=8, factor=res.factor,
                            inverse=res.inverse, split=res.split, precision=self.precision,
                            arith="auto", fallback=True)
        self._check_or_forget(err, req.op_id)
        x = ir.x[:, : req.n].contiguous()
        return Completion(req.rid, x, max(ir.berr), "lu_mixed", ir.fallback, reused)

    def _run_chol_mixed(self, req: Request) -> Completion:
        res = self._acquire(req.op_id)
        reused = res is not None
        n4 = (req.n + 3) // 4 * 4
        err = None
        if res is None:
            err = torch.zeros(1, dtype=torch.int32, device=self.device)
            ap = _pad_identity(self._matrix(req), n4)
            f = mixed.cholesky_factor_tf32(ap, err=err)
            if int(f.info.item()) == 0:
                inv = mixed.cholesky_inverse(f, err=err)
            else:  # not positive definite in FP32: the mixed LU instead
                f = mixed.lu_factor_tf32(ap, self.precision, err=err)
                inv = mixed.lu_inverse(f, self.precision, err=err)
            res = _Resident(ap, factor=f, inverse=inv, split=mixed.split_matrix(ap))
            self._publish(req.op_id, "chol_mixed", req.n, res)
        ir = mixed.gmres_ir(res.a, self._padded_rhs(req, n4), tol=self.tol, max_outer=20,
                            inner_max_steps=5, restart=8, factor=res.factor,
                            inverse=res.inverse, split=res.split, precision=self.precision,
                            arith="auto", fallback=True)
        self._check_or_forget(err, req.op_id)
        x = ir.x[:, : req.n].contiguous()
        return Completion(req.rid, x, max(ir.berr), "chol_mixed", ir.fallback, reused)

    def _run_qr_mixed(self, req: Request) -> Completion:
        res = self._acquire(req.op_id)
        reused = res is not None
        n4 = (req.n + 3) // 4 * 4
        err = None
        if res is None:
            err = torch.zeros(1, dtype=torch.int32, device=self.device)
            ap = _pad_identity(self._matrix(req), n4)
            res = _Resident(ap, qr=mixed.qr_square_tf32(ap, err=err), split=mixed.split_matrix(ap))
            self._publish(req.op_id, "qr_mixed", req.n, res)
        ir = mixed.gmres_ir(res.a, self._padded_rhs(req, n4), tol=self.tol, max_outer=20,
                            inner_max_steps=5, restart=8, split=res.split, qr=res.qr,
                            arith="auto", fallback=True)
        self._check_or_forget(err, req.op_id)
        x = ir.x[:, : req.n].contiguous()
        return Completion(req.rid, x, max(ir.berr), "qr_mixed", ir.fallback, reused)

    def _run_f64(self, req: Request, route: str) -> Completion:
        """The plain FP64 GPU path of lineax's solvers: LU (getrf/getrs),
        Cholesky (multi-CTA potrf, triangular solves) or Householder QR
        (geqrf/ormqr/trsm), the factor resident for later requests."""
        res = self._acquire(req.op_id)
        reused = res is not None
        if res is None:
            a = self._matrix(req)
            if route == "lu_f64":
                lu, piv = _dense.lu_factor(a)
                res = _Resident(a, lu=lu, piv=piv)
            elif route == "chol_f64":
                res = _Resident(a, u=_dense.cho_factor(a))
            else:
                res = _Resident(a, qr=_dense.geqrf(a))
            self._publish(req.op_id, route, req.n, res)
        b = self._rhs(req)
        if route == "lu_f64":
            x = _dense.lu_solve(res.lu, res.piv, b)
        elif route == "chol_f64":
            x = _dense.cho_solve(res.u, b)
        else:
            x = mixed.qr_solve_f64(res.qr, b)
        return Completion(req.rid, x, float(_berr(res.a, x, b).max()), route, False, reused)

    def _jobs(self, batch: list) -> list:
        """Admitted requests as jobs: one per ragged Cholesky group, one per
        small-LU group, one per other request."""
        groups = collections.defaultdict(list)
        for r in batch:
            groups[route_of(r.kind, r.n, self.mode)].append(r)
        jobs = []
        if groups["chol_ragged"]:
            jobs.append((self._run_chol, groups["chol_ragged"]))
        if groups["lu_small"]:
            jobs.append((self._run_small, groups["lu_small"]))
        for r in groups["lu_mixed"]:
            jobs.append((lambda rs: [self._run_mixed(rs[0])], [r]))
        for r in groups["chol_mixed"]:
            jobs.append((lambda rs: [self._run_chol_mixed(rs[0])], [r]))
        for r in groups["qr_mixed"]:
            jobs.append((lambda rs: [self._run_qr_mixed(rs[0])], [r]))
        for route in ("lu_f64", "chol_f64", "qr_f64"):
            for r in groups[route]:
                jobs.append((lambda rs, rt=route: [self._run_f64(rs[0], rt)], [r]))
        return jobs

    def execute(self, batch: list) -> list:
        """Serve one admitted batch on the current stream (synchronises
        before returning)."""
        out = []
        for fn, reqs in self._jobs(batch):
            out += fn(reqs)
        torch.cuda.synchronize(self.device)
        return out

    def _work(self, fn, reqs, t0: float):
        """One job on this worker thread's stream; returns its completions
        stamped with the time the device finished them."""
        st = getattr(self._tls, "stream", None)
        if st is None:
            st = torch.cuda.Stream(self.device)
            self._tls.stream = st
        with torch.cuda.device(self.device), torch.cuda.stream(st):
            out = fn(reqs)
            st.synchronize()
        t = time.perf_counter() - t0
        for c in out:
            c.finished = t
        return out

    def run(self, requests: list, realtime: bool = True) -> list:
        """Serve requests whose `arrival` times are seconds after the start
        (open loop: arrivals do not wait for completions).  Admission keeps
        running while admitted work is on the GPU; jobs run on `streams`
        worker threads with one CUDA stream each.  Returns the completions in
        request-id order with finish times and latencies."""
        for r in sorted(requests, key=lambda q: q.arrival):
            # A request carrying its matrix registers the client's copy when
            # it is sent, so a later request on the same operator finds it
            # even if it executes first (its worker may run ahead of the
            # defining request's worker).
            if r.a is not None:
                self.registry.setdefault(r.op_id, r.a)
            self.sched.submit(r)
        arrival = {r.rid: r.arrival for r in requests}
        done = {}
        t0 = time.perf_counter()
        inflight = {}
        with concurrent.futures.ThreadPoolExecutor(max_workers=self.streams) as pool:
            while self.sched.pending() or inflight:
                now = time.perf_counter() - t0 if realtime else float("inf")
                batch = self.sched.admit(now) if self.sched.pending() else []
                for fn, reqs in self._jobs(batch):
                    inflight[pool.submit(self._work, fn, reqs, t0)] = reqs
                if batch:
                    continue
                if not inflight:
                    nxt = self.sched.next_arrival()
                    if nxt is None:
                        break
                    if nxt > now:
                        time.sleep(min(nxt - now, 0.002))
                        continue
                    raise MemoryError("a request does not fit the HBM budget")
                nxt = self.sched.next_arrival()
                timeout = None if nxt is None else max(0.0, min(nxt - now, 0.002))
                finished, _ = concurrent.futures.wait(
                    list(inflight), timeout=timeout,
                    return_when=concurrent.futures.FIRST_COMPLETED)
                for f in finished:
                    reqs = inflight.pop(f)
                    self.sched.release(reqs)
                    for c in f.result():
                        c.latency = c.finished - arrival[c.rid]
                        done[c.rid] = c
        return [done[k] for k in sorted(done)]


def synthetic_requests(count: int, seed: int = 0, nmin: int = 32, nmax: int = 4096,
                       reuse: float = 0.3, rate: float | None = None, mix=(0.5, 0.3, 0.2),
                       device=None):
    """The serving mix: kinds LU/Cholesky/QR with probabilities `mix`, n
    log-uniform on [nmin, nmax], 1-16 right-hand sides, a fraction `reuse`
    of requests on an operator seen before (no matrix sent), Poisson arrivals
    at `rate` per second (all at t = 0 when rate is None).  Matrices as in the
    single-workload benchmarks: Cholesky operators G Gᵀ/n + 1e-2 I (the ragged
    SPD workload), the others G/sqrt(n) + I (the batched-LU workload), with G
    i.i.d. N(0,1) from a per-operator seed.  Built on `device` when given (the
    G Gᵀ products of large orders), returned as host tensors."""
    import numpy as np

    rng = np.random.default_rng([seed, 0x5E7])
    reqs, ops, t = [], [], 0.0
    for rid in range(count):
        if rate:
            t += float(rng.exponential(1.0 / rate))
        if ops and rng.random() < reuse:
            op_id, kind, n = ops[int(rng.integers(len(ops)))]
            a = None
        else:
            kind = KINDS[int(rng.choice(3, p=list(mix)))]
            n = int(np.clip(np.floor(np.exp(rng.uniform(np.log(nmin), np.log(nmax + 1)))),
                            nmin, nmax))
            op_id = len(ops)
            gen = torch.Generator(device=device or "cpu").manual_seed(seed * 1_000_003 + op_id)
            g = torch.randn(n, n, dtype=torch.float64, device=device or "cpu", generator=gen)
            eye = torch.eye(n, dtype=torch.float64, device=g.device)
            a = (g @ g.T / n + 1e-2 * eye) if kind == "cholesky" else (g / np.sqrt(n) + eye)
            a = a.cpu()
            ops.append((op_id, kind, n))
        k = int(rng.integers(1, 17))
        b = torch.from_numpy(rng.standard_normal((k, n)))
        reqs.append(Request(rid, kind, b, op_id, a, t))
    return reqs
