"""Host drivers of the device Krylov solvers (CG, GMRES, BiCGStab) for a
block of k right-hand sides.

The loop structure restates lineax/_solver/cg.py:114-227 and
lineax/_solver/gmres.py:106-413; every vector operation and reduction of the
loop body runs in liblxgb.so (lxgb_cg_* / lxgb_gmres_*).  Operator and
preconditioner products are formed here: MatrixLinearOperator through
lxgb_gemv_f64, operators with a ``mv_block`` method (e.g. the Poisson stencil)
on a whole (k, n) block, and other FunctionLinearOperators through torch.vmap
(vector by vector when the function cannot be batched).
Each right-hand side has device-side flags, so the host checks convergence
only every few iterations; iterations past a right-hand side's stop leave it
untouched, which makes every right-hand side's result the same as when it is
solved alone.

When the operator and preconditioner are dense matrices or the Poisson
stencil (possibly negated), cg_run / gmres_run make one call of the
single-call entry points (lxgb_cg_run / lxgb_gmres_run): the same launch
sequence replayed by a CUDA graph's conditional while loop on the device,
with no host round trip until the solve ends.
"""

from __future__ import annotations

import ctypes
import dataclasses

import torch

from . import _blas, _ffi
from ._operator import IdentityLinearOperator, MatrixLinearOperator
from ._structure import ravel, tree_flatten

SUCCESSFUL, MAX_STEPS_REACHED, SINGULAR, BREAKDOWN, STAGNATION = 0, 1, 2, 3, 4
EPS64 = 2.220446049250313e-16


def _stream(dev) -> int:
    return _ffi.stream_handle(dev)


def _work(nbytes: int, dev) -> torch.Tensor:
    """FP64-typed scratch of at least nbytes (torch's caching allocator returns
    512-byte aligned blocks, as the workspaces require)."""
    return torch.empty(max(int(nbytes), 256) // 8 + 1, dtype=torch.float64, device=dev)


def block_mv(operator, x: torch.Tensor) -> torch.Tensor:
    """operator applied to each row of the (k, n) float64 block x."""
    if isinstance(operator, IdentityLinearOperator):
        return x
    if isinstance(operator, MatrixLinearOperator):
        return _blas.gemv(operator.matrix, x)
    if hasattr(operator, "mv_block"):
        return operator.mv_block(x)
    from ._operator import apply_columns

    return apply_columns(operator, x).to(torch.float64).contiguous()


def device_operator(operator):
    """(lxgb_linear_operator, tensors to keep alive) for operators the
    single-call device loops apply themselves — dense matrices and the
    Poisson stencil, possibly negated — or None (then the host drives the
    loop and calls the operator every iteration)."""
    from ._operator import NegLinearOperator, Poisson2DOperator

    sign, op = 1.0, operator
    while isinstance(op, NegLinearOperator):
        sign, op = -sign, op.operator
    if isinstance(op, Poisson2DOperator):
        d = _ffi.LinearOperatorDesc(kind=_ffi.OP_POISSON5, n=op.nx * op.ny, nx=op.nx, ny=op.ny,
                                    scale=sign * op.scale)
        return d, ()
    if isinstance(op, MatrixLinearOperator):
        m = _blas.as_device_f64(op.matrix)
        if m.ndim != 2 or m.shape[0] != m.shape[1] or m.stride(1) != 1:
            m = m.contiguous()
        if m.shape[0] != m.shape[1]:
            return None
        d = _ffi.LinearOperatorDesc(kind=_ffi.OP_DENSE, n=m.shape[0], a=m.data_ptr(),
                                    lda=m.stride(0), scale=sign)
        return d, (m,)
    return None


def _run_results(steps_d, res_d):
    return steps_d.cpu().tolist(), res_d.cpu().tolist()


def cg_run(operator, b: torch.Tensor, *, rtol: float, atol: float, max_steps=None,
           stabilise_every=10, preconditioner=None, y0: torch.Tensor | None = None):
    """CG through the single-call entry point lxgb_cg_run (the loop on the
    device), or None when the operator or preconditioner cannot be described
    to it (the caller then runs cg_block)."""
    od = device_operator(operator)
    pd = device_operator(preconditioner) if preconditioner is not None else (None, ())
    every = 0 if stabilise_every is None else int(stabilise_every)
    if od is None or pd is None or not 0 <= every <= 64:
        return None
    b = _blas.as_device_f64(b)
    if b.ndim == 1:
        b = b.reshape(1, -1)
    b = b.contiguous()
    k, n = b.shape
    if od[0].n != n:
        return None
    dev = b.device
    y = torch.empty_like(b) if y0 is None else _blas.as_device_f64(y0).reshape(k, n).clone()
    lib = _ffi.load()
    has_pre = pd[0] is not None
    work = _work(int(lib.lxgb_cg_run_workspace_size(k, n, int(has_pre))), dev)
    steps_d = torch.empty(k, dtype=torch.int32, device=dev)
    res_d = torch.empty(k, dtype=torch.int32, device=dev)
    desc, pdesc = od[0], pd[0]
    _ffi.call("lxgb_cg_run", k, n, ctypes.addressof(desc),
              ctypes.addressof(pdesc) if has_pre else None, _ffi.ptr(b), _ffi.ptr(y),
              int(y0 is not None), float(rtol), float(atol),
              -1 if max_steps is None else int(max_steps), every, _ffi.ptr(steps_d),
              _ffi.ptr(res_d), _ffi.ptr(work), work.numel() * 8, _stream(dev))
    steps, results = _run_results(steps_d, res_d)
    return KrylovResult(y, steps, results)


def gmres_run(operator, b: torch.Tensor, *, rtol: float, atol: float, max_steps=None,
              restart=20, stagnation_iters=20, preconditioner=None,
              y0: torch.Tensor | None = None):
    """GMRES through lxgb_gmres_run (the loop on the device), or None when
    the operator or preconditioner cannot be described to it."""
    od = device_operator(operator)
    pd = device_operator(preconditioner) if preconditioner is not None else (None, ())
    if od is None or pd is None:
        return None
    b = _blas.as_device_f64(b)
    if b.ndim == 1:
        b = b.reshape(1, -1)
    b = b.contiguous()
    k, n = b.shape
    if od[0].n != n or min(int(restart), n) > 128:
        return None
    dev = b.device
    y = torch.empty_like(b) if y0 is None else _blas.as_device_f64(y0).reshape(k, n).clone()
    lib = _ffi.load()
    R = min(int(restart), n)
    work = _work(int(lib.lxgb_gmres_run_workspace_size(k, n, R)), dev)
    steps_d = torch.empty(k, dtype=torch.int32, device=dev)
    res_d = torch.empty(k, dtype=torch.int32, device=dev)
    desc, pdesc = od[0], pd[0]
    _ffi.call("lxgb_gmres_run", k, n, ctypes.addressof(desc),
              ctypes.addressof(pdesc) if pdesc is not None else None, _ffi.ptr(b),
              _ffi.ptr(y), int(y0 is not None), float(rtol), float(atol),
              -1 if max_steps is None else int(max_steps), R, int(stagnation_iters),
              _ffi.ptr(steps_d), _ffi.ptr(res_d), _ffi.ptr(work), work.numel() * 8,
              _stream(dev))
    steps, results = _run_results(steps_d, res_d)
    return KrylovResult(y, steps, results)


def _check_schedule(it: int) -> bool:
    """Iterations after which the host reads the flags: every iteration for the
    first 8, then every 8th (stopped right-hand sides are frozen meanwhile)."""
    return it < 8 or (it + 1) % 8 == 0


@dataclasses.dataclass
class KrylovResult:
    y: torch.Tensor          # (k, n) solutions
    steps: list              # per right-hand side
    results: list            # RESULTS codes per right-hand side


def cg_block(operator, b: torch.Tensor, *, rtol: float, atol: float, max_steps=None,
             stabilise_every=10, preconditioner=None, y0: torch.Tensor | None = None
             ) -> KrylovResult:
    """CG on the (k, n) block b (operator positive definite)."""
    b = _blas.as_device_f64(b)
    if b.ndim == 1:
        b = b.reshape(1, -1)
    k, n = b.shape
    dev = b.device
    size = n
    max_steps_ = 10 * size if max_steps is None else int(max_steps)
    has_scale = not (atol == 0 and rtol == 0)
    rcond = 2 * EPS64 * size  # lineax/_misc.py:30-38
    pre = preconditioner if preconditioner is not None else None
    y = (torch.zeros_like(b) if y0 is None else _blas.as_device_f64(y0).reshape(k, n).clone())
    wbytes = int(_ffi.load().lxgb_cg_workspace_size(k, n))
    work = _work(wbytes, dev)
    st = _stream(dev)
    r = (b - block_mv(operator, y)).contiguous() if y0 is not None else b.clone()
    z = block_mv(pre, r).contiguous() if pre is not None else r
    p = torch.empty_like(b)
    _ffi.call("lxgb_cg_start", k, n, _ffi.ptr(r), _ffi.ptr(z), _ffi.ptr(p), max_steps_,
              int(has_scale), _ffi.ptr(work), work.numel() * 8, st)
    steps_d = torch.empty(k, dtype=torch.int32, device=dev)
    act_d = torch.empty(k, dtype=torch.int32, device=dev)

    def status(parity):
        _ffi.call("lxgb_cg_status", k, n, parity, _ffi.ptr(steps_d), _ffi.ptr(act_d),
                  _ffi.ptr(work), work.numel() * 8, st)
        return steps_d.cpu().tolist(), act_d.cpu().tolist()

    _, act = status(0)
    it = 0
    while any(act) and it < max_steps_:
        par = it & 1
        mat_p = block_mv(operator, p)
        step_no = it + 1
        if stabilise_every == 1:
            stable = True
        elif stabilise_every is None:
            stable = False
        else:
            stable = step_no % stabilise_every == 0
        _ffi.call("lxgb_cg_step_alpha", k, n, _ffi.ptr(mat_p), _ffi.ptr(p), _ffi.ptr(y),
                  _ffi.ptr(r), int(not stable), par, float(rtol), float(atol), rcond,
                  _ffi.ptr(work), work.numel() * 8, st)
        if stable:
            ay = block_mv(operator, y)
            _ffi.call("lxgb_cg_true_residual", k, n, _ffi.ptr(b), _ffi.ptr(ay), _ffi.ptr(r),
                      par, _ffi.ptr(work), work.numel() * 8, st)
        z = block_mv(pre, r).contiguous() if pre is not None else r
        _ffi.call("lxgb_cg_step_beta", k, n, _ffi.ptr(b), _ffi.ptr(r), _ffi.ptr(z), _ffi.ptr(p),
                  par, max_steps_, int(has_scale), float(rtol), float(atol), _ffi.ptr(work),
                  work.numel() * 8, st)
        if _check_schedule(it):
            _, act = status(par ^ 1)
        it += 1
    steps, _ = status(it & 1)
    results = []
    for s in steps:
        if max_steps is None:
            results.append(SINGULAR if s == max_steps_ else SUCCESSFUL)
        elif has_scale:
            results.append(MAX_STEPS_REACHED if s == max_steps_ else SUCCESSFUL)
        else:
            results.append(SUCCESSFUL)
    return KrylovResult(y, steps, results)


def cg_poisson_mixed(operator, b: torch.Tensor, *, rtol: float, atol: float, max_steps=None,
                     check: int = 16, y0: torch.Tensor | None = None) -> KrylovResult:
    """CG on a Poisson2DOperator (scale 1) for the (k, n) block b with FP32
    iterations and an FP64 residual replacement every `check` iterations
    (lxgb_cg32_*): the stopping test is lineax's max-norm test on the FP64
    true residual, evaluated at the replacements.  HBM traffic per iteration
    is that of FP32 vectors; the FP64 pipe sees only the replacements."""
    if getattr(operator, "scale", None) != 1.0 or not hasattr(operator, "nx"):
        raise ValueError("the mixed-precision CG needs a Poisson2DOperator with scale 1")
    b = _blas.as_device_f64(b)
    if b.ndim == 1:
        b = b.reshape(1, -1)
    b = b.contiguous()
    k, n = b.shape
    nx, ny = operator.nx, operator.ny
    if nx * ny != n:
        raise ValueError("right-hand side length does not match the grid")
    dev = b.device
    max_steps_ = 10 * n if max_steps is None else int(max_steps)
    x = torch.zeros_like(b) if y0 is None else _blas.as_device_f64(y0).reshape(k, n).clone()
    xlo = torch.zeros((k, n), dtype=torch.float32, device=dev)
    r = torch.empty((k, n), dtype=torch.float32, device=dev)
    p = torch.empty_like(r)
    ap = torch.empty_like(r)
    wbytes = int(_ffi.load().lxgb_cg32_workspace_size(k))
    work = _work(wbytes, dev)
    st = _stream(dev)
    wb = work.numel() * 8
    stat = torch.empty((k, 3), dtype=torch.int32, device=dev)
    _ffi.call("lxgb_cg32_init", k, nx, ny, max_steps_, _ffi.ptr(work), wb, st)
    _ffi.call("lxgb_cg32_refresh", k, nx, ny, _ffi.ptr(b), _ffi.ptr(x), _ffi.ptr(xlo), _ffi.ptr(r),
              float(rtol), float(atol), max_steps_, _ffi.ptr(work), wb, st)
    _ffi.call("lxgb_cg32_start_direction", k, n, _ffi.ptr(r), _ffi.ptr(p), st)
    done = 0
    while True:
        _ffi.call("lxgb_cg32_status", k, _ffi.ptr(stat), _ffi.ptr(work), wb, st)
        rows = stat.cpu().tolist()
        if not any(row[0] for row in rows):
            break
        iters = max(1, min(int(check), max_steps_ - done))
        _ffi.call("lxgb_cg32_iterate", k, nx, ny, iters, _ffi.ptr(p), _ffi.ptr(ap), _ffi.ptr(xlo),
                  _ffi.ptr(r), _ffi.ptr(work), wb, st)
        done += iters
        _ffi.call("lxgb_cg32_refresh", k, nx, ny, _ffi.ptr(b), _ffi.ptr(x), _ffi.ptr(xlo),
                  _ffi.ptr(r), float(rtol), float(atol), max_steps_, _ffi.ptr(work), wb, st)
    results, steps = [], []
    for _, s_, conv in rows:
        if conv == 1:
            res = SUCCESSFUL
        elif conv == 2:
            res = SINGULAR
        else:
            res = SINGULAR if max_steps is None else MAX_STEPS_REACHED
        results.append(res)
        steps.append(s_)
    return KrylovResult(x, steps, results)


def gmres_block(operator, b: torch.Tensor, *, rtol: float, atol: float, max_steps=None,
                restart=20, stagnation_iters=20, preconditioner=None,
                y0: torch.Tensor | None = None) -> KrylovResult:
    """Restarted GMRES on the (k, n) block b."""
    b = _blas.as_device_f64(b)
    if b.ndim == 1:
        b = b.reshape(1, -1)
    k, n = b.shape
    dev = b.device
    size = n
    max_steps_ = 10 * size if max_steps is None else int(max_steps)
    has_scale = not (atol == 0 and rtol == 0)
    R = min(int(restart), size)
    if R > 128:
        raise ValueError("lineax_gb300 GMRES supports restart <= 128")
    lib = _ffi.load()
    wbytes = int(lib.lxgb_gmres_workspace_size(k, n, R))
    work = _work(wbytes, dev)
    st = _stream(dev)
    pre = preconditioner

    def mpre(x):
        return block_mv(pre, x).contiguous() if pre is not None else x

    y = torch.zeros_like(b) if y0 is None else _blas.as_device_f64(y0).reshape(k, n).clone()
    r = torch.zeros_like(b)
    diff = torch.full_like(b, float("inf"))
    on = torch.empty(k, dtype=torch.int32, device=dev)
    stat = torch.empty((k, 5), dtype=torch.int32, device=dev)
    _ffi.call("lxgb_gmres_init", k, n, R, _ffi.ptr(work), work.numel() * 8, st)
    work_f64 = work
    base_off = [int(lib.lxgb_gmres_basis_offset(k, n, R, kk)) // 8 for kk in range(R + 1)]

    def status(parity):
        _ffi.call("lxgb_gmres_status", k, n, R, parity, _ffi.ptr(stat), _ffi.ptr(work),
                  work.numel() * 8, st)
        return stat.cpu().tolist()

    it = 0
    while True:
        par = it & 1
        first = it == 0
        if not first:
            _ffi.call("lxgb_gmres_cycle_begin", k, n, R, par, _ffi.ptr(r), _ffi.ptr(work),
                      work.numel() * 8, st)
            for kk in range(R):
                vk = torch.as_strided(work_f64, (k, n), ((R + 1) * n, 1), base_off[kk])
                w = mpre(block_mv(operator, vk)).contiguous()
                if w.data_ptr() == vk.data_ptr():
                    w = w.clone()
                _ffi.call("lxgb_gmres_arnoldi", k, n, R, par, kk, _ffi.ptr(w), _ffi.ptr(on),
                          _ffi.ptr(work), work.numel() * 8, st)
        _ffi.call("lxgb_gmres_cycle_end", k, n, R, par, int(first), _ffi.ptr(y), _ffi.ptr(diff),
                  _ffi.ptr(work), work.numel() * 8, st)
        t = mpre((b - block_mv(operator, y)).contiguous()).contiguous()
        _ffi.call("lxgb_gmres_outer", k, n, R, par, int(first), _ffi.ptr(b), _ffi.ptr(t),
                  _ffi.ptr(r), _ffi.ptr(diff), _ffi.ptr(y), float(rtol), float(atol), max_steps_,
                  int(stagnation_iters), int(has_scale), _ffi.ptr(work), work.numel() * 8, st)
        it += 1
        rows = status(it & 1)
        if not any(row[0] for row in rows) or it >= max_steps_ + 1:
            break
    results, steps = [], []
    for active, s, stag, deferred, nc in rows:
        if max_steps is None:
            res = SINGULAR if s == max_steps_ else SUCCESSFUL
        elif has_scale:
            res = MAX_STEPS_REACHED if s == max_steps_ else SUCCESSFUL
        else:
            res = SUCCESSFUL
        if stag >= stagnation_iters:
            res = STAGNATION
        if deferred and nc:
            res = BREAKDOWN
        results.append(res)
        steps.append(s)
    return KrylovResult(y, steps, results)


def bicgstab_block(operator, b: torch.Tensor, *, rtol: float, atol: float, max_steps=None,
                   preconditioner=None, y0: torch.Tensor | None = None) -> KrylovResult:
    """BiCGStab (lineax/_solver/bicgstab.py:78-205) on the (k, n) block b,
    right-preconditioned; every vector update and reduction in liblxgb.so
    (lxgb_bicgstab_*), operator and preconditioner products here."""
    b = _blas.as_device_f64(b)
    if b.ndim == 1:
        b = b.reshape(1, -1)
    k, n = b.shape
    dev = b.device
    max_steps_ = 10 * n if max_steps is None else int(max_steps)   # :82-88
    has_scale = not (atol == 0 and rtol == 0)
    pre = preconditioner
    y = (torch.zeros_like(b) if y0 is None else _blas.as_device_f64(y0).reshape(k, n).clone())
    r = (b - block_mv(operator, y)).contiguous() if y0 is not None else b.clone()  # :105
    r0 = torch.empty_like(b)
    p = torch.empty_like(b)
    v = torch.empty_like(b)
    s_ = torch.empty_like(b)
    wbytes = int(_ffi.load().lxgb_bicgstab_workspace_size(k, n))
    work = _work(wbytes, dev)
    wb = work.numel() * 8
    st = _stream(dev)
    _ffi.call("lxgb_bicgstab_start", k, n, _ffi.ptr(r), _ffi.ptr(r0), _ffi.ptr(p), _ffi.ptr(v),
              max_steps_, int(has_scale), _ffi.ptr(work), wb, st)
    steps_d = torch.empty(k, dtype=torch.int32, device=dev)
    act_d = torch.empty(k, dtype=torch.int32, device=dev)
    scal_d = torch.empty(3 * k, dtype=torch.float64, device=dev)
    nc_d = torch.empty(k, dtype=torch.int32, device=dev)

    def active():
        _ffi.call("lxgb_bicgstab_status", k, n, 0, _ffi.ptr(act_d), 0, 0, _ffi.ptr(work), wb, st)
        return act_d.cpu().tolist()

    act = active()
    it = 0
    while any(act) and it < max_steps_:
        _ffi.call("lxgb_bicgstab_direction", k, n, _ffi.ptr(r0), _ffi.ptr(r), _ffi.ptr(v),
                  _ffi.ptr(p), _ffi.ptr(work), wb, st)
        x = block_mv(pre, p).contiguous() if pre is not None else p
        v = block_mv(operator, x).contiguous()
        _ffi.call("lxgb_bicgstab_s", k, n, _ffi.ptr(r0), _ffi.ptr(r), _ffi.ptr(v), _ffi.ptr(s_),
                  _ffi.ptr(work), wb, st)
        z = block_mv(pre, s_).contiguous() if pre is not None else s_
        t = block_mv(operator, z).contiguous()
        _ffi.call("lxgb_bicgstab_update", k, n, _ffi.ptr(x), _ffi.ptr(z), _ffi.ptr(s_),
                  _ffi.ptr(t), _ffi.ptr(b), _ffi.ptr(y), _ffi.ptr(r), float(rtol), float(atol),
                  max_steps_, int(has_scale), _ffi.ptr(work), wb, st)
        if _check_schedule(it):
            act = active()
        it += 1
    _ffi.call("lxgb_bicgstab_status", k, n, _ffi.ptr(steps_d), 0, _ffi.ptr(scal_d),
              _ffi.ptr(nc_d), _ffi.ptr(work), wb, st)
    steps = steps_d.cpu().tolist()
    scal = scal_d.cpu().view(3, k).tolist()
    ncs = nc_d.cpu().tolist()
    results = []
    for c in range(k):                                               # :188-202
        if max_steps is None:
            res = SINGULAR if steps[c] == max_steps_ else SUCCESSFUL
        elif has_scale:
            res = MAX_STEPS_REACHED if steps[c] == max_steps_ else SUCCESSFUL
        else:
            res = SUCCESSFUL
        rho, alpha, omega = scal[0][c], scal[1][c], scal[2][c]
        if (omega == 0.0 or alpha == 0.0 or rho == 0.0) and ncs[c]:
            res = BREAKDOWN
        results.append(res)
    return KrylovResult(y, steps, results)


def vector_block(vector):
    """(k=1, n) float64 block of a lineax vector PyTree, and its structure."""
    leaves, _ = tree_flatten(vector)
    flat = ravel(vector, torch.float64).contiguous()
    return flat.reshape(1, -1), leaves
