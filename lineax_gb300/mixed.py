"""Mixed-precision LU with GMRES-IR.

The factor is computed in FP32 with partial pivoting and tensor-core (TF32)
trailing updates (lxgb_getrf_f32_tc); FP64 GMRES on the original operator,
left-preconditioned by the FP32 LU solve, recovers FP64 accuracy (GMRES-based
iterative refinement, Carson & Higham 2017).  Through the lineax API this is

    M = lu_preconditioner(operator)
    lx.linear_solve(operator, b, lx.GMRES(rtol, atol, restart=20),
                    options={"preconditioner": M})

the preconditioned-GMRES call path of lineax/_solver/gmres.py:106-240 with an
LU (lineax/_solver/lu.py) as the preconditioner.
"""

from __future__ import annotations

import dataclasses

import torch

from . import _ffi, _krylov
from ._blas import as_device_f64
from ._operator import AbstractLinearOperator, MatrixLinearOperator
from ._structure import ShapeDtypeStruct


@dataclasses.dataclass
class LU32:
    lu: torch.Tensor    # n×n FP32 factor (L unit-lower, U upper)
    piv: torch.Tensor   # 0-based swaps
    info: torch.Tensor  # device int32


PRECISIONS = {"tf32": 0, "3xtf32": 1}


def lu_factor_tf32(a: torch.Tensor, precision: str = "tf32") -> LU32:
    """FP32 LU with partial pivoting and tensor-core trailing updates:
    precision "tf32" (one TF32 product) or "3xtf32" (FP32-level accuracy)."""
    a64 = as_device_f64(a)
    n = a64.shape[0]
    if a64.shape != (n, n):
        raise ValueError("lu_factor_tf32 needs a square matrix")
    if n % 4:
        raise ValueError("lu_factor_tf32 needs n to be a multiple of 4")
    dev = a64.device
    lu = torch.empty((n, n), dtype=torch.float32, device=dev)
    piv = torch.empty(n, dtype=torch.int32, device=dev)
    info = torch.empty(1, dtype=torch.int32, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    prec = PRECISIONS[precision]
    wbytes = int(_ffi.load().lxgb_getrf_f32_tc_workspace_size(n, prec))
    work = torch.empty(wbytes // 8 + 1, dtype=torch.float64, device=dev)
    _ffi.call("lxgb_getrf_f32_tc", n, _ffi.ptr(a64), _ffi.ptr(lu), _ffi.ptr(piv), _ffi.ptr(info),
              prec, _ffi.ptr(err), _ffi.ptr(work), work.numel() * 8, _ffi.stream_handle(dev))
    if int(err.item()) != 0:
        raise RuntimeError("tensor-core pipeline timed out during the LU update")
    return LU32(lu, piv, info)


class LUPreconditioner(AbstractLinearOperator):  # noqa: D101
    """M = (P^T L U)^{-1} applied in FP32 to FP64 vectors (lxgb_getrs_f32)."""

    def __init__(self, factor: LU32):
        self.factor = factor
        n = factor.lu.shape[0]
        self._s = ShapeDtypeStruct((n,), torch.float64)
        self.tags = frozenset()

    def mv_block(self, x: torch.Tensor) -> torch.Tensor:
        xb = as_device_f64(x)
        k, n = xb.shape
        out = torch.empty_like(xb)
        _ffi.call("lxgb_getrs_f32", n, k, _ffi.ptr(self.factor.lu), _ffi.ptr(self.factor.piv),
                  _ffi.ptr(xb), _ffi.ptr(out), _ffi.stream_handle(xb.device))
        return out

    def mv(self, vector):
        return self.mv_block(vector.reshape(1, -1)).reshape(vector.shape)

    def as_matrix(self):
        raise NotImplementedError("the LU preconditioner is matrix-free")

    def transpose(self):
        raise NotImplementedError("transposed FP32 LU solves are not provided")

    def in_structure(self):
        return self._s

    def out_structure(self):
        return self._s


def lu_preconditioner(operator, precision: str = "3xtf32") -> LUPreconditioner:
    """FP32 LU (tensor-core updates) of the operator's matrix as a GMRES preconditioner."""
    mat = operator.matrix if isinstance(operator, MatrixLinearOperator) else operator.as_matrix()
    return LUPreconditioner(lu_factor_tf32(mat, precision))


def _kmax(x: torch.Tensor) -> torch.Tensor:
    """Per-vector max |x_c| of a (k, n) block (device, lxgb_kreduce_f64 op 1)."""
    k, n = x.shape
    out = torch.empty(k, dtype=torch.float64, device=x.device)
    wbytes = int(_ffi.load().lxgb_kreduce_workspace_size(k, n))
    work = torch.empty(wbytes // 8 + 1, dtype=torch.float64, device=x.device)
    _ffi.call("lxgb_kreduce_f64", 1, k, n, _ffi.ptr(x), n, 0, 0, _ffi.ptr(out), _ffi.ptr(work),
              work.numel() * 8, _ffi.stream_handle(x.device))
    return out


def norm_inf(a: torch.Tensor) -> torch.Tensor:
    """||A||_inf of a matrix (device scalar, lxgb_norm_inf_f64)."""
    a64 = as_device_f64(a)
    m, n = a64.shape
    out = torch.empty(1, dtype=torch.float64, device=a64.device)
    wbytes = int(_ffi.load().lxgb_norm_inf_workspace_size(m))
    work = torch.empty(wbytes // 8 + 1, dtype=torch.float64, device=a64.device)
    _ffi.call("lxgb_norm_inf_f64", m, n, _ffi.ptr(a64), n, _ffi.ptr(out), _ffi.ptr(work),
              work.numel() * 8, _ffi.stream_handle(a64.device))
    return out


@dataclasses.dataclass
class IRResult:
    x: torch.Tensor          # (k, n) solutions
    berr: list               # normwise backward error per right-hand side
    outer: int               # refinement steps
    inner_steps: list        # GMRES outer iterations (restart cycles) per refinement step
    converged: bool


def gmres_ir(a: torch.Tensor, b: torch.Tensor, *, tol: float = 1e-12, inner_rtol: float = 1e-6,
             restart: int = 20, stagnation_iters: int = 20, max_outer: int = 20,
             factor: LU32 | None = None, precision: str = "3xtf32") -> IRResult:
    """GMRES-based iterative refinement for A X = B (B: (k, n) FP64).

    Each refinement step solves A d = r / ||r||_inf with FP64 GMRES (lineax
    semantics, rtol = atol = inner_rtol) left-preconditioned by the FP32/TF32
    LU, then x += ||r||_inf d and r = b - A x in FP64, until the normwise
    backward error of every right-hand side is <= tol."""
    a64 = as_device_f64(a)
    b64 = as_device_f64(b)
    if b64.ndim == 1:
        b64 = b64.reshape(1, -1)
    k, n = b64.shape
    dev = a64.device
    st = _ffi.stream_handle(dev)
    if factor is None:
        factor = lu_factor_tf32(a64, precision)
    op = MatrixLinearOperator(a64)
    pre = LUPreconditioner(factor)
    anorm = float(norm_inf(a64).item())
    bnorm = _kmax(b64).cpu()
    x = torch.zeros_like(b64)
    r = b64.clone()
    inner_steps, berr, converged, it = [], [float("inf")] * k, False, 0
    for it in range(1, max_outer + 1):
        rn = _kmax(r)
        rhat = r.clone()
        _ffi.call("lxgb_rows_scale_f64", k, n, _ffi.ptr(rn), 1, _ffi.ptr(rhat), st)
        res = _krylov.gmres_block(op, rhat, rtol=inner_rtol, atol=inner_rtol, restart=restart,
                                  stagnation_iters=stagnation_iters, preconditioner=pre)
        inner_steps.append(max(res.steps))
        _ffi.call("lxgb_rows_axpy_f64", k, n, _ffi.ptr(rn), _ffi.ptr(res.y), _ffi.ptr(x), st)
        r.copy_(b64)
        _ffi.call("lxgb_gemv_f64", n, n, _ffi.ptr(a64), n, 0, k, _ffi.ptr(x), n, _ffi.ptr(r), n,
                  -1.0, 1.0, st)
        rn_h = _kmax(r).cpu()
        xn_h = _kmax(x).cpu()
        berr = [float(rn_h[c] / (anorm * xn_h[c] + bnorm[c])) if (anorm * xn_h[c] + bnorm[c]) > 0
                else 0.0 for c in range(k)]
        if all(e <= tol for e in berr):
            converged = True
            break
    return IRResult(x, berr, it, inner_steps, converged)
