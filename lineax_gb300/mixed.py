"""Mixed-precision LU with GMRES-IR.

The factor is computed in FP32 with partial pivoting and tensor-core (TF32)
trailing updates (lxgb_getrf_f32_tc); FP64 GMRES on the original operator,
left-preconditioned by the FP32 LU, recovers FP64 accuracy (GMRES-based
iterative refinement, Carson & Higham 2017).  The preconditioner is applied
as M x = U^{-1} (L^{-1} (P x)) with the triangular inverses formed once on
the tensor cores (lxgb_lu32_inverse): two matrix-vector products that spread
over every SM, in double-float arithmetic so that M stays one fixed linear
operator to FP64 accuracy however ill-conditioned the factor is (the
preconditioner precision u_p of five-precision GMRES-IR, Amestoy et al.
2023).  Through the lineax API this is

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


PRECISIONS = {"tf32": 0, "3xtf32": 1, "bf16": 2}
# Factor precisions from the cheapest to the most accurate: a solve that stalls
# with one factor moves to the next before it falls back to FP64.
LADDER = ("bf16", "tf32", "3xtf32")


def _pipeline_err(err: torch.Tensor | None, dev) -> tuple:
    """(err tensor, whether to check it now): callers that pass their own
    device flag read it later themselves (one synchronisation per request
    instead of one per stage, so the host keeps enqueueing while the GPU
    works)."""
    if err is None:
        return torch.zeros(1, dtype=torch.int32, device=dev), True
    return err, False


def lu_factor_tf32(a: torch.Tensor, precision: str = "tf32",
                   err: torch.Tensor | None = None) -> LU32:
    """FP32 LU with partial pivoting and tensor-core trailing updates:
    precision "bf16" (BF16 products, FP32 accumulation), "tf32" (one TF32
    product) or "3xtf32" (FP32-level accuracy)."""
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
    err, check = _pipeline_err(err, dev)
    prec = PRECISIONS[precision]
    wbytes = int(_ffi.load().lxgb_getrf_f32_tc_workspace_size(n, prec))
    work = torch.empty(wbytes // 8 + 1, dtype=torch.float64, device=dev)
    _ffi.call("lxgb_getrf_f32_tc", n, _ffi.ptr(a64), _ffi.ptr(lu), _ffi.ptr(piv), _ffi.ptr(info),
              prec, _ffi.ptr(err), _ffi.ptr(work), work.numel() * 8, _ffi.stream_handle(dev))
    if check and int(err.item()) != 0:
        raise RuntimeError("tensor-core pipeline timed out during the LU update")
    return LU32(lu, piv, info)


def cholesky_factor_tf32(a: torch.Tensor, err: torch.Tensor | None = None) -> LU32:
    """FP32 Cholesky A = L Lᵀ with 3xTF32 tensor-core updates
    (lxgb_potrf_f32_tc; A read from its upper triangle), returned in the
    unit-lower / upper form of lu_factor_tf32 (L' = L D⁻¹, U' = D Lᵀ, no
    interchanges) so that gmres_ir applies unchanged.  info > 0 when a pivot
    is not positive in FP32."""
    a64 = as_device_f64(a)
    n = a64.shape[0]
    if a64.shape != (n, n):
        raise ValueError("cholesky_factor_tf32 needs a square matrix")
    if n % 4:
        raise ValueError("cholesky_factor_tf32 needs n to be a multiple of 4")
    dev = a64.device
    l = torch.empty((n, n), dtype=torch.float32, device=dev)
    lu = torch.empty((n, n), dtype=torch.float32, device=dev)
    piv = torch.empty(n, dtype=torch.int32, device=dev)
    info = torch.empty(1, dtype=torch.int32, device=dev)
    err, check = _pipeline_err(err, dev)
    wbytes = int(_ffi.load().lxgb_potrf_f32_tc_workspace_size(n))
    work = torch.empty(wbytes // 8 + 1, dtype=torch.float64, device=dev)
    s = _ffi.stream_handle(dev)
    _ffi.call("lxgb_potrf_f32_tc", n, _ffi.ptr(a64), _ffi.ptr(l), _ffi.ptr(info), _ffi.ptr(err),
              _ffi.ptr(work), work.numel() * 8, s)
    _ffi.call("lxgb_chol32_to_lu32", n, _ffi.ptr(l), _ffi.ptr(lu), _ffi.ptr(piv), s)
    if check and int(err.item()) != 0:
        raise RuntimeError("tensor-core pipeline timed out during the Cholesky update")
    return LU32(lu, piv, info)


def cholesky_inverse(factor: LU32, err: torch.Tensor | None = None) -> InverseLU32:
    """Triangular inverses of a factor from cholesky_factor_tf32: L'⁻¹ by the
    tensor-core substitution of lu_inverse, U'⁻¹ = L'⁻ᵀ D⁻² by a transposing
    copy (no second substitution)."""
    lu = factor.lu
    n = lu.shape[0]
    dev = lu.device
    linv = torch.empty((n, n), dtype=torch.float32, device=dev)
    uinv = torch.empty((n, n), dtype=torch.float32, device=dev)
    perm = torch.empty(n, dtype=torch.int32, device=dev)
    err, check = _pipeline_err(err, dev)
    wbytes = int(_ffi.load().lxgb_lu32_inverse_workspace_size(n, 1))
    work = torch.empty(wbytes // 8 + 1, dtype=torch.float64, device=dev)
    s = _ffi.stream_handle(dev)
    _ffi.call("lxgb_lu32_inverse", n, _ffi.ptr(lu), _ffi.ptr(factor.piv), _ffi.ptr(linv), None,
              _ffi.ptr(perm), 1, _ffi.ptr(err), _ffi.ptr(work), work.numel() * 8, s)
    _ffi.call("lxgb_chol32_uinv", n, _ffi.ptr(lu), _ffi.ptr(linv), _ffi.ptr(uinv), s)
    if check and int(err.item()) != 0:
        raise RuntimeError("tensor-core pipeline timed out during the triangular inversion")
    return InverseLU32(linv, uinv, perm)


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


ARITH = {"fp32": 0, "df": 1}


@dataclasses.dataclass
class InverseLU32:
    linv: torch.Tensor  # L^{-1}, n×n FP32 (unit lower, zeros above the diagonal)
    uinv: torch.Tensor  # U^{-1}, n×n FP32 (zeros below the diagonal)
    perm: torch.Tensor  # (P b)_i = b[perm[i]]


def lu_inverse(factor: LU32, precision: str = "3xtf32",
               err: torch.Tensor | None = None) -> InverseLU32:
    """Triangular inverses of an FP32 LU, off-diagonal blocks on the tensor cores."""
    lu = factor.lu
    n = lu.shape[0]
    dev = lu.device
    linv = torch.empty((n, n), dtype=torch.float32, device=dev)
    uinv = torch.empty((n, n), dtype=torch.float32, device=dev)
    perm = torch.empty(n, dtype=torch.int32, device=dev)
    err, check = _pipeline_err(err, dev)
    prec = min(PRECISIONS[precision], 1)  # a BF16 factor's inverses use TF32 updates
    wbytes = int(_ffi.load().lxgb_lu32_inverse_workspace_size(n, prec))
    work = torch.empty(wbytes // 8 + 1, dtype=torch.float64, device=dev)
    _ffi.call("lxgb_lu32_inverse", n, _ffi.ptr(lu), _ffi.ptr(factor.piv), _ffi.ptr(linv),
              _ffi.ptr(uinv), _ffi.ptr(perm), prec, _ffi.ptr(err), _ffi.ptr(work),
              work.numel() * 8, _ffi.stream_handle(dev))
    if check and int(err.item()) != 0:
        raise RuntimeError("tensor-core pipeline timed out during the triangular inversion")
    return InverseLU32(linv, uinv, perm)


class _BlockOperator(AbstractLinearOperator):
    """Square n×n FP64 operator defined by a (k, n) block product."""

    def __init__(self, n: int):
        self._s = ShapeDtypeStruct((n,), torch.float64)
        self.tags = frozenset()

    def mv(self, vector):
        return self.mv_block(vector.reshape(1, -1)).reshape(vector.shape)

    def as_matrix(self):
        raise NotImplementedError("matrix-free operator")

    def transpose(self):
        raise NotImplementedError("transpose not provided")

    def in_structure(self):
        return self._s

    def out_structure(self):
        return self._s


class InverseLUPreconditioner(_BlockOperator):
    """M = U^{-1} L^{-1} P from the triangular inverses of an FP32 LU, applied
    in "df" (double-float, FP64-accurate) or "fp32" arithmetic."""

    def __init__(self, factor: LU32, inverse: InverseLU32, arith: str = "df"):
        super().__init__(inverse.linv.shape[0])
        self.factor = factor
        self.inverse = inverse
        self.mode = ARITH[arith]
        self._work = None

    def mv_block(self, x: torch.Tensor) -> torch.Tensor:
        xb = as_device_f64(x).contiguous()
        k, n = xb.shape
        out = torch.empty_like(xb)
        wbytes = int(_ffi.load().lxgb_lu32_apply_workspace_size(n, k))
        if self._work is None or self._work.numel() * 8 < wbytes:
            self._work = torch.empty(wbytes // 8 + 1, dtype=torch.float64, device=xb.device)
        inv = self.inverse
        _ffi.call("lxgb_lu32_apply", n, k, _ffi.ptr(inv.linv), _ffi.ptr(inv.uinv),
                  _ffi.ptr(inv.perm), self.mode, _ffi.ptr(xb), _ffi.ptr(out),
                  _ffi.ptr(self._work), self._work.numel() * 8, _ffi.stream_handle(xb.device))
        return out


@dataclasses.dataclass
class SplitMatrix:
    hi: torch.Tensor  # A truncated to 24 significant bits (FP32)
    lo: torch.Tensor  # the next 24 bits (FP32)


def split_matrix(a: torch.Tensor) -> SplitMatrix:
    """A (FP64) as an FP32 hi + lo pair: 48 significant bits."""
    a64 = as_device_f64(a)
    m, n = a64.shape
    hi = torch.empty((m, n), dtype=torch.float32, device=a64.device)
    lo = torch.empty_like(hi)
    _ffi.call("lxgb_split_f64", m, n, _ffi.ptr(a64), a64.stride(0), _ffi.ptr(hi), _ffi.ptr(lo), n,
              _ffi.stream_handle(a64.device))
    return SplitMatrix(hi, lo)


class SplitMatrixOperator(_BlockOperator):
    """A x with A held as a SplitMatrix: "df" gives FP64-accurate products in
    double-float arithmetic on the FP32 pipe, "fp32" uses the hi part in FP32."""

    def __init__(self, split: SplitMatrix, arith: str = "df"):
        super().__init__(split.hi.shape[0])
        self.split = split
        self.mode = ARITH[arith]
        self._work = None

    def _run(self, x: torch.Tensor, b: torch.Tensor | None) -> torch.Tensor:
        xb = as_device_f64(x).contiguous()
        k, n = xb.shape
        out = torch.empty_like(xb)
        wbytes = int(_ffi.load().lxgb_gemv_df_workspace_size(n, k))
        if self._work is None or self._work.numel() * 8 < wbytes:
            self._work = torch.empty(wbytes // 8 + 1, dtype=torch.float64, device=xb.device)
        lo = self.split.lo if self.mode == 1 else None
        _ffi.call("lxgb_gemv_df", n, n, _ffi.ptr(self.split.hi), _ffi.ptr(lo), n, k, _ffi.ptr(xb),
                  n, _ffi.ptr(b), _ffi.ptr(out), n, self.mode, _ffi.ptr(self._work),
                  self._work.numel() * 8, _ffi.stream_handle(xb.device))
        return out

    def mv_block(self, x: torch.Tensor) -> torch.Tensor:
        return self._run(x, None)

    def residual(self, x: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
        """b - A x for (k, n) blocks."""
        return self._run(x, as_device_f64(b).contiguous())


def lu_preconditioner(operator, precision: str = "3xtf32", arith: str = "df"
                      ) -> InverseLUPreconditioner:
    """FP32 LU (tensor-core updates) of the operator's matrix as a GMRES
    preconditioner, applied through its triangular inverses."""
    mat = operator.matrix if isinstance(operator, MatrixLinearOperator) else operator.as_matrix()
    f = lu_factor_tf32(mat, precision)
    return InverseLUPreconditioner(f, lu_inverse(f, precision), arith)


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
    inner_steps: list        # GMRES restart cycles per refinement step (0: plain refinement)
    converged: bool
    fallback: bool = False   # solved by the FP64 LU after GMRES-IR stalled
    inverse: InverseLU32 | None = None  # the triangular inverses, when they were formed
    tiers: list = dataclasses.field(default_factory=list)  # (factor, outer, converged) tried


def gmres_ir(a: torch.Tensor, b: torch.Tensor, *, tol: float = 1e-12, inner_rtol: float = 1e-6,
             restart: int = 20, stagnation_iters: int = 20, max_outer: int = 20,
             inner_max_steps: int | None = None, factor: LU32 | None = None,
             inverse: InverseLU32 | None = None, split: SplitMatrix | None = None,
             precision: str = "3xtf32", arith: str = "df", fallback: bool = False,
             qr: "SquareQR32 | None" = None, device_loop: bool = True,
             escalate: bool = False, stop_on_stall: bool | None = None) -> IRResult:
    """GMRES-based iterative refinement for A X = B (B: (k, n) FP64).

    Each refinement step solves A d = r / ||r||_inf with GMRES (lineax
    semantics, rtol = atol = inner_rtol) left-preconditioned by the FP32 LU,
    then x += ||r||_inf d and r = b - A x, until the normwise backward error
    of every right-hand side is <= tol.  arith "df" runs the inner operator
    and preconditioner products in double-float (FP64-accurate) arithmetic,
    "fp32" in FP32; "ir" replaces the GMRES solve by one preconditioner
    product (x += M^{-1} r: classic LU iterative refinement, enough when
    kappa(A) u_f is well below 1); "auto" starts with "ir" and moves to "df"
    GMRES when a step stalls.  The triangular inverses are formed here when
    `inverse` is not given: the preconditioner is applied through them
    (one-CTA-per-vector triangular solves stream the whole factor through a
    single SM and cost far more at these sizes).  The outer residual is always FP64-accurate (A
    as a 48-bit hi + lo pair, double-float sums).

    fallback=True stops refining as soon as it stalls (an inner solve that
    does not reach inner_rtol, or a refinement step that shrinks the largest
    backward error by less than 2x) and solves with the FP64 LU instead, as
    mixed-precision solvers do when the low-precision factor is too far from
    A (kappa(A) u_f well above 1): IRResult.fallback is then True.

    With `qr` (a SquareQR32 of A) the preconditioner is M = R^{-1} Qᵀ from
    the TF32 Householder QR instead of the LU, and the fallback is the FP64
    Householder QR solve: lineax's QR solver (lineax/_solver/qr.py:55-94) on
    a square operator, recovered to FP64 accuracy the same way.

    escalate=True (LU preconditioner, arith "auto"): a solve that stalls with
    the given factor precision is repeated with the next one of LADDER (BF16 →
    TF32 → 3xTF32) before the FP64 fallback; IRResult.tiers lists what was
    tried.  stop_on_stall (default: fallback) ends the loop at the first stall
    of the GMRES tier.

    device_loop (arith "auto", with the LU or the QR preconditioner) runs the
    whole refinement loop as one call of lxgb_gmres_ir_run — the same kernels
    in the same order, with the loop decisions taken on the device — and
    returns to the host once, at the end."""
    a64 = as_device_f64(a)
    b64 = as_device_f64(b)
    if b64.ndim == 1:
        b64 = b64.reshape(1, -1)
    b64 = b64.contiguous()
    k, n = b64.shape
    if stop_on_stall is None:
        stop_on_stall = fallback
    if escalate and qr is None and arith == "auto" and precision in LADDER:
        if split is None:
            split = split_matrix(a64)
        tried, res = [], None
        for prec in LADDER[LADDER.index(precision):]:
            f = factor if prec == precision and factor is not None else lu_factor_tf32(a64, prec)
            inv = inverse if prec == precision else None
            res = gmres_ir(a64, b64, tol=tol, inner_rtol=inner_rtol, restart=restart,
                           stagnation_iters=stagnation_iters, max_outer=max_outer,
                           inner_max_steps=inner_max_steps, factor=f, inverse=inv, split=split,
                           precision=prec, arith=arith, fallback=False, device_loop=device_loop,
                           stop_on_stall=True)
            tried.append((prec, res.outer, res.converged))
            if res.converged:
                res.tiers = tried
                return res
        if fallback:
            outer_op = SplitMatrixOperator(split, "df")
            res = _fp64_fallback(a64, b64, outer_op, float(norm_inf(a64).item()),
                                 _kmax(b64).cpu(), tol, res.outer, res.inner_steps)
            tried.append(("fp64", 1, res.converged))
        res.tiers = tried
        return res
    if factor is None and qr is None:
        factor = lu_factor_tf32(a64, precision)
    if split is None:
        split = split_matrix(a64)
    outer_op = SplitMatrixOperator(split, "df")
    if device_loop and arith == "auto":
        if qr is None and inverse is None:
            inverse = lu_inverse(factor, precision)
        return _gmres_ir_device(a64, b64, split, inverse, tol, inner_rtol, restart,
                                stagnation_iters, max_outer, inner_max_steps, fallback,
                                stop_on_stall, qr=qr)
    tiers = ["ir", "df"] if arith == "auto" else [arith]
    tier = 0
    made = {"inverse": inverse}

    def inner(t):
        kind = tiers[t]
        if qr is not None:
            op = outer_op if kind in ("df", "ir") else SplitMatrixOperator(split, kind)
            return op, QRPreconditioner(qr, "df" if kind == "ir" else kind)
        if made["inverse"] is None:
            made["inverse"] = lu_inverse(factor, precision)
        op = outer_op if kind in ("df", "ir") else SplitMatrixOperator(split, kind)
        return op, InverseLUPreconditioner(factor, made["inverse"], "df" if kind == "ir" else kind)

    inner_op, pre = inner(tier)
    anorm = float(norm_inf(a64).item())
    bnorm = _kmax(b64).cpu()
    x = torch.zeros_like(b64)
    r = b64.clone()
    st = _ffi.stream_handle(a64.device)
    inner_steps, berr, converged, it = [], [float("inf")] * k, False, 0
    for it in range(1, max_outer + 1):
        if tiers[tier] == "ir":
            # plain refinement: x += M^{-1} r (one preconditioner product)
            x.add_(pre.mv_block(r))
            inner_steps.append(0)
            inner_ok = True
        else:
            rn = _kmax(r)
            rhat = r.clone()
            _ffi.call("lxgb_rows_scale_f64", k, n, _ffi.ptr(rn), 1, _ffi.ptr(rhat), st)
            res = _krylov.gmres_block(inner_op, rhat, rtol=inner_rtol, atol=inner_rtol,
                                      restart=restart, stagnation_iters=stagnation_iters,
                                      max_steps=inner_max_steps, preconditioner=pre)
            inner_steps.append(max(res.steps))
            _ffi.call("lxgb_rows_axpy_f64", k, n, _ffi.ptr(rn), _ffi.ptr(res.y), _ffi.ptr(x), st)
            inner_ok = all(code == _krylov.SUCCESSFUL for code in res.results)
        r = outer_op.residual(x, b64)
        prev = max(berr)
        berr = _berr(r, x, anorm, bnorm)
        if all(e <= tol for e in berr):
            converged = True
            break
        stalled = not inner_ok or not (max(berr) <= prev / 2)
        if stalled and tier + 1 < len(tiers):
            tier += 1
            inner_op, pre = inner(tier)
        elif stop_on_stall and stalled:
            if not fallback:
                break
            return _fp64_fallback(a64, b64, outer_op, anorm, bnorm, tol, it, inner_steps,
                                  qr is not None)
    if fallback and not converged:
        return _fp64_fallback(a64, b64, outer_op, anorm, bnorm, tol, it, inner_steps,
                              qr is not None)
    return IRResult(x, berr, it, inner_steps, converged, inverse=made["inverse"])


def _gmres_ir_device(a64, b64, split, inverse, tol, inner_rtol, restart, stagnation_iters,
                     max_outer, inner_max_steps, fallback, stop_on_stall,
                     qr: "SquareQR32 | None" = None) -> IRResult:
    """gmres_ir's "auto" loop as one lxgb_gmres_ir_run call, preconditioned by
    the LU inverses (LXGB_OP_LU32_INV) or by R^{-1} Qᵀ (LXGB_OP_QR32)."""
    import ctypes

    k, n = b64.shape
    dev = b64.device
    op = _ffi.LinearOperatorDesc(kind=_ffi.OP_SPLIT_DF, n=n, lda=n, scale=1.0,
                                 hi=split.hi.data_ptr(), lo=split.lo.data_ptr())
    if qr is not None:
        pre = _ffi.LinearOperatorDesc(kind=_ffi.OP_QR32, n=n, scale=1.0,
                                      hi=qr.qt.data_ptr(), lo=qr.rinv.data_ptr())
    else:
        pre = _ffi.LinearOperatorDesc(kind=_ffi.OP_LU32_INV, n=n, scale=1.0,
                                      hi=inverse.linv.data_ptr(), lo=inverse.uinv.data_ptr(),
                                      perm=inverse.perm.data_ptr())
    anorm = norm_inf(a64).reshape(1)
    x = torch.empty_like(b64)
    berr = torch.empty(k, dtype=torch.float64, device=dev)
    status = torch.zeros(3, dtype=torch.int32, device=dev)
    R = min(int(restart), n)
    wbytes = int(_ffi.load().lxgb_gmres_ir_run_workspace_size(k, n, R))
    work = torch.empty(wbytes // 8 + 1, dtype=torch.float64, device=dev)
    inner_steps = 5 if inner_max_steps is None else int(inner_max_steps)
    _ffi.call("lxgb_gmres_ir_run", k, n, ctypes.addressof(op), ctypes.addressof(pre),
              _ffi.ptr(b64), _ffi.ptr(x), _ffi.ptr(anorm), float(tol), float(inner_rtol),
              int(max_outer), R, inner_steps, int(stagnation_iters), int(bool(stop_on_stall)),
              _ffi.ptr(berr), _ffi.ptr(status), _ffi.ptr(work), work.numel() * 8,
              _ffi.stream_handle(dev))
    outer, reached_gmres, code = status.cpu().tolist()
    berr_h = berr.cpu().tolist()
    converged = code == 0
    if fallback and not converged:
        outer_op = SplitMatrixOperator(split, "df")
        return _fp64_fallback(a64, b64, outer_op, float(anorm.item()), _kmax(b64).cpu(), tol,
                              outer, [int(reached_gmres)] * outer, use_qr=qr is not None)
    return IRResult(x, berr_h, outer, [int(reached_gmres)] * outer, converged, inverse=inverse)


def _berr(r, x, anorm, bnorm) -> list:
    rn_h = _kmax(r).cpu()
    xn_h = _kmax(x).cpu()
    return [float(rn_h[c] / (anorm * xn_h[c] + bnorm[c])) if (anorm * xn_h[c] + bnorm[c]) > 0
            else 0.0 for c in range(r.shape[0])]


def _fp64_fallback(a64, b64, outer_op, anorm, bnorm, tol, it, inner_steps,
                   use_qr: bool = False) -> IRResult:
    """FP64 LU solve (lxgb_getrf/getrs), or with use_qr the FP64 Householder
    QR solve (lxgb_geqrf/ormqr/trsm), after GMRES-IR stalled."""
    from . import _dense

    if use_qr:
        x = qr_solve_f64(_dense.geqrf(a64), b64)
    else:
        lu, piv = _dense.lu_factor(a64)
        x = _dense.lu_solve(lu, piv, b64)
    berr = _berr(outer_op.residual(x, b64), x, anorm, bnorm)
    return IRResult(x, berr, it, inner_steps, all(e <= tol for e in berr), fallback=True)


# ---------------------------------------------------------------------------
# Mixed-precision least squares: TF32 tensor-core QR + corrected semi-normal
# equations refined in FP64-accurate arithmetic.
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class QR32:
    h: torch.Tensor     # n × m FP32, jnp.linalg.qr(mode="raw") layout (h = Aᵀ factored)
    tau: torch.Tensor   # n FP32
    t: torch.Tensor     # compact-WY T of each 32-column panel
    rt: torch.Tensor    # Rᵀ (n × n, lower, FP64)
    rinv: InverseLU32 | None  # R^{-T} (linv, lower), R^{-1} (uinv, upper); None if n % 4


def qr_factor_tf32(a: torch.Tensor) -> QR32:
    """Householder QR of a tall A (m × n, m % 4 == 0) in FP32 with the
    trailing updates on the tcgen05 tensor cores (lxgb_geqrf_f32_tc)."""
    a64 = as_device_f64(a).contiguous()
    m, n = a64.shape
    if n > m or m % 4:
        raise ValueError("qr_factor_tf32 needs a tall matrix with m a multiple of 4")
    dev = a64.device
    lib = _ffi.load()
    h = torch.empty((n, m), dtype=torch.float32, device=dev)
    tau = torch.empty(n, dtype=torch.float32, device=dev)
    t = torch.empty(max(1, int(lib.lxgb_geqrf_t_elems(n))), dtype=torch.float32, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    wbytes = int(lib.lxgb_geqrf_f32_tc_workspace_size(m, n))
    work = torch.empty(wbytes // 8 + 1, dtype=torch.float64, device=dev)
    _ffi.call("lxgb_geqrf_f32_tc", m, n, _ffi.ptr(a64), _ffi.ptr(h), _ffi.ptr(tau), _ffi.ptr(t),
              _ffi.ptr(err), _ffi.ptr(work), work.numel() * 8, _ffi.stream_handle(dev))
    if int(err.item()) != 0:
        raise RuntimeError("tensor-core pipeline timed out during the QR update")
    rt = h[:, :n].double().contiguous()
    # R^{-1} through the LU inversion machinery: R in the upper triangle of a
    # square FP32 array with identity pivots (its lower triangle is ignored)
    if n % 4:
        return QR32(h, tau, t, rt, None)  # 16-byte TMA rows: FP64 triangular solves instead
    uinv, perm = _upper_inverse(h[:, :n].t().contiguous())
    inv = InverseLU32(uinv.t().contiguous(), uinv, perm)
    return QR32(h, tau, t, rt, inv)


def _upper_inverse(r_sq: torch.Tensor, err: torch.Tensor | None = None):
    """(R^{-1}, identity perm) for R in the upper triangle of a square FP32
    array (its lower triangle holds Householder vectors and is not read):
    lxgb_lu32_inverse with linv NULL, 3xTF32 off-diagonal updates."""
    n = r_sq.shape[0]
    dev = r_sq.device
    piv = torch.arange(n, dtype=torch.int32, device=dev)
    uinv = torch.empty((n, n), dtype=torch.float32, device=dev)
    perm = torch.empty(n, dtype=torch.int32, device=dev)
    err, check = _pipeline_err(err, dev)
    wbytes = int(_ffi.load().lxgb_lu32_inverse_workspace_size(n, 1))
    work = torch.empty(wbytes // 8 + 1, dtype=torch.float64, device=dev)
    _ffi.call("lxgb_lu32_inverse", n, _ffi.ptr(r_sq), _ffi.ptr(piv), None, _ffi.ptr(uinv),
              _ffi.ptr(perm), 1, _ffi.ptr(err), _ffi.ptr(work), work.numel() * 8,
              _ffi.stream_handle(dev))
    if check and int(err.item()) != 0:
        raise RuntimeError("tensor-core pipeline timed out during the triangular inversion")
    return uinv, perm


def _gemv_df(split: SplitMatrix, x: torch.Tensor, b: torch.Tensor | None) -> torch.Tensor:
    """y = A x or b - A x for a rectangular SplitMatrix A (rows × cols) and a
    (k, cols) block x, in double-float arithmetic."""
    rows, cols = split.hi.shape
    xb = x.contiguous()
    k = xb.shape[0]
    out = torch.empty((k, rows), dtype=torch.float64, device=xb.device)
    wbytes = int(_ffi.load().lxgb_gemv_df_workspace_size(cols, k))
    work = torch.empty(wbytes // 8 + 1, dtype=torch.float64, device=xb.device)
    _ffi.call("lxgb_gemv_df", rows, cols, _ffi.ptr(split.hi), _ffi.ptr(split.lo), cols, k,
              _ffi.ptr(xb), cols, _ffi.ptr(b), _ffi.ptr(out), rows, 1, _ffi.ptr(work),
              work.numel() * 8, _ffi.stream_handle(xb.device))
    return out


@dataclasses.dataclass
class LstsqResult:
    x: torch.Tensor     # (k, n) least-squares solutions
    iters: int          # refinement steps
    step: list          # last max|dx| / max|x| per right-hand side
    converged: bool


def qr_lstsq(a: torch.Tensor, b: torch.Tensor, *, tol: float = 1e-12, max_iter: int = 10,
             factor: QR32 | None = None, split: SplitMatrix | None = None,
             split_t: SplitMatrix | None = None) -> LstsqResult:
    """min ||b - A x||_2 for a tall full-rank A by corrected semi-normal
    equations: R from the TF32 QR (qr_factor_tf32), then
        x += R^{-1} R^{-T} Aᵀ (b - A x)
    with b - A x and Aᵀ r in double-float arithmetic (A and Aᵀ held as FP32
    hi + lo pairs) and R^{-1} R^{-T} applied as two double-float triangular
    products with the tensor-core inverse of R (lxgb_lu32_inverse), until
    max|dx| <= tol max|x|.  Each step contracts the error by about
    kappa(A)^2 u_TF32, so well-conditioned problems reach FP64 accuracy in a
    few steps (Björck's CSNE; no Q is applied)."""
    a64 = as_device_f64(a).contiguous()
    m, n = a64.shape
    b64 = as_device_f64(b)
    if b64.ndim == 1:
        b64 = b64.reshape(1, -1)
    b64 = b64.contiguous()
    k = b64.shape[0]
    if factor is None:
        factor = qr_factor_tf32(a64)
    if split is None:
        split = split_matrix(a64)
    if split_t is None:
        split_t = split_matrix(a64.T.contiguous())
    x = torch.zeros((k, n), dtype=torch.float64, device=a64.device)
    r = b64.clone()
    rinv = (InverseLUPreconditioner(None, factor.rinv, "df")  # d = R^{-1} (R^{-T} g)
            if factor.rinv is not None else None)
    steps, it, converged = [float("inf")] * k, 0, False
    for it in range(1, max_iter + 1):
        g = _gemv_df(split_t, r, None)                                     # Aᵀ r
        if rinv is not None:
            d = rinv.mv_block(g)
        else:
            from . import _dense

            y = _dense.trsv(factor.rt, g, lower=True, trans=False, unit=False)  # Rᵀ y = g
            d = _dense.trsv(factor.rt, y, lower=True, trans=True, unit=False)   # R d = y
        x += d
        r = _gemv_df(split, x, b64)                                        # b - A x
        dn = d.abs().amax(dim=1)
        xn = x.abs().amax(dim=1)
        steps = (dn / torch.clamp(xn, min=1e-300)).cpu().tolist()
        if all(s_ <= tol for s_ in steps):
            converged = True
            break
    return LstsqResult(x, it, steps, converged)



# ---------------------------------------------------------------------------
# Square systems through the QR factor: TF32 Householder QR with Q formed
# explicitly, M = R^{-1} Qᵀ as the GMRES-IR preconditioner.
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class SquareQR32:
    qt: torch.Tensor    # Qᵀ, n×n FP32
    rinv: torch.Tensor  # R^{-1}, n×n FP32 (zeros below the diagonal)


def qr_square_tf32(a: torch.Tensor, err: torch.Tensor | None = None) -> SquareQR32:
    """A = Q R for a square A (n % 4 == 0): FP32 Householder QR with tcgen05
    TF32 updates that also forms Q (lxgb_geqrf_f32_tc_q), and R^{-1} by the
    tensor-core triangular inversion (3xTF32)."""
    a64 = as_device_f64(a).contiguous()
    n = a64.shape[0]
    if a64.shape != (n, n) or n % 4:
        raise ValueError("qr_square_tf32 needs a square matrix with n a multiple of 4")
    dev = a64.device
    lib = _ffi.load()
    h = torch.empty((n, n), dtype=torch.float32, device=dev)
    tau = torch.empty(n, dtype=torch.float32, device=dev)
    t = torch.empty(max(1, int(lib.lxgb_geqrf_t_elems(n))), dtype=torch.float32, device=dev)
    q = torch.empty((n, n), dtype=torch.float32, device=dev)
    err, check = _pipeline_err(err, dev)
    wbytes = int(lib.lxgb_geqrf_f32_tc_q_workspace_size(n, n))
    work = torch.empty(wbytes // 8 + 1, dtype=torch.float64, device=dev)
    _ffi.call("lxgb_geqrf_f32_tc_q", n, n, _ffi.ptr(a64), _ffi.ptr(h), _ffi.ptr(tau), _ffi.ptr(t),
              _ffi.ptr(q), _ffi.ptr(err), _ffi.ptr(work), work.numel() * 8,
              _ffi.stream_handle(dev))
    if check and int(err.item()) != 0:
        raise RuntimeError("tensor-core pipeline timed out during the QR update")
    del work, t, tau
    r_sq = h.t().contiguous()  # R on and above the diagonal
    del h
    uinv, _ = _upper_inverse(r_sq, None if check else err)
    return SquareQR32(q.t().contiguous(), uinv)


class QRPreconditioner(_BlockOperator):
    """M x = R^{-1} (Qᵀ x) for a block of FP64 vectors (lxgb_qr32_apply),
    in FP32 ("fp32") or double-float ("df") arithmetic."""

    def __init__(self, qr: SquareQR32, arith: str = "df"):
        super().__init__(qr.qt.shape[0])
        self.qr, self.mode = qr, ARITH[arith]

    def mv_block(self, x: torch.Tensor) -> torch.Tensor:
        xb = as_device_f64(x).contiguous()
        k, n = xb.shape
        out = torch.empty_like(xb)
        wbytes = int(_ffi.load().lxgb_qr32_apply_workspace_size(n, k))
        work = torch.empty(wbytes // 8 + 1, dtype=torch.float64, device=xb.device)
        _ffi.call("lxgb_qr32_apply", n, k, _ffi.ptr(self.qr.qt), _ffi.ptr(self.qr.rinv),
                  self.mode, _ffi.ptr(xb), _ffi.ptr(out), _ffi.ptr(work), work.numel() * 8,
                  _ffi.stream_handle(xb.device))
        return out


def qr_solve_f64(factor, b: torch.Tensor) -> torch.Tensor:
    """x_r = R^{-1} (Qᵀ b_r)[:n] with an FP64 factor from _dense.geqrf of a
    square or tall operator (lineax/_solver/qr.py:87-92), for a (k, m) block."""
    from . import _dense

    h, tau, t = factor
    n = h.shape[0]
    b64 = as_device_f64(b)
    if b64.ndim == 1:
        b64 = b64.reshape(1, -1)
    qhb = _dense.ormqr(h, tau, t, b64.contiguous(), trans=True)[:, :n].contiguous()
    return _dense.trsv(h, qhb, lower=True, trans=True, unit=False)
