"""Python wrappers of the engine's level-2 kernels (GEMV, non-finite scan)."""

from __future__ import annotations

import torch

from . import _ffi


def as_device_f64(x: torch.Tensor) -> torch.Tensor:
    """The tensor as a contiguous CUDA float64 tensor (copy only if needed)."""
    if x.device.type != "cuda":
        raise ValueError("lineax_gb300 operates on CUDA tensors; got a tensor on "
                         f"{x.device}")
    if x.dtype != torch.float64:
        if x.is_complex():
            raise ValueError("complex dtypes are not supported by lineax_gb300")
        x = x.to(torch.float64)
    return x.contiguous()


def gemv(matrix: torch.Tensor, vector, trans: bool = False, alpha: float = 1.0,
         beta: float = 0.0, out: torch.Tensor | None = None) -> torch.Tensor:
    """alpha * op(matrix) @ vector (+ beta * out) on lxgb_gemv_f64.

    `vector` may be 1-D (one vector) or 2-D (nvec, n) (several vectors).
    Non-float64 operands are computed in float64 and cast back.
    """
    if isinstance(vector, (tuple, list, dict)):
        raise ValueError("MatrixLinearOperator.mv expects a single 1-D tensor")
    out_dtype = torch.promote_types(matrix.dtype, vector.dtype)
    a = as_device_f64(matrix)
    x = as_device_f64(vector)
    m, n = a.shape
    rows_out = n if trans else m
    single = x.ndim == 1
    xv = x.reshape(1, -1) if single else x
    nvec = xv.shape[0]
    if xv.shape[1] != (m if trans else n):
        raise ValueError(f"gemv: vector of length {xv.shape[1]} for a {m}x{n} matrix")
    if out is None:
        y = torch.empty((nvec, rows_out), dtype=torch.float64, device=a.device)
        beta = 0.0
    else:
        y = out.reshape(nvec, rows_out)
    _ffi.call("lxgb_gemv_f64", m, n, _ffi.ptr(a), n, int(trans), nvec, _ffi.ptr(xv),
              xv.shape[1], _ffi.ptr(y), rows_out, float(alpha), float(beta),
              _ffi.stream_handle(a.device))
    y = y[0] if single else y
    return y if out_dtype == torch.float64 else y.to(out_dtype)


def any_nonfinite(x: torch.Tensor) -> torch.Tensor:
    """Device int32 flag (shape [1]): 1 if x holds a NaN or inf."""
    flag = torch.empty(1, dtype=torch.int32, device=x.device)
    xf = as_device_f64(x).reshape(-1)
    _ffi.call("lxgb_nonfinite_f64", xf.numel(), _ffi.ptr(xf), _ffi.ptr(flag),
              _ffi.stream_handle(x.device))
    return flag


def gemm_tf32_nt(a: torch.Tensor, b: torch.Tensor, c: torch.Tensor | None = None,
                 alpha: float = 1.0, beta: float = 0.0) -> torch.Tensor:
    """alpha * a @ b.T + beta * c on the tcgen05 tensor cores (TF32 products,
    FP32 accumulation).  a: (m, k), b: (n, k) float32 CUDA tensors with row
    strides that are multiples of 4."""
    if a.dtype != torch.float32 or b.dtype != torch.float32:
        raise ValueError("gemm_tf32_nt takes float32 operands")
    m, k = a.shape
    n, k2 = b.shape
    if k != k2:
        raise ValueError("inner dimensions differ")
    if c is None:
        c = torch.zeros((m, n), dtype=torch.float32, device=a.device)
        beta = 0.0
    err = torch.zeros(1, dtype=torch.int32, device=a.device)
    _ffi.call("lxgb_gemm_tf32_nt", m, n, k, _ffi.ptr(a), a.stride(0), _ffi.ptr(b), b.stride(0),
              _ffi.ptr(c), c.stride(0), float(alpha), float(beta), _ffi.ptr(err),
              _ffi.stream_handle(a.device))
    if int(err.item()) != 0:
        raise RuntimeError("tcgen05 GEMM pipeline timed out")
    return c


def gemm_3xtf32_nt(a: torch.Tensor, b: torch.Tensor, c: torch.Tensor | None = None,
                   alpha: float = 1.0, beta: float = 0.0) -> torch.Tensor:
    """alpha * a @ b.T + beta * c with 3xTF32 tensor-core products (FP32-level
    accuracy): the operands are split into TF32-exact hi parts and lo remainders."""
    def split(x):
        hi = (x.view(torch.int32) & -8192).view(torch.float32).contiguous()
        return hi, (x - hi).contiguous()
    m, k = a.shape
    n = b.shape[0]
    ah, al = split(a.contiguous())
    bh, bl = split(b.contiguous())
    if c is None:
        c = torch.zeros((m, n), dtype=torch.float32, device=a.device)
        beta = 0.0
    err = torch.zeros(1, dtype=torch.int32, device=a.device)
    _ffi.call("lxgb_gemm_3xtf32_nt", m, n, k, _ffi.ptr(ah), _ffi.ptr(al), k, _ffi.ptr(bh),
              _ffi.ptr(bl), k, _ffi.ptr(c), c.stride(0), float(alpha), float(beta), _ffi.ptr(err),
              _ffi.stream_handle(a.device))
    if int(err.item()) != 0:
        raise RuntimeError("tcgen05 GEMM pipeline timed out")
    return c
