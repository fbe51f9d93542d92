"""Norms and inner products of vector PyTrees (mirrors lineax/_norm.py).

Each reduction runs on lxgb_reduce_f64 and returns a 0-d CUDA float64 tensor
(no host synchronisation); leaves are combined in leaf order.
"""

from __future__ import annotations

import math

import torch

from . import _ffi
from ._blas import as_device_f64
from ._structure import tree_flatten

_DOT, _MAX, _SUMSQ, _TWO = 0, 1, 2, 3


def _reduce(op: int, x: torch.Tensor, y: torch.Tensor | None = None) -> torch.Tensor:
    xf = as_device_f64(x).reshape(-1)
    yf = as_device_f64(y).reshape(-1) if y is not None else None
    n = xf.numel()
    out = torch.empty((), dtype=torch.float64, device=xf.device)
    wbytes = int(_ffi.load().lxgb_reduce_workspace_size(n))
    work = torch.empty(max(1, wbytes // 8), dtype=torch.float64, device=xf.device)
    _ffi.call("lxgb_reduce_f64", op, n, _ffi.ptr(xf), _ffi.ptr(yf), _ffi.ptr(out),
              _ffi.ptr(work), wbytes, _ffi.stream_handle(xf.device))
    return out


def tree_dot(tree1, tree2) -> torch.Tensor:
    """Σ over leaves of <leaf1, leaf2> (lineax/_norm.py:27-47; real dtypes)."""
    l1, t1 = tree_flatten(tree1)
    l2, t2 = tree_flatten(tree2)
    if t1 != t2:
        raise ValueError("trees must have the same structure")
    if not l1:
        return torch.zeros((), dtype=torch.float64, device="cuda")
    out = _reduce(_DOT, l1[0], l2[0])
    for a, b in zip(l1[1:], l2[1:]):
        out = out + _reduce(_DOT, a, b)
    return out


def sum_squares(x) -> torch.Tensor:
    leaves, _ = tree_flatten(x)
    if not leaves:
        return torch.zeros((), dtype=torch.float64, device="cuda")
    out = _reduce(_SUMSQ, leaves[0])
    for a in leaves[1:]:
        out = out + _reduce(_SUMSQ, a)
    return out


def two_norm(x) -> torch.Tensor:
    """sqrt(Σ x²), or |x| for a single element (lineax/_norm.py:59-77)."""
    leaves, _ = tree_flatten(x)
    if len(leaves) == 1:
        return _reduce(_TWO, leaves[0])
    return torch.sqrt(sum_squares(x))


def rms_norm(x) -> torch.Tensor:
    leaves, _ = tree_flatten(x)
    size = sum(leaf.numel() for leaf in leaves)
    if size == 0:
        return torch.zeros((), dtype=torch.float64, device="cuda")
    return two_norm(x) / math.sqrt(size)


def max_norm(x) -> torch.Tensor:
    """max |x| over all leaves, NaN-propagating (lineax/_norm.py:123-143)."""
    leaves, _ = tree_flatten(x)
    leaves = [a for a in leaves if a.numel() > 0]
    if not leaves:
        return torch.zeros((), dtype=torch.float64, device="cuda")
    out = _reduce(_MAX, leaves[0])
    for a in leaves[1:]:
        out = torch.maximum(out, _reduce(_MAX, a))
    return out
