"""Tensor-level wrappers of the dense entry points of liblxgb.so.

Every function takes and returns CUDA tensors and launches on the current
torch stream.  Factorisations work in FP64 (inputs of other float dtypes are
promoted); mixed-precision paths live in ``batched``.
"""

from __future__ import annotations

import torch

from . import _ffi
from ._blas import as_device_f64 as as_f64


def _stream(t: torch.Tensor) -> int:
    return _ffi.stream_handle(t.device)


# -- LU ---------------------------------------------------------------------


def lu_factor_batched(a: torch.Tensor):
    """P A = L U for a (batch, n, n) or (n, n) tensor.  Returns (lu, piv, info)
    with piv 0-based int32 swap indices (jax.scipy.linalg.lu_factor layout)."""
    single = a.ndim == 2
    a3 = a.reshape(1, *a.shape) if single else a
    lu = as_f64(a3).clone()
    batch, n, n2 = lu.shape
    if n != n2:
        raise ValueError("LU needs square matrices")
    piv = torch.empty((batch, n), dtype=torch.int32, device=lu.device)
    info = torch.empty(batch, dtype=torch.int32, device=lu.device)
    _ffi.call("lxgb_getrf_batched_f64", batch, n, _ffi.ptr(lu), n * n, _ffi.ptr(piv), n,
              _ffi.ptr(info), _stream(lu))
    if single:
        return lu[0], piv[0], info[0]
    return lu, piv, info


def lu_factor(a: torch.Tensor):
    lu, piv, _ = lu_factor_batched(a)
    return lu, piv


def diagonal_lu(a: torch.Tensor):
    """The diagonal-operator shortcut of lineax/_solver/lu.py:50-51."""
    n = a.shape[0]
    return as_f64(a), torch.arange(n, dtype=torch.int32, device=a.device)


def lu_solve_batched(lu: torch.Tensor, piv: torch.Tensor, b: torch.Tensor, trans: int = 0):
    """Solve with a batched factor.  b: (batch, n) or (batch, nrhs, n)."""
    batch, n, _ = lu.shape
    x = as_f64(b).clone()
    nrhs = 1 if x.ndim == 2 else x.shape[1]
    _ffi.call("lxgb_getrs_batched_f64", batch, n, nrhs, _ffi.ptr(lu), n * n, _ffi.ptr(piv), n,
              _ffi.ptr(x), n * nrhs, int(trans), _stream(lu))
    return x


def lu_solve(lu: torch.Tensor, piv: torch.Tensor, b: torch.Tensor, trans: int = 0):
    """Solve with one factor; b is (n,) or (nrhs, n)."""
    n = lu.shape[0]
    x = as_f64(b).clone()
    nrhs = 1 if x.ndim == 1 else x.shape[0]
    _ffi.call("lxgb_getrs_batched_f64", 1, n, nrhs, _ffi.ptr(lu), n * n, _ffi.ptr(piv), n,
              _ffi.ptr(x), n * nrhs, int(trans), _stream(lu))
    return x


# -- Cholesky ---------------------------------------------------------------


def _one_system_meta(n: int, nrhs: int, device):
    meta = torch.tensor([n, nrhs], dtype=torch.int32)
    offs = torch.zeros(2, dtype=torch.int64)
    return (meta[0:1].to(device), meta[1:2].to(device), offs[0:1].to(device),
            offs[1:2].to(device))


# Largest order factored by the one-CTA kernel (in shared memory); larger
# matrices use the multi-CTA lxgb_potrf_f64.
POTRF_ONE_CTA_MAX = 160


def gram(a: torch.Tensor, tall: bool) -> torch.Tensor:
    """AᵀA (tall) or AAᵀ (wide) of the row-major FP64 matrix a, full and
    symmetric (lxgb_syrk_f64)."""
    a = as_f64(a).contiguous()
    m, n = a.shape
    order = n if tall else m
    c = torch.empty(order, order, dtype=torch.float64, device=a.device)
    _ffi.call("lxgb_syrk_f64", 0 if tall else 1, order, m if tall else n, _ffi.ptr(a), n, 0,
              _ffi.ptr(c), order, 1, _stream(a))
    return c


def cho_factor(a: torch.Tensor, negate: bool = False) -> torch.Tensor:
    """Upper U with (±)A = Uᵀ U, zeros below the diagonal; NaNs if the matrix
    is not positive definite (jax.lax.linalg.cholesky's failure value)."""
    u = as_f64(a).clone()
    if negate:
        u.neg_()
    n = u.shape[0]
    info = torch.empty(1, dtype=torch.int32, device=u.device)
    if n > POTRF_ONE_CTA_MAX:
        # many CTAs (same bits as the one-CTA kernel)
        _ffi.call("lxgb_potrf_f64", n, _ffi.ptr(u), n, _ffi.ptr(info), _stream(u))
    else:
        nvec, _, aoff, _ = _one_system_meta(n, 1, u.device)
        _ffi.call("lxgb_potrf_ragged_f64", 1, n, _ffi.ptr(nvec), _ffi.ptr(aoff), _ffi.ptr(u),
                  _ffi.ptr(info), _stream(u))
    # A failed factorisation is reported like jax: a NaN factor, which the
    # solve turns into RESULTS.singular.
    u.masked_fill_((info != 0).reshape(1, 1), float("nan"))
    return u


# From this order on the Cholesky solve runs as two multi-CTA triangular
# solves (lxgb_trsm_f64's blocked path) instead of the one-CTA potrs.
POTRS_ONE_CTA_MAX = 767


def cho_solve(u: torch.Tensor, b: torch.Tensor, negate: bool = False) -> torch.Tensor:
    n = u.shape[0]
    if n > POTRS_ONE_CTA_MAX:
        y = trsv(u, b, lower=False, trans=True, unit=False)     # Uᵀ y = b
        x = trsv(u, y, lower=False, trans=False, unit=False)    # U x = y
        if negate:
            x.neg_()
        return x
    x = as_f64(b).clone()
    nrhs = 1 if x.ndim == 1 else x.shape[0]
    nvec, nr, aoff, boff = _one_system_meta(n, nrhs, u.device)
    _ffi.call("lxgb_potrs_ragged_f64", 1, n, _ffi.ptr(nvec), _ffi.ptr(nr), _ffi.ptr(aoff),
              _ffi.ptr(u), _ffi.ptr(boff), _ffi.ptr(x), _stream(u))
    if negate:
        x.neg_()
    return x


# -- triangular ---------------------------------------------------------------


def trsv(t: torch.Tensor, b: torch.Tensor, *, lower: bool, trans: bool, unit: bool):
    """Solve op(T) x = b; b is (n,) or (nrhs, n)."""
    t = as_f64(t)
    n = t.shape[0]  # order of the triangle; rows of t may be longer (ld = t.stride(0))
    x = as_f64(b).clone()
    nrhs = 1 if x.ndim == 1 else x.shape[0]
    _ffi.call("lxgb_trsm_f64", n, nrhs, _ffi.ptr(t), t.stride(0), int(lower), int(trans),
              int(unit), _ffi.ptr(x), _stream(t))
    return x


# -- QR -----------------------------------------------------------------------


def _workspace(nbytes: int, device) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)


def geqrf(a: torch.Tensor, already_transposed: bool = False):
    """Householder QR of the tall matrix M (a = M, or a = Mᵀ when
    already_transposed).  Returns (h, tau, t) with h = n×m in jnp.linalg.qr's
    raw layout and t the per-panel compact-WY T blocks."""
    a = as_f64(a)
    if already_transposed:
        n, m = a.shape
    else:
        m, n = a.shape
    lib = _ffi.load()
    h = torch.empty((n, m), dtype=torch.float64, device=a.device)
    tau = torch.empty(n, dtype=torch.float64, device=a.device)
    t = torch.empty(max(1, int(lib.lxgb_geqrf_t_elems(n))), dtype=torch.float64, device=a.device)
    wbytes = int(lib.lxgb_geqrf_workspace_size(m, n))
    work = _workspace(wbytes, a.device)
    _ffi.call("lxgb_geqrf_f64", m, n, _ffi.ptr(a), int(already_transposed), _ffi.ptr(h),
              _ffi.ptr(tau), _ffi.ptr(t), _ffi.ptr(work), work.numel(), _stream(a))
    return h, tau, t


def ormqr(h: torch.Tensor, tau: torch.Tensor, t: torch.Tensor, c: torch.Tensor, trans: bool):
    """Qᵀ c (trans) or Q c for c of shape (m,) or (nrhs, m); returns a new tensor."""
    n, m = h.shape
    x = as_f64(c).clone()
    nrhs = 1 if x.ndim == 1 else x.shape[0]
    wbytes = int(_ffi.load().lxgb_ormqr_workspace_size(m, nrhs))
    work = _workspace(wbytes, h.device)
    _ffi.call("lxgb_ormqr_f64", m, n, _ffi.ptr(h), _ffi.ptr(tau), _ffi.ptr(t), nrhs, _ffi.ptr(x),
              int(trans), _ffi.ptr(work), work.numel(), _stream(h))
    return x
