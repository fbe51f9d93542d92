"""Dense solves of the reference lineax path restated with SciPy LAPACK.

Test infrastructure only (see oracle/__init__.py).  Each function cites the
lineax call site whose result it reproduces.
"""

from __future__ import annotations

import numpy as np
import scipy.linalg as sl
from scipy.linalg import lapack


# ---------------------------------------------------------------------------
# LU — lineax/_solver/lu.py:43-66
# ---------------------------------------------------------------------------
def lu_factor(a: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(lu, piv) as jax.scipy.linalg.lu_factor returns them (lu.py:53): LAPACK
    getrf, 0-based swap pivots, row-major result."""
    lu, piv = sl.lu_factor(np.asarray(a, dtype=np.float64), check_finite=False)
    return np.ascontiguousarray(lu), piv.astype(np.int32)


def lu_solve(lu_piv, b: np.ndarray, trans: int = 0) -> np.ndarray:
    """jax.scipy.linalg.lu_solve(lu_piv, b, trans) at lu.py:64."""
    lu, piv = lu_piv
    return sl.lu_solve((lu, piv), b, trans=trans, check_finite=False)


def lu_linear_solve(a: np.ndarray, b: np.ndarray, transpose: bool = False) -> np.ndarray:
    """LU.init + LU.compute (lu.py:43-66); `transpose` is LU.transpose (lu.py:68-81)."""
    return lu_solve(lu_factor(a), b, trans=1 if transpose else 0)


# ---------------------------------------------------------------------------
# Cholesky — lineax/_solver/cholesky.py:43-78
# ---------------------------------------------------------------------------
def cho_factor_upper(a: np.ndarray, nsd: bool = False) -> np.ndarray:
    """cho_factor(matrix) with lower=False (cholesky.py:58-62); the matrix is
    negated first for negative-definite operators.  Returns U with zeros below
    the diagonal (jax's output layout).  A failed factorisation gives NaNs, as
    jax.lax.linalg.cholesky does."""
    m = -np.asarray(a, np.float64) if nsd else np.asarray(a, np.float64)
    try:
        u, _ = sl.cho_factor(m, lower=False, check_finite=False)
    except np.linalg.LinAlgError:
        return np.full_like(m, np.nan)
    return np.triu(u)


def cho_solve(u: np.ndarray, b: np.ndarray, nsd: bool = False) -> np.ndarray:
    """cho_solve((factor, False), vector) at cholesky.py:74, negated for NSD (:75-76)."""
    x = sl.cho_solve((u, False), b, check_finite=False)
    return -x if nsd else x


def cholesky_linear_solve(a: np.ndarray, b: np.ndarray, nsd: bool = False) -> np.ndarray:
    return cho_solve(cho_factor_upper(a, nsd), b, nsd)


# ---------------------------------------------------------------------------
# QR — lineax/_solver/qr.py:55-94
# ---------------------------------------------------------------------------
def qr_factor(a: np.ndarray) -> tuple[np.ndarray, np.ndarray, bool]:
    """QR.init (qr.py:55-65): transpose wide matrices, geqrf in raw mode.
    Returns (h, tau, transpose) with h the m×n geqrf output (R on and above the
    diagonal, Householder vectors below)."""
    m = np.asarray(a)
    transpose = m.shape[1] > m.shape[0]
    if transpose:
        m = m.T
    (h, tau), _ = sl.qr(m, mode="raw", check_finite=False)
    return np.asarray(h), np.asarray(tau), transpose


def _ormqr(h, tau, c, side, trans):
    fn = lapack.dormqr if h.dtype == np.float64 else lapack.sormqr
    lwork = max(1, 64 * max(c.shape))
    out, _, info = fn(side, trans, h, tau, c, lwork=lwork)
    if info != 0:
        raise RuntimeError(f"ormqr info={info}")
    return out


def qr_solve(state, b: np.ndarray) -> np.ndarray:
    """QR.compute (qr.py:67-94)."""
    h, tau, transpose = state
    n_full, n_min = h.shape
    r = np.triu(h[:n_min])
    if transpose:
        # minimum-norm solution: x = Q (R^{-T} b) padded (qr.py:79-86)
        y = sl.solve_triangular(r, b, trans="T", check_finite=False)
        y_pad = np.concatenate([y, np.zeros(n_full - n_min, dtype=y.dtype)])
        return _ormqr(h, tau, np.asfortranarray(y_pad[:, None]), "L", "N")[:, 0]
    # least squares (qr.py:87-92)
    qhv = _ormqr(h, tau, np.asfortranarray(np.asarray(b)[:, None]), "L", "T")[:n_min, 0]
    return sl.solve_triangular(r, qhv, trans="N", check_finite=False)


def qr_linear_solve(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    return qr_solve(qr_factor(a), b)


# ---------------------------------------------------------------------------
# Triangular — lineax/_solver/triangular.py:49-85
# ---------------------------------------------------------------------------
def normal_linear_solve(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """lineax Normal(Cholesky()) (lineax/_solver/normal.py:102-136): the
    Cholesky solve of AᵀA x = Aᵀb when A is tall (m >= n), else of
    A Aᵀ y = b followed by x = Aᵀ y; FP64 LAPACK."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    m, n = a.shape
    if m >= n:
        return cholesky_linear_solve(a.T @ a, a.T @ b)
    return a.T @ cholesky_linear_solve(a @ a.T, b)


def triangular_solve(t, b, lower: bool, unit_diagonal: bool, transpose: bool = False):
    """solve_triangular(matrix, b, trans, lower, unit_diagonal) at triangular.py:81."""
    return sl.solve_triangular(
        t, b, trans="T" if transpose else "N", lower=lower, unit_diagonal=unit_diagonal,
        check_finite=False,
    )


# ---------------------------------------------------------------------------
# Error metrics used by every parity check
# ---------------------------------------------------------------------------
def backward_error(a: np.ndarray, x: np.ndarray, b: np.ndarray) -> float:
    """Normwise relative backward error ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf),
    computed in FP64 (longdouble where the platform has more bits)."""
    a = np.asarray(a, np.float64)
    r = np.asarray(b, np.longdouble) - a.astype(np.longdouble) @ np.asarray(x, np.longdouble)
    num = float(np.max(np.abs(r))) if r.size else 0.0
    den = float(np.max(np.sum(np.abs(a), axis=1))) * float(np.max(np.abs(x))) + float(
        np.max(np.abs(b))
    )
    return num / den if den > 0 else (0.0 if num == 0 else float("inf"))


def forward_error(x: np.ndarray, x_ref: np.ndarray) -> float:
    """||x - x_ref||_inf / ||x_ref||_inf."""
    d = float(np.max(np.abs(np.asarray(x) - np.asarray(x_ref))))
    s = float(np.max(np.abs(x_ref)))
    return d / s if s > 0 else d


# ---------------------------------------------------------------------------
# Residuals without rounding error (for backward errors at full configuration
# sizes, where a longdouble product is slow on platforms without 80-bit
# hardware floats).
# ---------------------------------------------------------------------------
def _slices(m: np.ndarray, axis: int, beta: int, terms: int) -> list:
    """Split m = s_1 + ... + s_terms + rest by error-free extraction (Ozaki,
    Ogita, Oishi, Rump 2012): every slice along `axis` is a multiple of
    2^(e+1-beta), e = ceil(log2 max|row|), so it carries at most beta bits
    relative to the row's largest element; rest < 2^(1-terms*beta) of it."""
    out, r = [], np.array(m, dtype=np.float64, copy=True)
    for _ in range(terms):
        mu = np.max(np.abs(r), axis=axis, keepdims=True)
        e = np.ceil(np.log2(np.where(mu > 0, mu, 1.0)))
        sigma = np.ldexp(1.0, (e + 53 - beta).astype(np.int64))
        hi = (r + sigma) - sigma
        hi = np.where(mu > 0, hi, 0.0)
        out.append(hi)
        r = r - hi
    return out


def _two_sum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def residual_exact(a: np.ndarray, x: np.ndarray, b: np.ndarray) -> np.ndarray:
    """R = B - X Aᵀ row by row (X, B: (k, n) right-hand sides as rows; A
    (m, n)), accurate to about 2^-70 of |A||x|: A and X are cut into four
    slices each whose pairwise products sum exactly in FP64 (beta bits per
    slice with 2 beta + log2 n <= 53), and the exact partial products are
    added in double-double."""
    a = np.asarray(a, np.float64)
    x = np.atleast_2d(np.asarray(x, np.float64))
    b = np.atleast_2d(np.asarray(b, np.float64))
    n = a.shape[1]
    beta = (53 - int(np.ceil(np.log2(max(n, 2))))) // 2
    terms = 4
    sa = _slices(a, 1, beta, terms)
    sx = _slices(x, 1, beta, terms)
    hi, lo = b.copy(), np.zeros_like(b)
    for p in range(terms):
        for q in range(terms - p):
            prod = sx[q] @ sa[p].T            # exact: every partial sum fits 53 bits
            hi, e = _two_sum(hi, -prod)
            lo += e
    return hi + lo


def backward_errors_exact(a: np.ndarray, x: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Normwise backward error of every right-hand side (rows of x and b),
    ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf), with the residual
    from residual_exact."""
    x = np.atleast_2d(np.asarray(x, np.float64))
    b = np.atleast_2d(np.asarray(b, np.float64))
    r = residual_exact(a, x, b)
    anorm = float(np.max(np.sum(np.abs(np.asarray(a, np.float64)), axis=1)))
    den = anorm * np.max(np.abs(x), axis=1) + np.max(np.abs(b), axis=1)
    num = np.max(np.abs(r), axis=1)
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(den > 0, num / den, np.where(num == 0, 0.0, np.inf))
