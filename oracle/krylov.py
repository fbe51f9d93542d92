"""Statement-for-statement NumPy restatements of lineax's CG, GMRES and BiCGStab.

Test infrastructure only (see oracle/__init__.py).  One right-hand side per
call: under ``jax.vmap`` the reference evaluates every batch element exactly
as it would alone (converged elements are masked by select, and the shared
``unvmap_max(step)`` equals every still-active element's own step), so a
batch is the same as independent calls.

`matvec` and `precond` are callables on 1-D float64 arrays.
"""

from __future__ import annotations

import numpy as np

from .dense import qr_linear_solve

SUCCESSFUL, MAX_STEPS_REACHED, SINGULAR, BREAKDOWN, STAGNATION = 0, 1, 2, 3, 4


def max_norm(x: np.ndarray) -> float:
    """lineax/_norm.py:123-143 — max |x|, NaN-propagating like jnp.max."""
    if x.size == 0:
        return 0.0
    return float(np.max(np.abs(x)))


def two_norm(x: np.ndarray) -> float:
    """lineax/_norm.py:59-77 — |x| for a single element, else sqrt(sum x^2)."""
    if x.size == 1:
        return float(abs(x.reshape(())))
    return float(np.sqrt(np.dot(x, x)))


def _resolve_rcond(size: int, dtype) -> float:
    """lineax/_misc.py:30-38 with rcond=None."""
    return 2 * float(np.finfo(dtype).eps) * size


def _has_scale(rtol, atol) -> bool:
    return not (atol == 0 and rtol == 0)


def _not_converged(r, diff, y, b_scale, rtol, atol, norm) -> bool:
    """cg.py:149-160 / gmres.py:130-141 — the two-space test."""
    if b_scale is None:
        return True
    with np.errstate(divide="ignore", invalid="ignore"):
        y_scale = atol + rtol * np.abs(y)
        norm1 = norm(r / b_scale)
        norm2 = norm(diff / y_scale)
    return bool(norm1 > 1) or bool(norm2 > 1)


def cg(matvec, b, *, rtol, atol, norm=max_norm, stabilise_every=10, max_steps=None,
       precond=None, y0=None, nsd=False):
    """lineax CG (cg.py:88-227).  `nsd` reproduces init's negation of a
    negative-definite operator (cg.py:100-101) and compute's sign flip (:224-225).
    Returns (solution, result, num_steps)."""
    b = np.asarray(b, np.float64)
    if nsd:
        mv = lambda v: -matvec(v)  # noqa: E731
    else:
        mv = matvec
    pre = precond if precond is not None else (lambda v: v)
    y0 = np.zeros_like(b) if y0 is None else np.asarray(y0, np.float64)
    size = b.size
    max_steps_ = 10 * size if max_steps is None else max_steps
    r = b - mv(y0)
    p = pre(r)
    gamma = float(np.dot(p, r))
    rcond = _resolve_rcond(size, np.float64)
    diff = np.full_like(y0, np.inf)
    y = y0
    step = 0
    b_scale = (atol + rtol * np.abs(b)) if _has_scale(rtol, atol) else None

    def cond(diff, y, r, gamma, step):
        out = gamma > 0
        out = out and (step < max_steps_)
        return out and _not_converged(r, diff, y, b_scale, rtol, atol, norm)

    while cond(diff, y, r, gamma, step):
        mat_p = mv(p)
        inner_prod = float(np.dot(mat_p, p))
        with np.errstate(divide="ignore", invalid="ignore"):
            alpha = float(np.float64(gamma) / np.float64(inner_prod))
        if not (abs(inner_prod) > 100 * rcond * abs(gamma)):
            alpha = np.nan
        diff = alpha * p
        y = y + diff
        step += 1
        if stabilise_every == 1:
            r = b - mv(y)
        elif stabilise_every is None:
            r = r - alpha * mat_p
        elif step % stabilise_every == 0:
            r = b - mv(y)
        else:
            r = r - alpha * mat_p
        z = pre(r)
        gamma_prev = gamma
        gamma = float(np.dot(z, r))
        with np.errstate(divide="ignore", invalid="ignore"):
            beta = np.float64(gamma) / np.float64(gamma_prev)
        p = z + beta * p
    num_steps = step
    if max_steps is None:
        result = SINGULAR if num_steps == max_steps_ else SUCCESSFUL
    elif b_scale is not None:
        result = MAX_STEPS_REACHED if num_steps == max_steps_ else SUCCESSFUL
    else:
        result = SUCCESSFUL
    sol = -y if nsd else y
    return sol, result, num_steps


def _normalise(x, eps):
    """gmres.py:401-413."""
    nrm = two_norm(x)
    if eps is None:
        eps = float(np.finfo(np.float64).eps)
    breakdown = nrm < eps
    safe = np.inf if breakdown else nrm
    return x / safe, nrm, breakdown


def _arnoldi(mv, pre, basis, coeff, step, initial_breakdown):
    """gmres.py:331-399 — one step of single-pass classical Gram-Schmidt."""
    w = pre(mv(basis[:, step]))
    step_norm = two_norm(w)
    proj = basis.T @ w
    w_new = w - basis @ proj
    eps = step_norm * float(np.finfo(np.float64).eps)
    wn, wnorm, breakdown = _normalise(w_new, eps)
    basis = basis.copy()
    basis[:, step + 1] = wn
    proj = proj.copy()
    proj[step + 1] = wnorm
    if not initial_breakdown:
        coeff = coeff.copy()
        coeff[step, :] = proj
    return basis, coeff, breakdown


def gmres(matvec, b, *, rtol, atol, norm=max_norm, max_steps=None, restart=20,
          stagnation_iters=20, precond=None, y0=None, return_stats=False):
    """lineax GMRES (gmres.py:106-240).  Returns (solution, result, num_steps)."""
    b = np.asarray(b, np.float64)
    mv = matvec
    pre = precond if precond is not None else (lambda v: v)
    y0 = np.zeros_like(b) if y0 is None else np.asarray(y0, np.float64)
    size = b.size
    max_steps_ = 10 * size if max_steps is None else max_steps
    restart = min(restart, size)
    b_scale = (atol + rtol * np.abs(b)) if _has_scale(rtol, atol) else None

    def not_conv(r, diff, y):
        return _not_converged(r, diff, y, b_scale, rtol, atol, norm)

    def gmres_compute(y, r, first_pass):
        """gmres.py:242-320."""
        if first_pass:
            y_new, diff, breakdown = y, np.full_like(y, np.inf), False
        else:
            r_n, r_norm, breakdown = _normalise(r, None)
            basis = np.zeros((size, restart + 1))
            basis[:, 0] = r_n
            coeff = np.eye(restart, restart + 1)
            k = 0
            while k < restart and not breakdown:
                basis, coeff, breakdown = _arnoldi(mv, pre, basis, coeff, k, breakdown)
                k += 1
            beta_vec = np.zeros(restart + 1)
            beta_vec[0] = r_norm
            with np.errstate(all="ignore"):
                try:
                    z = qr_linear_solve(coeff.T, beta_vec)
                except (ValueError, np.linalg.LinAlgError):
                    z = np.full(restart, np.nan)
                diff = basis[:, :-1] @ z
            y_new = y + diff
        with np.errstate(all="ignore"):
            r_new = pre(b - mv(y_new))
        return y_new, r_new, breakdown, diff

    y = y0
    r = np.zeros_like(b)
    breakdown = False
    deferred = False
    diff = np.full_like(y0, np.inf)
    r_min = np.inf
    step = 0
    stag = 0

    def cond():
        out = (not deferred) and (stag < stagnation_iters)
        out = out and not_conv(r, diff, y)
        out = out and (step < max_steps_)
        return out or step == 0

    while cond():
        prev_breakdown = breakdown
        y, r, breakdown, diff = gmres_compute(y, r, step == 0)
        deferred = prev_breakdown
        r_norm = norm(r)
        with np.errstate(invalid="ignore"):
            decreased = (r_norm - r_min) < 0
        stag = 0 if decreased else stag + 1
        r_min = float(np.minimum(r_norm, r_min))
        step += 1
    num_steps = step
    if max_steps is None:
        result = SINGULAR if num_steps == max_steps_ else SUCCESSFUL
    elif b_scale is not None:
        result = MAX_STEPS_REACHED if num_steps == max_steps_ else SUCCESSFUL
    else:
        result = SUCCESSFUL
    if stag >= stagnation_iters:
        result = STAGNATION
    if deferred and not_conv(r, diff, y):
        result = BREAKDOWN
    return y, result, num_steps


def bicgstab(matvec, b, *, rtol, atol, norm=max_norm, max_steps=None, precond=None,
             y0=None):
    """lineax BiCGStab (lineax/_solver/bicgstab.py:78-205), right-preconditioned,
    FP64 (the ``jax_enable_x64`` branch of the breakdown test, :107-113).
    Returns (solution, result, num_steps)."""
    b = np.asarray(b, np.float64)
    pre = precond if precond is not None else (lambda v: v)
    y0 = np.zeros_like(b) if y0 is None else np.asarray(y0, np.float64)
    size = b.size
    max_steps_ = 10 * size if max_steps is None else max_steps          # :82-88
    b_scale = (atol + rtol * np.abs(b)) if _has_scale(rtol, atol) else None  # :89-96
    r0 = b - matvec(y0)                                                  # :105

    def breakdown_occurred(omega, alpha, rho):                          # :107-113
        return omega == 0.0 or alpha == 0.0 or rho == 0.0

    def not_converged(r, diff, y):                                       # :115-126
        return _not_converged(r, diff, y, b_scale, rtol, atol, norm)

    y, r = y0, r0
    alpha = omega = rho = 1.0                                            # :171
    p = np.zeros_like(b)
    v = np.zeros_like(b)
    diff = np.full_like(y0, np.inf)
    step = 0
    # cond_fun :128-133
    while (not breakdown_occurred(omega, alpha, rho)) and not_converged(r, diff, y) \
            and step < max_steps_:
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            rho_new = float(np.dot(r0, r))                               # :138
            beta = (np.float64(rho_new) / np.float64(rho)) * (np.float64(alpha) / np.float64(omega))
            p = r + beta * (p - omega * v)                               # :140
            x = pre(p)                                                   # :144
            v = matvec(x)
            alpha = float(np.float64(rho_new) / np.float64(np.dot(r0, v)))  # :147
            s = r - alpha * v
            z = pre(s)                                                   # :150
            t = matvec(z)
            omega = float(np.float64(np.dot(s, t)) / np.float64(np.dot(t, t)))  # :153
            diff = alpha * x + omega * z                                 # :155
            y = y + diff
            r = s - omega * t
        rho = rho_new
        step += 1
    if max_steps is None:                                                # :188-197
        result = SINGULAR if step == max_steps_ else SUCCESSFUL
    elif b_scale is not None:
        result = MAX_STEPS_REACHED if step == max_steps_ else SUCCESSFUL
    else:
        result = SUCCESSFUL
    if breakdown_occurred(omega, alpha, rho) and not_converged(r, diff, y):  # :199-202
        result = BREAKDOWN
    return y, result, step


def finalize_result(x, result, b) -> int:
    """lineax/_solve.py:104-123 — non-finite output → singular; non-finite
    input turns singular into nonfinite_input."""
    if result == SUCCESSFUL and not np.all(np.isfinite(x)):
        result = SINGULAR
    if result == SINGULAR and not np.all(np.isfinite(b)):
        result = 6
    return result
