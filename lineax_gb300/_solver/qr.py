"""QR solver (mirrors lineax/_solver/qr.py:40-118) on lxgb_geqrf_f64 /
lxgb_ormqr_f64 / lxgb_trsm_f64.

The factor is stored as jnp.linalg.qr(mode="raw") returns it: h = Mᵀ (n_min
rows) for the tall matrix M (the operator, or its transpose when it is wide).
Rᵀ is the lower triangle of h's first n_min columns, so R solves are
triangular solves on h with leading dimension n_full.
"""

from __future__ import annotations

import torch

from .. import _dense
from .._solution import RESULTS
from .._solve import AbstractLinearSolver
from .misc import pack_structures, ravel_vector, transpose_packed_structures, unravel_solution


class QR(AbstractLinearSolver):
    """QR solver: least squares for tall operators, minimum norm for wide ones,
    the usual solution for square nonsingular ones (full rank assumed).

    ``precision="mixed"`` (an extension, tall operators with a row count that
    is a multiple of 4): TF32 tensor-core QR and corrected semi-normal
    equations refined to FP64 accuracy (``mixed.qr_lstsq``); other shapes use
    the FP64 path."""

    def __init__(self, precision: str = "fp64"):
        if precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        self.precision = precision

    def __repr__(self):
        return "QR()"

    def init(self, operator, options):
        matrix = operator.as_matrix()
        m, n = matrix.shape
        transpose = n > m
        if self.precision == "mixed" and not transpose and m % 4 == 0:
            from .. import mixed

            a64 = matrix.to(torch.float64).contiguous()
            return (mixed.qr_factor_tf32(a64), a64), "mixed", pack_structures(operator)
        # QR.init factors M = matrix (tall) or M = matrixᵀ (wide, qr.py:59-61);
        # h = Mᵀ is `matrix` itself in the wide case.
        h, tau, t = _dense.geqrf(matrix, already_transposed=transpose)
        return (h, tau, t), transpose, pack_structures(operator)

    def compute(self, state, vector, options):
        if state[1] == "mixed":
            from .. import mixed

            (factor, a64), _, packed = state
            b = ravel_vector(vector, packed)
            res = mixed.qr_lstsq(a64, b, factor=factor)
            return unravel_solution(res.x[0], packed), RESULTS.successful, {
                "refinement_steps": res.iters}
        (h, tau, t), transpose, packed = state
        b = ravel_vector(vector, packed)
        n_min, n_full = h.shape
        if transpose:
            # minimum norm: x = Q [R^{-T} b; 0] (qr.py:79-86)
            y = _dense.trsv(h, b, lower=True, trans=False, unit=False)
            pad = torch.zeros(n_full, dtype=torch.float64, device=b.device)
            pad[:n_min] = y
            x = _dense.ormqr(h, tau, t, pad, trans=False)
        else:
            # least squares: x = R^{-1} (Qᵀ b)[:n_min] (qr.py:87-92)
            qhb = _dense.ormqr(h, tau, t, b, trans=True)[:n_min].contiguous()
            x = _dense.trsv(h, qhb, lower=True, trans=True, unit=False)
        return unravel_solution(x, packed), RESULTS.successful, {}

    def transpose(self, state, options):
        if state[1] == "mixed":
            raise NotImplementedError("transpose of the mixed-precision QR state")
        factor, transpose, packed = state
        return (factor, not transpose, transpose_packed_structures(packed)), {}

    def conj(self, state, options):
        return state, {}

    def assume_full_rank(self):
        return True
