"""Cholesky solver (mirrors lineax/_solver/cholesky.py:32-92) on the engine's
ragged potrf/potrs kernels (a batch of one)."""

from __future__ import annotations

from .. import _dense
from .._operator import is_negative_semidefinite, is_positive_semidefinite
from .._solution import RESULTS
from .._solve import AbstractLinearSolver
from .._structure import ravel, structure_of, unravel


class Cholesky(AbstractLinearSolver):
    """Cholesky solver for positive or negative definite operators.

    State: (upper factor U with A = Uᵀ U, is_nsd) as in cholesky.py:41.
    """

    def __repr__(self):
        return "Cholesky()"

    def init(self, operator, options):
        is_nsd = is_negative_semidefinite(operator)
        if not (is_positive_semidefinite(operator) or is_nsd):
            raise ValueError(
                "`Cholesky(..., normal=False)` may only be used for positive "
                "or negative definite linear operators"
            )
        matrix = operator.as_matrix()
        m, n = matrix.shape
        if m != n:
            raise ValueError(
                "`Cholesky(..., normal=False)` may only be used for linear solves "
                "with square matrices"
            )
        factor = _dense.cho_factor(matrix, negate=is_nsd)
        return factor, is_nsd

    def compute(self, state, vector, options):
        factor, is_nsd = state
        structure = structure_of(vector)
        b = ravel(vector, factor.dtype).contiguous()
        x = _dense.cho_solve(factor, b, negate=is_nsd)
        return unravel(x, structure), RESULTS.successful, {}

    def transpose(self, state, options):
        return state, options

    def conj(self, state, options):
        return state, options

    def assume_full_rank(self):
        return True
