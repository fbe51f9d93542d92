"""LU solver (mirrors lineax/_solver/lu.py:32-98) on the engine's getrf/getrs."""

from __future__ import annotations

from .. import _dense
from .._operator import is_diagonal
from .._solution import RESULTS
from .._solve import AbstractLinearSolver
from .misc import pack_structures, ravel_vector, transpose_packed_structures, unravel_solution


class LU(AbstractLinearSolver):
    """LU solver for square nonsingular operators.

    State: ((lu, piv), packed structures, transpose flag) as in lu.py:34.  The
    factor is computed by lxgb_getrf_batched_f64 (FP64, partial pivoting,
    pivots identical to LAPACK getf2 on the same input).
    """

    def __repr__(self):
        return "LU()"

    def init(self, operator, options):
        if operator.in_size() != operator.out_size():
            raise ValueError("`LU` may only be used for linear solves with square matrices")
        packed = pack_structures(operator)
        matrix = operator.as_matrix()
        if is_diagonal(operator):
            lu = _dense.diagonal_lu(matrix)
        else:
            lu = _dense.lu_factor(matrix)
        return lu, packed, False

    def compute(self, state, vector, options):
        (lu, piv), packed, transpose = state
        b = ravel_vector(vector, packed)
        x = _dense.lu_solve(lu, piv, b, trans=1 if transpose else 0)
        return unravel_solution(x, packed), RESULTS.successful, {}

    def transpose(self, state, options):
        lu_piv, packed, transpose = state
        return (lu_piv, transpose_packed_structures(packed), not transpose), {}

    def conj(self, state, options):
        # Real factors only; lineax flips the transpose flag here (lu.py:83-95).
        (lu, piv), packed, transpose = state
        return ((lu, piv), packed, not transpose), {}

    def assume_full_rank(self):
        return True
