"""Triangular solver (mirrors lineax/_solver/triangular.py:36-115) on lxgb_trsm_f64."""

from __future__ import annotations

from .. import _dense
from .._operator import has_unit_diagonal, is_lower_triangular, is_upper_triangular
from .._solution import RESULTS
from .._solve import AbstractLinearSolver
from .misc import pack_structures, ravel_vector, transpose_packed_structures, unravel_solution


class Triangular(AbstractLinearSolver):
    """Solver for lower- or upper-triangular operators (tags decide which)."""

    def __repr__(self):
        return "Triangular()"

    def init(self, operator, options):
        if operator.in_size() != operator.out_size():
            raise ValueError(
                "`Triangular` may only be used for linear solves with square matrices"
            )
        if not (is_lower_triangular(operator) or is_upper_triangular(operator)):
            raise ValueError(
                "`Triangular` may only be used for linear solves with triangular matrices"
            )
        return (
            _dense.as_f64(operator.as_matrix()),
            is_lower_triangular(operator),
            has_unit_diagonal(operator),
            pack_structures(operator),
            False,
        )

    def compute(self, state, vector, options):
        matrix, lower, unit, packed, transpose = state
        b = ravel_vector(vector, packed)
        x = _dense.trsv(matrix, b, lower=lower, trans=transpose, unit=unit)
        return unravel_solution(x, packed), RESULTS.successful, {}

    def transpose(self, state, options):
        matrix, lower, unit, packed, transpose = state
        return (matrix, lower, unit, transpose_packed_structures(packed), not transpose), {}

    def conj(self, state, options):
        return state, {}

    def assume_full_rank(self):
        return True
