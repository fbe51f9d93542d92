"""Diagonal solver (lineax/_solver/diagonal.py:36-116), the target of
AutoLinearSolver for diagonal-tagged and 1×1 operators."""

from __future__ import annotations

import torch

from .. import _ffi
from .._blas import as_device_f64
from .._operator import is_diagonal
from .._solution import RESULTS
from .._solve import AbstractLinearSolver
from .misc import pack_structures, ravel_vector, transpose_packed_structures, unravel_solution


class Diagonal(AbstractLinearSolver):
    """x = b / diag(A); with well_posed=False zero entries give zero (pseudo-inverse)."""

    def __init__(self, well_posed: bool = False):
        self.well_posed = well_posed

    def __repr__(self):
        return f"Diagonal(well_posed={self.well_posed})"

    def init(self, operator, options):
        if operator.in_size() != operator.out_size():
            raise ValueError("`Diagonal` may only be used for linear solves with square matrices")
        if not is_diagonal(operator):
            raise ValueError("`Diagonal` may only be used for linear solves with diagonal matrices")
        return as_device_f64(operator.as_matrix()), pack_structures(operator)

    def compute(self, state, vector, options):
        matrix, packed = state
        b = ravel_vector(vector, packed)
        x = torch.empty_like(b)
        n = b.numel()
        _ffi.call("lxgb_diag_solve_f64", n, _ffi.ptr(matrix), n + 1, _ffi.ptr(b), _ffi.ptr(x),
                  int(self.well_posed), _ffi.stream_handle(b.device))
        return unravel_solution(x, packed), RESULTS.successful, {}

    def transpose(self, state, options):
        matrix, packed = state
        return (matrix, transpose_packed_structures(packed)), options

    def conj(self, state, options):
        return state, options

    def assume_full_rank(self):
        return self.well_posed
