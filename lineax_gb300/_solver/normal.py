"""Normal-equations wrapper (mirrors lineax/_solver/normal.py:17-188).

A possibly non-square A x = b is solved through the positive (semi)definite
AᵀA x = Aᵀb when A is tall (m >= n), else A Aᵀ y = b with x = Aᵀ y, by an
inner solver of definite systems.  With a ``Cholesky`` inner solver the
operator is materialised and the Gram matrix is formed once on the engine's
FP64 SYRK kernel (lxgb_syrk_f64), then factored by the multi-CTA Cholesky
(lxgb_potrf_f64); with an iterative inner solver (CG) the Gram operator stays
a composition of two matrix-vector products.  Real dtypes only, so lineax's
conjugations are identities.
"""

from __future__ import annotations

from copy import copy

from .. import _dense
from .._operator import (
    MatrixLinearOperator,
    TaggedLinearOperator,
    linearise,
    materialise,
)
from .._solve import AbstractLinearSolver
from .._tags import positive_semidefinite_tag, symmetric_tag
from .cholesky import Cholesky


def normal_preconditioner_and_y0(options: dict, tall: bool) -> dict:
    """normal.py:17-37: the preconditioner M becomes M Mᵀ (tall) or Mᵀ M
    (wide), and in the wide form y0 becomes Mᵀ y0."""
    preconditioner = options.get("preconditioner")
    y0 = options.get("y0")
    inner_options = copy(options)
    if preconditioner is not None:
        preconditioner = linearise(preconditioner)
        if tall:
            inner_options["preconditioner"] = TaggedLinearOperator(
                preconditioner @ preconditioner.transpose(), positive_semidefinite_tag)
        else:
            inner_options["preconditioner"] = TaggedLinearOperator(
                preconditioner.transpose() @ preconditioner, positive_semidefinite_tag)
            if y0 is not None:
                inner_options["y0"] = preconditioner.transpose().mv(y0)
    return inner_options


class Normal(AbstractLinearSolver):
    """Wrap an inner solver of positive (semi)definite systems so that it
    solves possibly non-square systems through the normal equations."""

    def __init__(self, inner_solver: AbstractLinearSolver):
        self.inner_solver = inner_solver

    def __repr__(self):
        return f"Normal({self.inner_solver!r})"

    def init(self, operator, options):
        tall = operator.out_size() >= operator.in_size()
        if isinstance(self.inner_solver, Cholesky):
            # normal.py:105-118 materialises first for Cholesky; here the
            # Gram matrix comes from one SYRK instead of (Aᵀ @ A).as_matrix().
            lin_op = materialise(operator)
            gram = _dense.gram(lin_op.matrix, tall)
            inner_operator = MatrixLinearOperator(gram, (positive_semidefinite_tag, symmetric_tag))
        else:
            lin_op = linearise(operator)
            if tall:
                inner_operator = lin_op.transpose() @ lin_op
            else:
                inner_operator = lin_op @ lin_op.transpose()
            inner_operator = TaggedLinearOperator(inner_operator, positive_semidefinite_tag)
        inner_options = normal_preconditioner_and_y0(options, tall)
        inner_state = self.inner_solver.init(inner_operator, inner_options)
        operator_transpose = lin_op.transpose()
        return inner_state, tall, operator_transpose, inner_options

    def compute(self, state, vector, options):
        inner_state, tall, operator_transpose, inner_options = state
        if tall:
            vector = operator_transpose.mv(vector)
        solution, result, stats = self.inner_solver.compute(inner_state, vector, inner_options)
        if not tall:
            solution = operator_transpose.mv(solution)
        return solution, result, stats

    def transpose(self, state, options):
        inner_state, tall, operator_transpose, inner_options = state
        inner_state_conj, inner_options = self.inner_solver.conj(inner_state, inner_options)
        return (inner_state_conj, not tall, operator_transpose.transpose(), inner_options), options

    def conj(self, state, options):
        inner_state, tall, operator_transpose, inner_options = state
        inner_state_conj, inner_options = self.inner_solver.conj(inner_state, inner_options)
        return (inner_state_conj, tall, operator_transpose, inner_options), options

    def assume_full_rank(self):
        return self.inner_solver.assume_full_rank()
