"""linear_solve, the solver interface and automatic solver selection
(mirrors lineax/_solve.py).

`linear_solve` keeps lineax's contract (lineax/_solve.py:656-806): it checks
the vector against the operator's out-structure, runs ``solver.init`` unless a
state is supplied, calls ``solver.compute``, maps non-finite output to
RESULTS.singular and non-finite input to RESULTS.nonfinite_input
(lineax/_solve.py:104-123), raises on failure when ``throw=True``, and returns
a Solution.
"""

from __future__ import annotations

import abc
import contextlib
from typing import Any

import torch

from . import _blas
from ._operator import (
    AbstractLinearOperator,
    FunctionLinearOperator,
    IdentityLinearOperator,
    has_unit_diagonal,
    is_diagonal,
    is_lower_triangular,
    is_negative_semidefinite,
    is_positive_semidefinite,
    is_symmetric,
    is_tridiagonal,
    is_upper_triangular,
)
from ._solution import RESULTS, LinearSolveError, Solution
from ._structure import structure_equal, structure_of, tree_flatten
from ._tags import (
    diagonal_tag,
    lower_triangular_tag,
    negative_semidefinite_tag,
    positive_semidefinite_tag,
    symmetric_tag,
    unit_diagonal_tag,
    upper_triangular_tag,
)

sentinel: Any = object()


class AbstractLinearSolver(abc.ABC):
    """The five-method solver contract of lineax/_solve.py:343-480."""

    @abc.abstractmethod
    def init(self, operator: AbstractLinearOperator, options: dict) -> Any:
        """Work done on the operator alone (e.g. a factorisation)."""

    @abc.abstractmethod
    def compute(self, state: Any, vector, options: dict) -> tuple[Any, int, dict]:
        """Solve against `vector`: returns (solution, RESULTS code, stats)."""

    @abc.abstractmethod
    def transpose(self, state: Any, options: dict) -> tuple[Any, dict]:
        """State (and options) of the transposed operator, reusing the work done."""

    @abc.abstractmethod
    def conj(self, state: Any, options: dict) -> tuple[Any, dict]:
        """State (and options) of the conjugated operator."""

    @abc.abstractmethod
    def assume_full_rank(self) -> bool:
        """Whether the solver assumes a full-rank operator."""


_qr_token = "qr_token"
_diagonal_token = "diagonal_token"
_well_posed_diagonal_token = "well_posed_diagonal_token"
_tridiagonal_token = "tridiagonal_token"
_triangular_token = "triangular_token"
_cholesky_token = "cholesky_token"
_lu_token = "lu_token"
_svd_token = "svd_token"


def _lookup(token) -> AbstractLinearSolver:
    from . import _solver

    table = {
        _qr_token: _solver.QR,
        _triangular_token: _solver.Triangular,
        _cholesky_token: _solver.Cholesky,
        _lu_token: _solver.LU,
        _diagonal_token: _solver.Diagonal,
        _well_posed_diagonal_token: lambda: _solver.Diagonal(well_posed=True),
    }
    if token not in table:
        raise NotImplementedError(
            f"AutoLinearSolver selected `{token}`, which lineax_gb300 does not implement "
            "(its GPU engine covers LU, Cholesky, QR, Triangular, CG and GMRES)."
        )
    return table[token]()


class AutoLinearSolver(AbstractLinearSolver):
    """Picks a solver from the operator's structure (lineax/_solve.py:518-645)."""

    def __init__(self, well_posed: bool | None):
        self.well_posed = well_posed

    def __repr__(self):
        return f"AutoLinearSolver(well_posed={self.well_posed})"

    def _select_solver(self, operator):
        """lineax/_solve.py:555-600."""
        if self.well_posed is True:
            if operator.in_size() != operator.out_size():
                raise ValueError(
                    "Cannot use `AutoLinearSolver(well_posed=True)` with a non-square "
                    "operator. If you are trying solve a least-squares problem then "
                    "you should pass `solver=AutoLinearSolver(well_posed=False)`. By "
                    "default `lineax.linear_solve` assumes that the operator is "
                    "square and nonsingular."
                )
            if is_diagonal(operator):
                return _well_posed_diagonal_token
            if is_tridiagonal(operator):
                return _tridiagonal_token
            if is_lower_triangular(operator) or is_upper_triangular(operator):
                return _triangular_token
            if is_positive_semidefinite(operator) or is_negative_semidefinite(operator):
                return _cholesky_token
            return _lu_token
        if self.well_posed is False:
            return _diagonal_token if is_diagonal(operator) else _svd_token
        if self.well_posed is None:
            if operator.in_size() != operator.out_size():
                return _qr_token
            if is_diagonal(operator):
                return _diagonal_token
            if is_tridiagonal(operator):
                return _tridiagonal_token
            if is_lower_triangular(operator) or is_upper_triangular(operator):
                return _triangular_token
            if is_positive_semidefinite(operator) or is_negative_semidefinite(operator):
                return _cholesky_token
            return _lu_token
        raise ValueError(f"Invalid value `well_posed={self.well_posed}`.")

    def select_solver(self, operator) -> AbstractLinearSolver:
        return _lookup(self._select_solver(operator))

    def init(self, operator, options):
        token = self._select_solver(operator)
        return token, _lookup(token).init(operator, options)

    def compute(self, state, vector, options):
        token, inner = state
        solution, result, _ = _lookup(token).compute(inner, vector, options)
        return solution, result, {}

    def transpose(self, state, options):
        token, inner = state
        st, opts = _lookup(token).transpose(inner, options)
        return (token, st), opts

    def conj(self, state, options):
        token, inner = state
        st, opts = _lookup(token).conj(inner, options)
        return (token, st), opts

    def assume_full_rank(self):
        return self.well_posed is not False


def _any_nonfinite(tree) -> bool:
    leaves, _ = tree_flatten(tree)
    leaves = [torch.view_as_real(x.to(torch.complex128)) if x.is_complex() else x
              for x in leaves]
    flags = [_blas.any_nonfinite(x) for x in leaves if x.numel() > 0]
    if not flags:
        return False
    return bool(torch.cat(flags).any().item())


def _finalize(solution, result: int, vector) -> int:
    """lineax/_solve.py:104-123."""
    if result == RESULTS.successful and _any_nonfinite(solution):
        result = RESULTS.singular
    if result == RESULTS.singular and _any_nonfinite(vector):
        result = RESULTS.nonfinite_input
    return result


def linear_solve(
    operator: AbstractLinearOperator,
    vector,
    solver: AbstractLinearSolver | None = None,
    *,
    options: dict | None = None,
    state: Any = sentinel,
    throw: bool = True,
) -> Solution:
    """Solve ``operator @ x = vector`` (lineax/_solve.py:656-806).

    The default solver is ``AutoLinearSolver(well_posed=True)``.  With
    ``throw=False`` failures are reported in ``Solution.result`` instead of
    raised.
    """
    if solver is None:
        solver = AutoLinearSolver(well_posed=True)
    if isinstance(operator, torch.Tensor):
        raise ValueError(
            "`lineax.linear_solve(operator=...)` should be an `AbstractLinearOperator`, not a "
            "raw array. If you are trying to pass a matrix then this should be passed as "
            "`lineax.MatrixLinearOperator(matrix)`."
        )
    if options is None:
        options = {}
    leaves, td = tree_flatten(vector)
    fixed = []
    for x in leaves:
        if not isinstance(x, torch.Tensor):
            x = torch.as_tensor(x, device="cuda")
        if not torch.is_floating_point(x) and not x.is_complex():
            x = x.to(torch.get_default_dtype())
        fixed.append(x)
    from ._structure import tree_unflatten

    vector = tree_unflatten(td, fixed)
    if not structure_equal(structure_of(vector), operator.out_structure()):
        raise ValueError(
            "Vector and operator structures do not match. Got a vector with structure "
            f"{structure_of(vector)} and an operator with out-structure "
            f"{operator.out_structure()}"
        )
    if isinstance(operator, IdentityLinearOperator):
        return Solution(value=vector, result=RESULTS.successful, state=state, stats={})
    from . import _complex

    if _complex.operator_is_complex(operator) or _complex.tree_is_complex(vector):
        # complex problems run on real forms of the operator (see _complex)
        solution, result, stats, state = _complex.linear_solve_complex(
            operator, vector, solver, options, state, sentinel)
        result = _finalize(solution, int(result), vector)
        if throw and result != RESULTS.successful:
            raise LinearSolveError(result)
        return Solution(value=solution, result=result, state=state, stats=stats)
    from . import _autodiff

    diff = _autodiff.needs_grad(operator, vector)
    with torch.no_grad() if diff else contextlib.nullcontext():
        if state is sentinel:
            state = solver.init(operator, options)
        solution, result, stats = solver.compute(state, vector, options)
    result = _finalize(solution, int(result), vector)
    if throw and result != RESULTS.successful:
        raise LinearSolveError(result)
    if diff:
        # derivative rules of lineax/_solve.py:151-317 (see _autodiff)
        solution = _autodiff.differentiable(
            operator, vector, solution, _autodiff.SolveContext(operator, solver, state, options))
    return Solution(value=solution, result=result, state=state, stats=stats)


def invert(operator, solver=None, *, options=None, throw=True) -> FunctionLinearOperator:
    """A FunctionLinearOperator applying the (pseudo)inverse of `operator`,
    with the factorisation done once (lineax/_solve.py:809-871)."""
    if solver is None:
        solver = AutoLinearSolver(well_posed=True)
    if options is None:
        options = {}
    state = solver.init(operator, options)

    def solve_fn(vector):
        return linear_solve(operator, vector, solver, state=state, options=options,
                            throw=throw).value

    tags = {
        tag
        for check, tag in [
            (is_symmetric, symmetric_tag),
            (is_diagonal, diagonal_tag),
            (is_lower_triangular, lower_triangular_tag),
            (is_upper_triangular, upper_triangular_tag),
            (is_positive_semidefinite, positive_semidefinite_tag),
            (is_negative_semidefinite, negative_semidefinite_tag),
        ]
        if check(operator)
    }
    if has_unit_diagonal(operator) and (
        is_diagonal(operator) or is_lower_triangular(operator) or is_upper_triangular(operator)
    ):
        tags.add(unit_diagonal_tag)
    return FunctionLinearOperator(solve_fn, operator.out_structure(), frozenset(tags),
                                  output_structure=operator.in_structure())
