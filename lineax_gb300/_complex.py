"""Complex operators and vectors (lineax runs every solver on complex128:
tests/test_well_posed.py:33), solved through real forms on the engine's FP64
kernels.

A complex linear map A: Cᵐ → Cⁿ acts on real coordinates [Re x; Im x] as the
real 2n×2m operator

    R(A) = [[Re A, -Im A],
            [Im A,  Re A]],

with the properties the solvers rely on:
  * R(A) is nonsingular exactly when A is (LU);
  * ‖R(A)[xr; xi] - [br; bi]‖₂ = ‖A x - b‖₂ and ‖[xr; xi]‖₂ = ‖x‖₂, so least
    squares and minimum-norm solutions correspond (QR, Normal);
  * A Hermitian positive (negative) definite ⇒ R(A) symmetric positive
    (negative) definite (Cholesky, CG) — lineax's positive_semidefinite_tag
    means Hermitian for complex operators (lineax/_operator.py:1605-1625);
  * Rᵀ = R(Aᴴ), the conjugate transpose, so real-arithmetic solvers that use
    the transpose (Normal, QR's minimum-norm branch) form Aᴴ A / A Aᴴ.
Diagonal operators are solved elementwise in complex arithmetic.  Triangular
operators are scaled by their diagonal, D⁻¹T x = D⁻¹b, which gives a unit
diagonal; with the unknowns interleaved (Re x₀, Im x₀, Re x₁, …) the real form
of a unit triangular matrix is itself unit triangular, so the engine's real
triangular solve applies unchanged (O(n²) work, no factorisation).

Krylov iterations on R(A) run over the real span of the Krylov vectors, so
step counts can differ from a complex-arithmetic CG or GMRES; the solutions
agree to the requested tolerance.
"""

from __future__ import annotations

import torch

from ._structure import ShapeDtypeStruct, ravel, tree_flatten, tree_size, tree_unflatten, unravel
from ._tags import negative_semidefinite_tag, positive_semidefinite_tag, symmetric_tag

COMPLEX_STATE = "lineax_gb300.complex"


def is_complex_dtype(dtype) -> bool:
    return dtype in (torch.complex64, torch.complex128)


def structure_is_complex(structure) -> bool:
    leaves, _ = tree_flatten(structure)
    return any(is_complex_dtype(x.dtype) for x in leaves)


def operator_is_complex(operator) -> bool:
    return structure_is_complex(operator.in_structure()) or structure_is_complex(
        operator.out_structure())


def tree_is_complex(tree) -> bool:
    leaves, _ = tree_flatten(tree)
    return any(isinstance(x, torch.Tensor) and x.is_complex() for x in leaves)


def real_form_matrix(a: torch.Tensor) -> torch.Tensor:
    """R(A) as a contiguous float64 (2n, 2m) matrix."""
    a = a.to(torch.complex128)
    ar, ai = a.real, a.imag
    top = torch.cat([ar, -ai], dim=1)
    bottom = torch.cat([ai, ar], dim=1)
    return torch.cat([top, bottom], dim=0).contiguous()


def real_form_tags(tags) -> frozenset:
    """Tags that hold for R(A): Hermitian definiteness becomes symmetric
    definiteness; symmetry (Aᵀ = A), triangularity and diagonality do not
    carry over in the [Re; Im] ordering."""
    out = set()
    if positive_semidefinite_tag in tags:
        out |= {positive_semidefinite_tag, symmetric_tag}
    if negative_semidefinite_tag in tags:
        out |= {negative_semidefinite_tag, symmetric_tag}
    return frozenset(out)


def to_real(x: torch.Tensor) -> torch.Tensor:
    """[Re x; Im x] (float64) of a 1-D complex vector, or of each row of a
    (k, n) block."""
    x = x.to(torch.complex128)
    return torch.cat([x.real, x.imag], dim=-1).contiguous()


def from_real(v: torch.Tensor) -> torch.Tensor:
    """Inverse of to_real."""
    m = v.shape[-1] // 2
    return torch.complex(v[..., :m].contiguous(), v[..., m:].contiguous())


def real_form(operator):
    """The real operator R(operator) on flat float64 vectors of length 2m."""
    from ._operator import (
        FunctionLinearOperator,
        MatrixLinearOperator,
        NegLinearOperator,
        apply_columns,
    )

    if isinstance(operator, MatrixLinearOperator):
        return MatrixLinearOperator(real_form_matrix(operator.matrix),
                                    real_form_tags(operator.tags))
    if isinstance(operator, NegLinearOperator):
        return NegLinearOperator(real_form(operator.operator))
    ins, outs = operator.in_structure(), operator.out_structure()
    m = tree_size(ins)

    def fn(v):
        y = ravel(operator.mv(unravel(from_real(v).to(_leaf_dtype(ins)), ins)), torch.complex128)
        return to_real(y)

    class _RealForm(FunctionLinearOperator):
        def mv_block(self, x):
            xc = from_real(x)
            return to_real(apply_columns(operator, xc.to(_leaf_dtype(ins))))

    return _RealForm(fn, ShapeDtypeStruct((2 * m,), torch.float64), real_form_tags(operator.tags),
                     output_structure=ShapeDtypeStruct((2 * tree_size(outs),), torch.float64))


def _leaf_dtype(structure):
    leaves, _ = tree_flatten(structure)
    out = leaves[0].dtype
    for x in leaves[1:]:
        out = torch.promote_types(out, x.dtype)
    if not is_complex_dtype(out):
        out = torch.complex128
    return out


def complex_vector(vector) -> torch.Tensor:
    """A vector PyTree flattened to one complex128 tensor."""
    return ravel(vector, torch.complex128).contiguous()


def solution_tree(x: torch.Tensor, in_structure):
    """Flat complex solution back into the operator's input structure (leaf
    dtypes promoted to complex where the operator's are real)."""
    leaves, td = tree_flatten(in_structure)
    out, i = [], 0
    for s in leaves:
        n = 1
        for d in s.shape:
            n *= d
        dt = s.dtype if is_complex_dtype(s.dtype) else torch.complex128
        out.append(x[i:i + n].reshape(s.shape).to(dt))
        i += n
    return tree_unflatten(td, out)


def _real_options(options: dict) -> dict:
    """Preconditioner and y0 carried over to the real form."""
    out = dict(options)
    if "preconditioner" in out:
        out["preconditioner"] = real_form(out["preconditioner"])
    if "y0" in out:
        out["y0"] = to_real(complex_vector(out["y0"]))
    return out


def diagonal_solve(operator, vector, well_posed: bool) -> torch.Tensor:
    """x = b / diag(A) elementwise in complex arithmetic; with well_posed
    False, zero diagonal entries give zero (the pseudo-inverse)."""
    d = torch.diagonal(operator.as_matrix()).to(torch.complex128)
    b = complex_vector(vector)
    if well_posed:
        return b / d
    safe = torch.where(d == 0, torch.ones_like(d), d)
    return torch.where(d == 0, torch.zeros_like(b), b / safe)


def triangular_solve(matrix: torch.Tensor, b: torch.Tensor, lower: bool, unit: bool,
                     trans: bool) -> torch.Tensor:
    """op(T) x = b for complex triangular T (op = transpose when trans): the
    diagonal-scaled, interleaved real form on the engine's real triangular
    solve."""
    from . import _dense

    t = matrix.to(torch.complex128)
    if trans:
        t = t.T
        lower = not lower
    n = t.shape[0]
    if not unit:
        d = torch.diagonal(t).clone()
        t = t / d[:, None]
        b = b / d
    e = torch.zeros(2 * n, 2 * n, dtype=torch.float64, device=t.device)
    e[0::2, 0::2] = t.real
    e[0::2, 1::2] = -t.imag
    e[1::2, 0::2] = t.imag
    e[1::2, 1::2] = t.real
    bi = torch.stack([b.real, b.imag], dim=1).reshape(-1).contiguous()
    y = _dense.trsv(e.contiguous(), bi, lower=lower, trans=False, unit=True)
    y = y.reshape(n, 2)
    return torch.complex(y[:, 0].contiguous(), y[:, 1].contiguous())


def linear_solve_complex(operator, vector, solver, options: dict, state, sentinel):
    """(solution tree, result code, stats, state) of a complex solve."""
    from ._solve import AutoLinearSolver, _lookup
    from ._solution import RESULTS
    from ._solver.diagonal import Diagonal
    from ._solver.triangular import Triangular
    from ._operator import has_unit_diagonal, is_diagonal, is_lower_triangular, is_upper_triangular

    concrete = solver
    if isinstance(solver, AutoLinearSolver):
        concrete = _lookup(solver._select_solver(operator))
    if isinstance(concrete, Diagonal):
        if operator.in_size() != operator.out_size() or not is_diagonal(operator):
            raise ValueError("`Diagonal` may only be used for linear solves with diagonal matrices")
        x = diagonal_solve(operator, vector, bool(concrete.well_posed))
        return solution_tree(x, operator.in_structure()), RESULTS.successful, {}, state
    if isinstance(concrete, Triangular):
        lower, upper = is_lower_triangular(operator), is_upper_triangular(operator)
        if operator.in_size() != operator.out_size() or not (lower or upper):
            raise ValueError(
                "`Triangular` may only be used for linear solves with triangular matrices")
        x = triangular_solve(operator.as_matrix(), complex_vector(vector), lower=lower,
                             unit=has_unit_diagonal(operator), trans=False)
        return solution_tree(x, operator.in_structure()), RESULTS.successful, {}, state
    real_op = real_form(operator)
    real_opts = _real_options(options)
    if state is sentinel:
        inner = concrete.init(real_op, real_opts)
    else:
        if not (isinstance(state, tuple) and len(state) == 2 and state[0] == COMPLEX_STATE):
            raise ValueError("`state` does not come from a complex solve of this operator")
        inner = state[1]
    b = to_real(complex_vector(vector))
    x, result, stats = concrete.compute(inner, b, real_opts)
    x = from_real(ravel(x, torch.float64))
    return solution_tree(x, operator.in_structure()), int(result), stats, (COMPLEX_STATE, inner)
