"""Derivatives of linear_solve for torch autograd (reverse mode) and forward
mode (torch.autograd.forward_ad), restating lineax's rules
(lineax/_solve.py:151-317) for x = A⁺ b, A⁺ the pseudo-inverse:

  JVP   x' = A⁺(-A'x + A⁺ᵀA'ᵀ(b - Ax) - Ay + b') + y,   y = A'ᵀA⁺ᵀx,
        where the A⁺ᵀA'ᵀ(b - Ax) term is dropped when the solver assumes full
        rank and A has independent rows (rows <= columns), and the y terms when
        it assumes full rank and A has independent columns (columns <= rows);
  VJP   for a cotangent g of x, with z = A⁺ᵀ g (the transpose solve of
        lineax/_solve.py:271-317):
          ḃ = z,
          Ā = -z xᵀ + (b - Ax)(A⁺z)ᵀ + (A⁺ᵀx)(g - A⁺Ag)ᵀ,
        the same terms dropped under the same conditions (the last two are the
        adjoints of the least-squares and minimum-norm terms of the JVP).
Every solve in these formulas reuses the primal factorisation: A⁺ v through
the solver's state, A⁺ᵀ v through solver.transpose(state).

Gradients reach the vector always, the matrix of a MatrixLinearOperator
(all terms), and tensors that the function of another operator closes over
through the -A'x term: x is returned as x* + S(b - A x*), where S applies A⁺
in its derivative and is zero in value (A⁺(b - A x*) = 0 for the
pseudo-inverse solution x*), so autograd differentiates A x* through the
operator's own torch function.  That is exact for nonsingular operators; the
rank-deficient terms above are applied for matrices only.
"""

from __future__ import annotations

import torch

from ._structure import ravel, unravel


class SolveContext:
    """Primal solve state shared by the derivative rules."""

    def __init__(self, operator, solver, state, options):
        self.operator, self.solver, self.state, self.options = operator, solver, state, options
        self._t = None

    def solve(self, v: torch.Tensor) -> torch.Tensor:
        """A⁺ v (v flat, in the operator's output space)."""
        out = self.operator.out_structure()
        x, _, _ = self.solver.compute(self.state, unravel(v.detach(), out), self.options)
        return ravel(x, torch.float64)

    def solve_t(self, v: torch.Tensor) -> torch.Tensor:
        """A⁺ᵀ v (v flat, in the operator's input space)."""
        if self._t is None:
            self._t = self.solver.transpose(self.state, self.options)
        st, opts = self._t
        x, _, _ = self.solver.compute(st, unravel(v.detach(), self.operator.in_structure()), opts)
        return ravel(x, torch.float64)

    def independent(self):
        rows, cols = self.operator.out_size(), self.operator.in_size()
        full = bool(self.solver.assume_full_rank())
        return full and rows <= cols, full and cols <= rows


class _MatrixSolve(torch.autograd.Function):
    """x = A⁺ b for a dense A (m×n) and b (m), with every term of the rules."""

    @staticmethod
    def forward(matrix, b, ctx_obj, x_star):
        return x_star.clone()

    @staticmethod
    def setup_context(ctx, inputs, output):
        matrix, b, ctx_obj, _ = inputs
        ctx.obj = ctx_obj
        ctx.save_for_backward(matrix, b, output)
        ctx.save_for_forward(matrix, b, output)

    @staticmethod
    def backward(ctx, g):
        matrix, b, x = ctx.saved_tensors
        obj = ctx.obj
        a = matrix.detach().to(torch.float64)
        g = g.detach().to(torch.float64)
        z = obj.solve_t(g)
        grad_a = None
        if ctx.needs_input_grad[0]:
            rows_ind, cols_ind = obj.independent()
            grad_a = -torch.outer(z, x)
            if not rows_ind:
                r = b.detach().to(torch.float64) - a @ x
                grad_a = grad_a + torch.outer(r, obj.solve(z))
            if not cols_ind:
                h = g - obj.solve(a @ g)
                grad_a = grad_a + torch.outer(obj.solve_t(x), h)
            grad_a = grad_a.to(matrix.dtype)
        grad_b = z.to(b.dtype) if ctx.needs_input_grad[1] else None
        return grad_a, grad_b, None, None

    @staticmethod
    def jvp(ctx, ta, tb, _obj, _x):
        matrix, b, x = ctx.saved_tensors
        obj = ctx.obj
        a = matrix.detach().to(torch.float64)
        x = x.detach().to(torch.float64)
        # the output-space vector that A⁺ maps (lineax/_solve.py:201-250)
        rhs = torch.zeros(b.numel(), dtype=torch.float64, device=x.device) if tb is None \
            else tb.to(torch.float64)
        y = None
        if ta is not None:
            ta = ta.to(torch.float64)
            rows_ind, cols_ind = obj.independent()
            rhs = rhs - ta @ x                                   # -A'x
            if not rows_ind:                                     # A⁺ᵀA'ᵀ(b - Ax)
                resid = b.detach().to(torch.float64) - a @ x
                rhs = rhs + obj.solve_t(ta.T @ resid)
            if not cols_ind:                                     # y = A'ᵀA⁺ᵀx, then -Ay
                y = ta.T @ obj.solve_t(x)
                rhs = rhs - a @ y
        t = obj.solve(rhs)
        if y is not None:
            t = t + y
        return t.to(matrix.dtype)


class _ZeroSolve(torch.autograd.Function):
    """S(v): zero in value, A⁺ v in its derivatives."""

    @staticmethod
    def forward(v, ctx_obj, n):
        return v.new_zeros(n)

    @staticmethod
    def setup_context(ctx, inputs, output):
        ctx.obj = inputs[1]

    @staticmethod
    def backward(ctx, g):
        return ctx.obj.solve_t(g.detach().to(torch.float64)), None, None

    @staticmethod
    def jvp(ctx, tv, _obj, _n):
        return ctx.obj.solve(tv.to(torch.float64))


def needs_grad(operator, vector) -> bool:
    """Whether derivatives must be attached: grad mode (or a forward-AD dual)
    and a vector, matrix or closed-over tensor that requires them."""
    from ._structure import tree_flatten

    leaves, _ = tree_flatten(vector)
    ts = [x for x in leaves if isinstance(x, torch.Tensor)]
    if any(_is_dual(x) for x in ts) or _operator_dual(operator):
        return True
    if not torch.is_grad_enabled():
        return False
    return any(x.requires_grad for x in ts) or _operator_requires_grad(operator)


def _tensors_of_function(fn):
    """Tensors a Python function closes over (closure cells, partial
    arguments, module parameters), where it is plain to see."""
    import functools

    out = []
    if isinstance(fn, functools.partial):
        out += [a for a in list(fn.args) + list(fn.keywords.values())
                if isinstance(a, torch.Tensor)]
        fn = fn.func
    if isinstance(fn, torch.nn.Module):
        out += list(fn.parameters())
    for cell in getattr(fn, "__closure__", None) or ():
        try:
            v = cell.cell_contents
        except ValueError:
            continue
        if isinstance(v, torch.Tensor):
            out.append(v)
        elif isinstance(v, torch.nn.Module):
            out += list(v.parameters())
    return out


def _operator_tensors(operator):
    from ._operator import (
        ComposedLinearOperator,
        FunctionLinearOperator,
        MatrixLinearOperator,
        NegLinearOperator,
        TaggedLinearOperator,
    )

    if isinstance(operator, MatrixLinearOperator):
        return [operator.matrix]
    if isinstance(operator, (NegLinearOperator, TaggedLinearOperator)):
        return _operator_tensors(operator.operator)
    if isinstance(operator, ComposedLinearOperator):
        return _operator_tensors(operator.outer) + _operator_tensors(operator.inner)
    if isinstance(operator, FunctionLinearOperator):
        return _tensors_of_function(operator.fn)
    return []


def _operator_requires_grad(operator) -> bool:
    return any(t.requires_grad for t in _operator_tensors(operator))


def _operator_dual(operator) -> bool:
    return any(_is_dual(t) for t in _operator_tensors(operator))


def _is_dual(x) -> bool:
    try:
        from torch.autograd import forward_ad

        return forward_ad.unpack_dual(x).tangent is not None
    except Exception:  # noqa: BLE001 - outside a forward-AD level
        return False


def differentiable(operator, vector, x_star, ctx_obj: SolveContext):
    """The solution tree with derivative rules attached."""
    from ._operator import MatrixLinearOperator

    ins = operator.in_structure()
    b = ravel(vector, torch.float64)
    xs = ravel(x_star, torch.float64).detach()
    if isinstance(operator, MatrixLinearOperator) and operator.matrix.ndim == 2:
        x = _MatrixSolve.apply(operator.matrix, b, ctx_obj, xs)
        return unravel(x, ins)
    # other operators: x* + S(b - A x*), the operator differentiated by torch
    ax = ravel(operator.mv(unravel(xs, ins)), torch.float64)
    x = xs + _ZeroSolve.apply(b - ax, ctx_obj, xs.numel())
    return unravel(x, ins)
