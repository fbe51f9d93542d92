"""BiCGStab (mirrors lineax/_solver/bicgstab.py:35-220) on the device Krylov
engine (lxgb_bicgstab_*)."""

from __future__ import annotations

from typing import Callable

from .. import _krylov
from .._norm import max_norm
from .._operator import conj_not_needed, linearise
from .._solve import AbstractLinearSolver
from .._structure import structure_equal, unravel
from .misc import preconditioner_and_y0


class BiCGStab(AbstractLinearSolver):
    """Biconjugate gradient stabilised method for square operators.

    Options: ``preconditioner`` (right preconditioning, a linear operator of
    the operator's structure) and ``y0``, as in lineax.  ``norm`` must be
    ``max_norm`` (the device stopping test implements lineax's default norm).
    Arithmetic is FP64, so breakdown is tested as omega, alpha or rho == 0
    (lineax's ``jax_enable_x64`` branch).
    """

    def __init__(self, rtol: float, atol: float, norm: Callable = max_norm,
                 max_steps: int | None = None):
        if isinstance(rtol, (int, float)) and rtol < 0:
            raise ValueError("Tolerances must be non-negative.")
        if isinstance(atol, (int, float)) and atol < 0:
            raise ValueError("Tolerances must be non-negative.")
        if atol == 0 and rtol == 0 and max_steps is None:
            raise ValueError(
                "Must specify `rtol`, `atol`, or `max_steps` (or some combination of all three)."
            )
        if norm is not max_norm:
            raise NotImplementedError("lineax_gb300 BiCGStab implements the default max_norm test")
        self.rtol, self.atol, self.norm, self.max_steps = rtol, atol, norm, max_steps

    def __repr__(self):
        return f"BiCGStab(rtol={self.rtol}, atol={self.atol}, max_steps={self.max_steps})"

    def init(self, operator, options):
        if not structure_equal(operator.in_structure(), operator.out_structure()):
            raise ValueError(
                "`BiCGstab(..., normal=False)` may only be used for linear solves with "
                "square matrices."
            )
        return linearise(operator)

    def compute(self, state, vector, options):
        operator = state
        preconditioner, y0 = preconditioner_and_y0(operator, vector, options)
        b, _ = _krylov.vector_block(vector)
        y0b = None if "y0" not in options else _krylov.vector_block(y0)[0]
        pre = None if "preconditioner" not in options else preconditioner
        res = _krylov.bicgstab_block(operator, b, rtol=self.rtol, atol=self.atol,
                                     max_steps=self.max_steps, preconditioner=pre, y0=y0b)
        sol = unravel(res.y[0], operator.in_structure())
        stats = {"num_steps": res.steps[0], "max_steps": self.max_steps}
        return sol, res.results[0], stats

    def transpose(self, state, options):
        opts = {}
        if "preconditioner" in options:
            opts["preconditioner"] = options["preconditioner"].transpose()
        return state.transpose(), opts

    def conj(self, state, options):
        return conj_not_needed(state, options)

    def assume_full_rank(self):
        return True
