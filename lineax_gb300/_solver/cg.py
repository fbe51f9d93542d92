"""Conjugate gradient (mirrors lineax/_solver/cg.py:48-267) on the device
Krylov engine (lxgb_cg_*)."""

from __future__ import annotations

from typing import Callable

from .. import _krylov
from .._norm import max_norm
from .._operator import (
    conj_not_needed,
    is_negative_semidefinite,
    is_positive_semidefinite,
    linearise,
)
from .._solve import AbstractLinearSolver
from .._structure import structure_equal, unravel
from .misc import preconditioner_and_y0


class CG(AbstractLinearSolver):
    """CG for positive (or negative) definite operators.

    Options: ``preconditioner`` (a positive definite linear operator) and
    ``y0``, as in lineax.  ``norm`` must be ``max_norm`` (the device stopping
    test implements lineax's default norm).

    ``precision="mixed"`` (an extension; Poisson2DOperator with scale 1, no
    preconditioner): FP32 iterations with an FP64 true-residual replacement
    every 16 iterations, stopping on lineax's test applied to that FP64
    residual (`_krylov.cg_poisson_mixed`).  The default "fp64" follows
    lineax's iteration statement for statement.
    """

    def __init__(self, rtol: float, atol: float, norm: Callable = max_norm,
                 stabilise_every: int | None = 10, max_steps: int | None = None,
                 precision: str = "fp64"):
        if precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        self.precision = precision
        if isinstance(rtol, (int, float)) and rtol < 0:
            raise ValueError("Tolerances must be non-negative.")
        if isinstance(atol, (int, float)) and atol < 0:
            raise ValueError("Tolerances must be non-negative.")
        if atol == 0 and rtol == 0 and max_steps is None:
            raise ValueError(
                "Must specify `rtol`, `atol`, or `max_steps` (or some combination of all three)."
            )
        if norm is not max_norm:
            raise NotImplementedError("lineax_gb300 CG implements the default max_norm test")
        self.rtol, self.atol, self.norm = rtol, atol, norm
        self.stabilise_every, self.max_steps = stabilise_every, max_steps

    def __repr__(self):
        return f"CG(rtol={self.rtol}, atol={self.atol}, max_steps={self.max_steps})"

    def init(self, operator, options):
        is_nsd = is_negative_semidefinite(operator)
        if not structure_equal(operator.in_structure(), operator.out_structure()):
            raise ValueError("`CG()` may only be used for linear solves with square matrices.")
        if not (is_positive_semidefinite(operator) or is_nsd):
            raise ValueError(
                "`CG()` may only be used for positive or negative definite linear operators"
            )
        if is_nsd:
            operator = -operator
        return linearise(operator), is_nsd

    def compute(self, state, vector, options):
        operator, is_nsd = state
        preconditioner, y0 = preconditioner_and_y0(operator, vector, options)
        if not is_positive_semidefinite(preconditioner):
            raise ValueError("The preconditioner must be positive definite.")
        b, _ = _krylov.vector_block(vector)
        y0b = None if "y0" not in options else _krylov.vector_block(y0)[0]
        pre = None if "preconditioner" not in options else preconditioner
        if self.precision == "mixed":
            if pre is not None:
                raise ValueError("the mixed-precision CG takes no preconditioner")
            res = _krylov.cg_poisson_mixed(operator, b, rtol=self.rtol, atol=self.atol,
                                           max_steps=self.max_steps, y0=y0b)
        else:
            kw = dict(rtol=self.rtol, atol=self.atol, max_steps=self.max_steps,
                      stabilise_every=self.stabilise_every, preconditioner=pre, y0=y0b)
            # one call with the loop on the device when the operators allow it
            res = _krylov.cg_run(operator, b, **kw) or _krylov.cg_block(operator, b, **kw)
        x = res.y[0]
        if is_nsd:
            x = -x
        sol = unravel(x, operator.in_structure())
        stats = {"num_steps": res.steps[0], "max_steps": self.max_steps}
        return sol, res.results[0], stats

    def transpose(self, state, options):
        opts = {}
        if "preconditioner" in options:
            opts["preconditioner"] = options["preconditioner"].transpose()
        op, is_nsd = state
        return (op.transpose(), is_nsd), opts

    def conj(self, state, options):
        return conj_not_needed(state, options)

    def assume_full_rank(self):
        return True
