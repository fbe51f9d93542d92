"""Restarted GMRES (mirrors lineax/_solver/gmres.py:37-447) on the device
Krylov engine (lxgb_gmres_*)."""

from __future__ import annotations

from typing import Callable

from .. import _krylov
from .._norm import max_norm
from .._operator import conj_not_needed, linearise
from .._solve import AbstractLinearSolver
from .._structure import structure_equal, unravel
from .misc import preconditioner_and_y0


class GMRES(AbstractLinearSolver):
    """GMRES(restart) with single-pass classical Gram-Schmidt, a QR least-squares
    solve of the Hessenberg system, stagnation and deferred-breakdown checks.

    Options: ``preconditioner`` (left) and ``y0``.  ``restart`` <= 128.
    """

    def __init__(self, rtol: float, atol: float, norm: Callable = max_norm,
                 max_steps: int | None = None, restart: int = 20, stagnation_iters: int = 20):
        if isinstance(rtol, (int, float)) and rtol < 0:
            raise ValueError("Tolerances must be non-negative.")
        if isinstance(atol, (int, float)) and atol < 0:
            raise ValueError("Tolerances must be non-negative.")
        if atol == 0 and rtol == 0 and max_steps is None:
            raise ValueError(
                "Must specify `rtol`, `atol`, or `max_steps` (or some combination of all three)."
            )
        if norm is not max_norm:
            raise NotImplementedError("lineax_gb300 GMRES implements the default max_norm test")
        self.rtol, self.atol, self.norm = rtol, atol, norm
        self.max_steps, self.restart, self.stagnation_iters = max_steps, restart, stagnation_iters

    def __repr__(self):
        return f"GMRES(rtol={self.rtol}, atol={self.atol}, restart={self.restart})"

    def init(self, operator, options):
        if not structure_equal(operator.in_structure(), operator.out_structure()):
            raise ValueError(
                "`GMRES(..., normal=False)` may only be used for linear solves with square "
                "matrices."
            )
        return linearise(operator)

    def compute(self, state, vector, options):
        operator = state
        preconditioner, y0 = preconditioner_and_y0(operator, vector, options)
        b, _ = _krylov.vector_block(vector)
        y0b = None if "y0" not in options else _krylov.vector_block(y0)[0]
        pre = None if "preconditioner" not in options else preconditioner
        kw = dict(rtol=self.rtol, atol=self.atol, max_steps=self.max_steps,
                  restart=self.restart, stagnation_iters=self.stagnation_iters,
                  preconditioner=pre, y0=y0b)
        # one call with the loop on the device when the operators allow it
        res = _krylov.gmres_run(operator, b, **kw) or _krylov.gmres_block(operator, b, **kw)
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
