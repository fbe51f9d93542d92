"""Result codes and the Solution record (mirrors lineax/_solution.py:52-88).

The integer value of each RESULTS member equals its index in lineax's
eqxi.Enumeration and the matching lxgb_status code of the C ABI, so a status
returned by a kernel is a RESULTS value as is.
"""

from __future__ import annotations

import dataclasses
from typing import Any

_singular_msg = (
    "A linear solver returned non-finite (NaN or inf) output. This usually means that an "
    "operator was not well-posed, and that its solver does not support this."
)
_nonfinite_msg = (
    "A linear solver received non-finite (NaN or inf) input and cannot determine a "
    "solution."
)


class _ResultsMeta(type):
    def __getitem__(cls, value) -> str:
        return cls._messages[int(value)]

    def __iter__(cls):
        return iter(cls._names)


class RESULTS(metaclass=_ResultsMeta):
    """Integer result codes of a linear solve; ``RESULTS[code]`` is its message."""

    successful = 0
    max_steps_reached = 1
    singular = 2
    breakdown = 3
    stagnation = 4
    conlim = 5
    nonfinite_input = 6

    _names = (
        "successful",
        "max_steps_reached",
        "singular",
        "breakdown",
        "stagnation",
        "conlim",
        "nonfinite_input",
    )
    _messages = (
        "",
        "The maximum number of solver steps was reached. Try increasing `max_steps`.",
        _singular_msg,
        "A form of iterative breakdown has occured in a linear solve. Try using a different "
        "solver for this problem or increase `restart` if using GMRES.",
        "A stagnation in an iterative linear solve has occurred. Try increasing "
        "`stagnation_iters` or `restart`.",
        "Condition number of A seems to be larger than `conlim`.",
        _nonfinite_msg,
    )

    @classmethod
    def name(cls, value) -> str:
        return cls._names[int(value)]


class LinearSolveError(RuntimeError):
    """Raised by ``linear_solve(..., throw=True)`` on an unsuccessful result
    (the counterpart of lineax's ``result.error_if``, lineax/_solve.py:124-128)."""

    def __init__(self, result: int):
        super().__init__(RESULTS[result])
        self.result = int(result)


@dataclasses.dataclass
class Solution:
    """The solution to a linear solve.

    - `value`: the solution.
    - `result`: an integer RESULTS code.
    - `stats`: solver statistics (e.g. number of steps).
    - `state`: the solver state used (reusable through ``linear_solve(..., state=)``).
    """

    value: Any
    result: int
    stats: dict
    state: Any
