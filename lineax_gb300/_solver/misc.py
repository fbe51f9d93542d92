"""Vector packing and option parsing shared by the solvers
(mirrors lineax/_solver/misc.py:30-114)."""

from __future__ import annotations

import torch

from .._operator import AbstractLinearOperator, IdentityLinearOperator, linearise
from .._structure import ravel, structure_equal, structure_of, tree_flatten, unravel


def preconditioner_and_y0(operator: AbstractLinearOperator, vector, options: dict):
    """Read options["preconditioner"] and options["y0"] (misc.py:30-60)."""
    structure = operator.in_structure()
    if "preconditioner" in options:
        preconditioner = linearise(options["preconditioner"])
        if not isinstance(preconditioner, AbstractLinearOperator):
            raise ValueError("The preconditioner must be a linear operator.")
        if not structure_equal(preconditioner.in_structure(), structure):
            raise ValueError(
                "The preconditioner must have `in_structure` that matches the "
                "operator's `in_strucure`."
            )
        if not structure_equal(preconditioner.out_structure(), structure):
            raise ValueError(
                "The preconditioner must have `out_structure` that matches the "
                "operator's `in_structure`."
            )
    else:
        preconditioner = IdentityLinearOperator(structure)
    if "y0" in options:
        y0 = options["y0"]
        if not structure_equal(structure_of(y0), structure_of(vector)):
            raise ValueError("`y0` must have the same structure, shape, and dtype as `vector`")
    else:
        leaves, td = tree_flatten(vector)
        from .._structure import tree_unflatten

        y0 = tree_unflatten(td, [torch.zeros_like(x) for x in leaves])
    return preconditioner, y0


def pack_structures(operator: AbstractLinearOperator):
    """(out_structure, in_structure) of the operator (misc.py:70-76)."""
    return (operator.out_structure(), operator.in_structure())


def transpose_packed_structures(packed):
    out_s, in_s = packed
    return (in_s, out_s)


def ravel_vector(vector, packed, dtype=torch.float64) -> torch.Tensor:
    """Flatten a vector PyTree matching the out-structure (misc.py:79-90)."""
    out_s, _ = packed
    if not structure_equal(structure_of(vector), out_s):
        raise ValueError("pytree does not match out_structure")
    return ravel(vector, dtype).contiguous()


def unravel_solution(solution: torch.Tensor, packed):
    """Split a flat solution into the in-structure (misc.py:93-105)."""
    _, in_s = packed
    return unravel(solution, in_s)
