"""Shape/dtype structures and PyTree flattening over torch tensors.

lineax describes operator inputs and outputs with PyTrees of
``jax.ShapeDtypeStruct`` and packs vectors with ravel/unravel helpers
(lineax/_solver/misc.py:70-114).  This module provides the same for nested
tuples / lists / dicts of torch tensors, leaves in the order jax.tree_util
uses (dict keys sorted).
"""

from __future__ import annotations

import dataclasses
import math
from typing import Any

import torch


@dataclasses.dataclass(frozen=True)
class ShapeDtypeStruct:
    """The shape and dtype of one array (a stand-in for jax.ShapeDtypeStruct)."""

    shape: tuple
    dtype: torch.dtype

    @property
    def size(self) -> int:
        return math.prod(self.shape)


def _is_leaf(x) -> bool:
    return isinstance(x, (torch.Tensor, ShapeDtypeStruct)) or not isinstance(
        x, (tuple, list, dict)
    )


def tree_flatten(tree) -> tuple[list, Any]:
    """Leaves in jax.tree_util order and a treedef to rebuild the tree."""
    if _is_leaf(tree):
        return [tree], None
    if isinstance(tree, dict):
        keys = sorted(tree)
        leaves, defs = [], []
        for k in keys:
            lv, d = tree_flatten(tree[k])
            leaves += lv
            defs.append((len(lv), d))
        return leaves, ("dict", keys, defs)
    leaves, defs = [], []
    for item in tree:
        lv, d = tree_flatten(item)
        leaves += lv
        defs.append((len(lv), d))
    return leaves, (type(tree).__name__, None, defs)


def tree_unflatten(treedef, leaves):
    leaves = list(leaves)
    if treedef is None:
        assert len(leaves) == 1
        return leaves[0]
    kind, keys, defs = treedef
    out, i = [], 0
    for count, d in defs:
        out.append(tree_unflatten(d, leaves[i : i + count]))
        i += count
    if kind == "dict":
        return dict(zip(keys, out))
    if kind == "tuple":
        return tuple(out)
    return list(out)


def structure_of(tree):
    """The ShapeDtypeStruct PyTree of a PyTree of tensors."""
    leaves, td = tree_flatten(tree)
    return tree_unflatten(
        td,
        [
            x if isinstance(x, ShapeDtypeStruct) else ShapeDtypeStruct(tuple(x.shape), x.dtype)
            for x in leaves
        ],
    )


def structure_equal(a, b) -> bool:
    la, ta = tree_flatten(structure_of(a))
    lb, tb = tree_flatten(structure_of(b))
    return ta == tb and la == lb


def tree_size(tree) -> int:
    return sum(math.prod(x.shape) for x in tree_flatten(tree)[0])


def result_dtype(dtypes) -> torch.dtype:
    out = None
    for d in dtypes:
        out = d if out is None else torch.promote_types(out, d)
    return out


def ravel(tree, dtype=None) -> torch.Tensor:
    """Concatenate the leaves of a vector PyTree into one 1-D tensor in leaf
    order, promoted to a common dtype (lineax/_solver/misc.py:79-90)."""
    leaves, _ = tree_flatten(tree)
    if dtype is None:
        dtype = result_dtype([x.dtype for x in leaves])
    if len(leaves) == 1:
        return leaves[0].reshape(-1).to(dtype)
    return torch.cat([x.reshape(-1).to(dtype) for x in leaves])


def unravel(flat: torch.Tensor, structure):
    """Split a 1-D tensor back into the leaves of `structure`
    (lineax/_solver/misc.py:93-105)."""
    leaves, td = tree_flatten(structure)
    out, i = [], 0
    for s in leaves:
        n = math.prod(s.shape)
        out.append(flat[i : i + n].reshape(s.shape).to(s.dtype))
        i += n
    return tree_unflatten(td, out)
