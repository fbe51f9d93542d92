"""Linear operators over torch tensors (mirrors the in-scope part of
lineax/_operator.py: MatrixLinearOperator :232-285, FunctionLinearOperator
:664-732, IdentityLinearOperator, negation, the tag predicates :1587-1929,
linearise :1206-1257 and materialise :1263-1388).

Matrix-vector products of MatrixLinearOperator run on the engine's own GEMV
kernel (lxgb_gemv_f64); FunctionLinearOperator calls the user's function.
"""

from __future__ import annotations

import abc
from typing import Callable

import torch

from . import _blas
from ._structure import ShapeDtypeStruct, ravel, structure_of, tree_flatten, tree_size, unravel
from ._tags import (
    diagonal_tag,
    lower_triangular_tag,
    negative_semidefinite_tag,
    positive_semidefinite_tag,
    symmetric_tag,
    transpose_tags,
    tridiagonal_tag,
    unit_diagonal_tag,
    upper_triangular_tag,
)


def _frozenset(tags) -> frozenset:
    if isinstance(tags, frozenset):
        return tags
    if isinstance(tags, (list, tuple, set)):
        return frozenset(tags)
    return frozenset([tags])


class AbstractLinearOperator(abc.ABC):
    """Abstract linear operator: `mv`, `as_matrix`, `transpose`, structures."""

    tags: frozenset = frozenset()

    @abc.abstractmethod
    def mv(self, vector):
        ...

    @abc.abstractmethod
    def as_matrix(self) -> torch.Tensor:
        ...

    @abc.abstractmethod
    def transpose(self) -> "AbstractLinearOperator":
        ...

    @abc.abstractmethod
    def in_structure(self):
        ...

    @abc.abstractmethod
    def out_structure(self):
        ...

    @property
    def T(self) -> "AbstractLinearOperator":
        return self.transpose()

    def in_size(self) -> int:
        return tree_size(self.in_structure())

    def out_size(self) -> int:
        return tree_size(self.out_structure())

    def __neg__(self) -> "AbstractLinearOperator":
        return NegLinearOperator(self)

    def __matmul__(self, other: "AbstractLinearOperator") -> "AbstractLinearOperator":
        return ComposedLinearOperator(self, other)


class MatrixLinearOperator(AbstractLinearOperator):
    """Wraps a 2-D tensor (lineax/_operator.py:232-285).  Vectors are 1-D."""

    def __init__(self, matrix: torch.Tensor, tags=()):
        if not isinstance(matrix, torch.Tensor) or matrix.ndim != 2:
            raise ValueError("`MatrixLinearOperator(matrix=...)` should be 2-dimensional.")
        if not torch.is_floating_point(matrix) and not matrix.is_complex():
            matrix = matrix.to(torch.get_default_dtype())
        self.matrix = matrix
        self.tags = _frozenset(tags)
        self._real = None   # real form of a complex matrix, built on first use

    def mv(self, vector):
        if self.matrix.is_complex() or (isinstance(vector, torch.Tensor) and vector.is_complex()):
            # complex product through the real form R(A) [Re x; Im x]
            from . import _complex

            if self._real is None:
                self._real = _complex.real_form_matrix(self.matrix)
            y = _blas.gemv(self._real, _complex.to_real(vector))
            return _complex.from_real(y)
        return _blas.gemv(self.matrix, vector)

    def as_matrix(self):
        return self.matrix

    def transpose(self):
        if symmetric_tag in self.tags:
            return self
        return MatrixLinearOperator(self.matrix.T.contiguous(), transpose_tags(self.tags))

    def in_structure(self):
        return ShapeDtypeStruct((self.matrix.shape[1],), self.matrix.dtype)

    def out_structure(self):
        return ShapeDtypeStruct((self.matrix.shape[0],), self.matrix.dtype)


class FunctionLinearOperator(AbstractLinearOperator):
    """Wraps a linear function of a PyTree of tensors
    (lineax/_operator.py:664-732).  `input_structure` is a PyTree of
    ShapeDtypeStruct (or of example tensors)."""

    def __init__(self, fn: Callable, input_structure, tags=(), output_structure=None):
        self.fn = fn
        self._in = structure_of(input_structure)
        self._out = structure_of(output_structure) if output_structure is not None else None
        self.tags = _frozenset(tags)

    def mv(self, vector):
        return self.fn(vector)

    def as_matrix(self):
        return materialise(self).matrix

    def transpose(self):
        if is_symmetric(self):
            return self
        return materialise(self).transpose()

    def in_structure(self):
        return self._in

    def out_structure(self):
        if self._out is None:
            return self._in
        return self._out


class IdentityLinearOperator(AbstractLinearOperator):
    """The identity on a structure (used as the default preconditioner)."""

    tags = frozenset(
        [symmetric_tag, diagonal_tag, unit_diagonal_tag, positive_semidefinite_tag]
    )

    def __init__(self, structure):
        self._s = structure_of(structure)

    def mv(self, vector):
        return vector

    def as_matrix(self):
        leaves, _ = tree_flatten(self._s)
        n = tree_size(self._s)
        return torch.eye(n, dtype=leaves[0].dtype, device="cuda")

    def transpose(self):
        return self

    def in_structure(self):
        return self._s

    def out_structure(self):
        return self._s


class NegLinearOperator(AbstractLinearOperator):
    """-operator (used by Cholesky/CG for negative-definite operators)."""

    def __init__(self, operator: AbstractLinearOperator):
        self.operator = operator
        t = operator.tags
        swapped = set(t)
        if positive_semidefinite_tag in t:
            swapped.discard(positive_semidefinite_tag)
            swapped.add(negative_semidefinite_tag)
        elif negative_semidefinite_tag in t:
            swapped.discard(negative_semidefinite_tag)
            swapped.add(positive_semidefinite_tag)
        swapped.discard(unit_diagonal_tag)
        self.tags = frozenset(swapped)

    def mv(self, vector):
        out = self.operator.mv(vector)
        leaves, td = tree_flatten(out)
        from ._structure import tree_unflatten

        return tree_unflatten(td, [-x for x in leaves])

    def as_matrix(self):
        return -self.operator.as_matrix()

    def transpose(self):
        return NegLinearOperator(self.operator.transpose())

    def in_structure(self):
        return self.operator.in_structure()

    def out_structure(self):
        return self.operator.out_structure()


class ComposedLinearOperator(AbstractLinearOperator):
    """outer @ inner: x -> outer.mv(inner.mv(x)) (lineax/_operator.py's
    ComposedLinearOperator).  `mv_block` applies both factors to a (k, n)
    block, so Krylov solvers iterate on the composition block-wise."""

    def __init__(self, outer: AbstractLinearOperator, inner: AbstractLinearOperator, tags=()):
        self.outer, self.inner = outer, inner
        self.tags = _frozenset(tags)

    def mv(self, vector):
        return self.outer.mv(self.inner.mv(vector))

    def mv_block(self, x):
        from ._krylov import block_mv

        return block_mv(self.outer, block_mv(self.inner, x))

    def as_matrix(self):
        return materialise(self).matrix

    def transpose(self):
        return ComposedLinearOperator(self.inner.transpose(), self.outer.transpose(),
                                      transpose_tags(self.tags))

    def in_structure(self):
        return self.inner.in_structure()

    def out_structure(self):
        return self.outer.out_structure()


class TaggedLinearOperator(AbstractLinearOperator):
    """An operator with extra tags (lineax/_operator.py's TaggedLinearOperator)."""

    def __init__(self, operator: AbstractLinearOperator, tags):
        self.operator = operator
        self.tags = _frozenset(tags) | frozenset(operator.tags)

    def mv(self, vector):
        return self.operator.mv(vector)

    def mv_block(self, x):
        from ._krylov import block_mv

        return block_mv(self.operator, x)

    def as_matrix(self):
        return self.operator.as_matrix()

    def transpose(self):
        return TaggedLinearOperator(self.operator.transpose(), transpose_tags(self.tags))

    def in_structure(self):
        return self.operator.in_structure()

    def out_structure(self):
        return self.operator.out_structure()


# -- tag predicates (lineax/_operator.py:1587-1929) -------------------------


def is_symmetric(op) -> bool:
    """Aᵀ = A: tagged symmetric or diagonal, or (real dtypes only) positive or
    negative semidefinite — for complex operators those tags mean Hermitian
    (lineax/_operator.py:1617-1631)."""
    t = op.tags
    if symmetric_tag in t or diagonal_tag in t:
        return True
    if positive_semidefinite_tag in t or negative_semidefinite_tag in t:
        from ._complex import operator_is_complex

        return not operator_is_complex(op)
    return False


def is_diagonal(op) -> bool:
    return diagonal_tag in op.tags or (op.in_size() == 1 and op.out_size() == 1)


def is_tridiagonal(op) -> bool:
    return tridiagonal_tag in op.tags or diagonal_tag in op.tags


def is_lower_triangular(op) -> bool:
    return lower_triangular_tag in op.tags


def is_upper_triangular(op) -> bool:
    return upper_triangular_tag in op.tags


def is_positive_semidefinite(op) -> bool:
    return positive_semidefinite_tag in op.tags


def is_negative_semidefinite(op) -> bool:
    return negative_semidefinite_tag in op.tags


def has_unit_diagonal(op) -> bool:
    return unit_diagonal_tag in op.tags


def linearise(op):
    """Matrix and function operators are already linear (lineax/_operator.py:1206)."""
    return op


def apply_columns(op, x: torch.Tensor) -> torch.Tensor:
    """op applied to every row of the (k, n) block x, as one batched call: a
    GEMM for matrices, the operator's own block product when it has one (the
    Poisson stencil, compositions, tagged and negated operators), and
    torch.vmap of the function for FunctionLinearOperator (the counterpart of
    the jax.vmap in lineax/_operator.py:1369-1388).  A function that torch.vmap
    cannot batch (one that calls out of torch) is applied row by row."""
    if isinstance(op, MatrixLinearOperator):
        if op.matrix.is_complex() or x.is_complex():
            return op.mv(x)
        return _blas.gemv(op.matrix, x)
    if isinstance(op, IdentityLinearOperator):
        return x
    if isinstance(op, NegLinearOperator):
        return -apply_columns(op.operator, x)
    if isinstance(op, ComposedLinearOperator):
        return apply_columns(op.outer, apply_columns(op.inner, x))
    if isinstance(op, TaggedLinearOperator):
        return apply_columns(op.operator, x)
    if hasattr(op, "mv_block"):
        return op.mv_block(x)
    ins, outs = op.in_structure(), op.out_structure()
    out_dtype = tree_flatten(outs)[0][0].dtype

    def one(row):
        return ravel(op.mv(unravel(row, ins)), out_dtype)

    try:
        return torch.vmap(one)(x).contiguous()
    except Exception:  # noqa: BLE001 - functions outside torch's batching rules
        return torch.stack([one(x[c]) for c in range(x.shape[0])]).contiguous()


def materialise(op) -> MatrixLinearOperator:
    """Turn an operator into a MatrixLinearOperator by applying it to the
    columns of the identity in one batched call (lineax/_operator.py:1369-1388)."""
    if isinstance(op, MatrixLinearOperator):
        return op
    ins = op.in_structure()
    leaves, _ = tree_flatten(ins)
    dtype = leaves[0].dtype
    n = tree_size(ins)
    eye = torch.eye(n, dtype=dtype, device="cuda")
    rows = apply_columns(op, eye)            # row j = op(e_j)
    return MatrixLinearOperator(rows.T.contiguous(), op.tags)


def conj_not_needed(state, options):
    """conj of a solver state over real operators is the state itself (complex
    operators are solved through real forms, whose states are real)."""
    return state, options


class Poisson2DOperator(FunctionLinearOperator):
    """The 5-point negative Laplacian on an nx×ny interior grid with zero
    Dirichlet boundary (times `scale`), matrix-free on lxgb_poisson5_f64: the
    FunctionLinearOperator of the CG benchmark configuration.  Positive
    definite and symmetric.  Vectors are flattened grids (length nx·ny)."""

    def __init__(self, nx: int, ny: int, scale: float = 1.0, dtype=torch.float64):
        self.nx, self.ny, self.scale = int(nx), int(ny), float(scale)
        super().__init__(self._apply, ShapeDtypeStruct((self.nx * self.ny,), dtype),
                         (symmetric_tag, positive_semidefinite_tag))

    def _apply(self, x):
        return self.mv_block(x.reshape(1, -1)).reshape(x.shape)

    def mv_block(self, x):
        from . import _ffi
        from ._blas import as_device_f64

        xb = as_device_f64(x)
        k = xb.shape[0]
        out = torch.empty_like(xb)
        _ffi.call("lxgb_poisson5_f64", self.nx, self.ny, k, self.scale, _ffi.ptr(xb),
                  _ffi.ptr(out), _ffi.stream_handle(xb.device))
        return out

    def transpose(self):
        return self

    def as_matrix(self):
        return materialise(self).matrix
