"""lineax_gb300 — a GB300 (sm_103a) solve engine behind lineax's solver API.

The public names mirror lineax/__init__.py for the hot path: ``linear_solve``
with the ``LU``, ``Cholesky``, ``QR``, ``Triangular``, ``CG``, ``GMRES`` and
``BiCGStab`` solvers and the ``Normal`` wrapper over ``MatrixLinearOperator`` / ``FunctionLinearOperator``, the tags,
``RESULTS`` and ``Solution``.  Vectors and matrices are CUDA torch tensors; all
arithmetic runs in the hand-written kernels of liblxgb.so (C ABI in
include/lxgb.h).  There is no CPU fallback: without the built library or a GPU
the solvers raise.
"""

from ._norm import max_norm, rms_norm, sum_squares, tree_dot, two_norm
from ._operator import (
    AbstractLinearOperator,
    ComposedLinearOperator,
    FunctionLinearOperator,
    IdentityLinearOperator,
    MatrixLinearOperator,
    Poisson2DOperator,
    TaggedLinearOperator,
    has_unit_diagonal,
    is_diagonal,
    is_lower_triangular,
    is_negative_semidefinite,
    is_positive_semidefinite,
    is_symmetric,
    is_tridiagonal,
    is_upper_triangular,
    linearise,
    materialise,
)
from ._solution import RESULTS, LinearSolveError, Solution
from ._solve import AbstractLinearSolver, AutoLinearSolver, invert, linear_solve
from ._solver import CG, GMRES, LU, QR, BiCGStab, Cholesky, Diagonal, Normal, Triangular
from ._structure import ShapeDtypeStruct
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

__version__ = "0.1.0"
