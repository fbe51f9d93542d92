"""Solvers of the GPU engine (the lineax solver types on the hot path)."""

from .cholesky import Cholesky
from .diagonal import Diagonal
from .lu import LU
from .triangular import Triangular

try:  # solvers added as their kernels land
    from .qr import QR
except ImportError:  # pragma: no cover
    QR = None
try:
    from .cg import CG
except ImportError:  # pragma: no cover
    CG = None
try:
    from .gmres import GMRES
except ImportError:  # pragma: no cover
    GMRES = None
try:
    from .bicgstab import BiCGStab
except ImportError:  # pragma: no cover
    BiCGStab = None
from .normal import Normal

__all__ = ["LU", "Cholesky", "QR", "Triangular", "CG", "GMRES", "BiCGStab", "Normal",
           "Diagonal"]
