"""Solvers of the GPU engine (the lineax solver types on the hot path)."""

from .bicgstab import BiCGStab
from .cg import CG
from .cholesky import Cholesky
from .diagonal import Diagonal
from .gmres import GMRES
from .lu import LU
from .normal import Normal
from .qr import QR
from .triangular import Triangular

__all__ = ["LU", "Cholesky", "QR", "Triangular", "CG", "GMRES", "BiCGStab", "Normal",
           "Diagonal"]
