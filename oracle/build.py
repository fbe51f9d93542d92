"""Build recipe for the C part of the oracle (test infrastructure only).

Compiles oracle/getf2.c into oracle/_build/liboracle.so with gcc.  -ffp-contract=off
keeps the compiler from fusing the multiply-adds that the C source spells out,
so only the explicit fma() calls are fused — the arithmetic the GPU LU
reproduces.
"""

from __future__ import annotations

import pathlib
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
OUT = HERE / "_build" / "liboracle.so"
SOURCES = [HERE / "getf2.c"]


def build(force: bool = False) -> pathlib.Path:
    OUT.parent.mkdir(parents=True, exist_ok=True)
    if (not force and OUT.exists()
            and OUT.stat().st_mtime > max(s.stat().st_mtime for s in SOURCES)):
        return OUT
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-o", str(OUT),
           *map(str, SOURCES), "-lm"]
    subprocess.run(cmd, check=True)
    return OUT


def load():
    import ctypes

    lib = ctypes.CDLL(str(build()))
    lib.oracle_getf2_batched_f64.restype = None
    lib.oracle_getf2_batched_f64.argtypes = [
        ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return lib


def getf2_batched(a):
    """Bit-exact CPU twin of the GPU FP64 LU: a is (batch, n, n) float64."""
    import numpy as np

    a = np.array(a, dtype=np.float64, order="C", copy=True)
    if a.ndim == 2:
        a = a[None]
    batch, n, _ = a.shape
    piv = np.zeros((batch, n), np.int32)
    info = np.zeros(batch, np.int32)
    load().oracle_getf2_batched_f64(batch, n, a.ctypes.data, piv.ctypes.data, info.ctypes.data)
    return a, piv, info


if __name__ == "__main__":
    print(build(force=True))
