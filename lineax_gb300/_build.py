"""Build recipe for liblxgb.so, the C-ABI library of the solve engine.

Compiles every ``csrc/*.cu`` for sm_103a with nvcc (one translation unit per
process, in parallel) and links them into ``lineax_gb300/_lib/liblxgb.so``.
Objects are rebuilt when a source or header is newer than the object.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
BUILD = PKG / "_lib" / "obj"
LIB = LIBDIR / "liblxgb.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC",
    "--expt-relaxed-constexpr",
    "-Xptxas",
    "-v",
]


def nvcc_path() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    return str(pathlib.Path(home) / "bin" / "nvcc")


def _sources() -> list[pathlib.Path]:
    return sorted(CSRC.glob("*.cu"))


def _headers() -> list[pathlib.Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _compile(src: pathlib.Path, obj: pathlib.Path, nvcc: str) -> tuple[str, str]:
    cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{proc.stderr}")
    return src.name, proc.stderr


def build(verbose: bool = False, force: bool = False) -> pathlib.Path:
    """Compile and link liblxgb.so; returns its path."""
    nvcc = nvcc_path()
    BUILD.mkdir(parents=True, exist_ok=True)
    newest_header = max((h.stat().st_mtime for h in _headers()), default=0.0)
    jobs = []
    for src in _sources():
        obj = BUILD / (src.stem + ".o")
        stale = (
            force
            or not obj.exists()
            or obj.stat().st_mtime < max(src.stat().st_mtime, newest_header)
        )
        jobs.append((src, obj, stale))
    logs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_compile, s, o, nvcc) for s, o, stale in jobs if stale]
        for f in futs:
            logs.append(f.result())
    objs = [str(o) for _, o, _ in jobs]
    relink = force or not LIB.exists() or any(
        pathlib.Path(o).stat().st_mtime > LIB.stat().st_mtime for o in objs
    )
    if relink:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc, *ARCH, "-shared", "-cudart", "shared", "-o", str(tmp), *objs]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"link failed:\n{proc.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        for name, err in logs:
            print(f"== {name}\n{err}")
    return LIB


if __name__ == "__main__":
    import sys

    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
