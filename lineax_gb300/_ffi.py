"""ctypes binding of liblxgb.so (the C ABI declared in include/lxgb.h).

This is the Python side of the drop-in boundary: every solver in this package
reaches the GPU only through the functions bound here.  The library is loaded
lazily on first use; if it is missing, or no CUDA device is visible, the call
raises — there is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import pathlib
import threading

_LIB_PATH = pathlib.Path(__file__).resolve().parent / "_lib" / "liblxgb.so"
_lock = threading.Lock()
_lib: ctypes.CDLL | None = None

c_i32 = ctypes.c_int32
c_i64 = ctypes.c_int64
c_f64 = ctypes.c_double
c_p = ctypes.c_void_p

# name -> (restype, argtypes); mirrors include/lxgb.h one to one.
SIGNATURES: dict[str, tuple[object, list[object]]] = {
    "lxgb_version": (ctypes.c_int, []),
    "lxgb_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "lxgb_last_error": (ctypes.c_char_p, []),
    "lxgb_getrf_batched_f64": (ctypes.c_int, [c_i64, c_i32, c_p, c_i64, c_p, c_i64, c_p, c_p]),
    "lxgb_getrs_batched_f64": (
        ctypes.c_int,
        [c_i64, c_i32, c_i32, c_p, c_i64, c_p, c_i64, c_p, c_i64, c_i32, c_p],
    ),
    "lxgb_potrf_ragged_f64": (ctypes.c_int, [c_i64, c_i32, c_p, c_p, c_p, c_p, c_p]),
    "lxgb_potrf_f64": (ctypes.c_int, [c_i64, c_p, c_i64, c_p, c_p]),
    "lxgb_syrk_f64": (ctypes.c_int, [c_i32, c_i64, c_i64, c_p, c_i64, c_i32, c_p, c_i64, c_i32,
                                     c_p]),
    "lxgb_potrs_ragged_f64": (ctypes.c_int, [c_i64, c_i32, c_p, c_p, c_p, c_p, c_p, c_p, c_p]),
    "lxgb_posv_ragged_mixed_workspace_size": (c_i64, [c_i64, c_i32, c_i32]),
    "lxgb_posv_ragged_mixed": (
        ctypes.c_int,
        [c_i64, c_i32, c_i32, c_p, c_p, c_p, c_p, c_p, c_p, c_p, c_f64, c_i32, c_p, c_p, c_p,
         c_p, c_i64, c_p],
    ),
    "lxgb_posv_ragged_mixed_factors": (
        ctypes.c_int,
        [c_i64, c_i32, c_i32, c_p, c_p, c_p, c_p, c_p, c_p, c_p, c_f64, c_i32, c_p, c_p, c_p,
         c_p, c_p, c_p, c_i64, c_p],
    ),
    "lxgb_geqrf_f32_tc_q_workspace_size": (c_i64, [c_i64, c_i64]),
    "lxgb_geqrf_f32_tc_q": (ctypes.c_int, [c_i64, c_i64, c_p, c_p, c_p, c_p, c_p, c_p, c_p, c_i64,
                                           c_p]),
    "lxgb_qr32_apply_workspace_size": (c_i64, [c_i32, c_i32]),
    "lxgb_qr32_apply": (ctypes.c_int, [c_i32, c_i32, c_p, c_p, c_i32, c_p, c_p, c_p, c_i64, c_p]),
    "lxgb_cg_run_workspace_size": (c_i64, [c_i32, c_i64, c_i32]),
    "lxgb_cg_run": (ctypes.c_int, [c_i32, c_i64, c_p, c_p, c_p, c_p, c_i32, c_f64, c_f64, c_i64,
                                   c_i32, c_p, c_p, c_p, c_i64, c_p]),
    "lxgb_gmres_run_workspace_size": (c_i64, [c_i32, c_i64, c_i32]),
    "lxgb_gmres_run": (ctypes.c_int, [c_i32, c_i64, c_p, c_p, c_p, c_p, c_i32, c_f64, c_f64,
                                      c_i64, c_i32, c_i32, c_p, c_p, c_p, c_i64, c_p]),
    "lxgb_gmres_ir_run_workspace_size": (c_i64, [c_i32, c_i64, c_i32]),
    "lxgb_gmres_ir_run": (ctypes.c_int, [c_i32, c_i64, c_p, c_p, c_p, c_p, c_p, c_f64, c_f64,
                                         c_i32, c_i32, c_i32, c_i32, c_i32, c_p, c_p, c_p, c_i64,
                                         c_p]),
    "lxgb_gemm_bf16_nt": (ctypes.c_int, [c_i32, c_i32, c_i32, c_p, c_i64, c_p, c_i64, c_p, c_i64,
                                         ctypes.c_float, ctypes.c_float, c_p, c_p]),
    "lxgb_posv_ragged_mixed_noalloc": (
        ctypes.c_int,
        [c_i64, c_i32, c_i32, c_p, c_p, c_p, c_p, c_p, c_p, c_p, c_f64, c_i32, c_p, c_p, c_p,
         c_p],
    ),
    "lxgb_posv_mixed_set_small_max": (ctypes.c_int, [c_i32]),
    "lxgb_posv_mixed_small_max": (c_i32, []),
    "lxgb_posv_mixed_set_tensor_cores": (ctypes.c_int, [c_i32]),
    "lxgb_gemm_set_persistent": (ctypes.c_int, [c_i32]),
    "lxgb_getrf_set_pair": (ctypes.c_int, [c_i32]),
    "lxgb_geqrf_t_elems": (c_i64, [c_i64]),
    "lxgb_geqrf_workspace_size": (c_i64, [c_i64, c_i64]),
    "lxgb_geqrf_f64": (ctypes.c_int, [c_i64, c_i64, c_p, c_i32, c_p, c_p, c_p, c_p, c_i64, c_p]),
    "lxgb_ormqr_workspace_size": (c_i64, [c_i64, c_i32]),
    "lxgb_ormqr_f64": (
        ctypes.c_int, [c_i64, c_i64, c_p, c_p, c_p, c_i32, c_p, c_i32, c_p, c_i64, c_p]),
    "lxgb_cg_workspace_size": (c_i64, [c_i32, c_i64]),
    "lxgb_cg_start": (ctypes.c_int, [c_i32, c_i64, c_p, c_p, c_p, c_i64, c_i32, c_p, c_i64, c_p]),
    "lxgb_cg_step_alpha": (
        ctypes.c_int,
        [c_i32, c_i64, c_p, c_p, c_p, c_p, c_i32, c_i32, c_f64, c_f64, c_f64, c_p, c_i64, c_p]),
    "lxgb_cg_true_residual": (
        ctypes.c_int, [c_i32, c_i64, c_p, c_p, c_p, c_i32, c_p, c_i64, c_p]),
    "lxgb_cg_step_beta": (
        ctypes.c_int,
        [c_i32, c_i64, c_p, c_p, c_p, c_p, c_i32, c_i64, c_i32, c_f64, c_f64, c_p, c_i64, c_p]),
    "lxgb_cg_status": (ctypes.c_int, [c_i32, c_i64, c_i32, c_p, c_p, c_p, c_i64, c_p]),
    "lxgb_bicgstab_workspace_size": (c_i64, [c_i32, c_i64]),
    "lxgb_bicgstab_start": (ctypes.c_int, [c_i32, c_i64, c_p, c_p, c_p, c_p, c_i64, c_i32, c_p,
                                           c_i64, c_p]),
    "lxgb_bicgstab_direction": (ctypes.c_int, [c_i32, c_i64, c_p, c_p, c_p, c_p, c_p, c_i64,
                                               c_p]),
    "lxgb_bicgstab_s": (ctypes.c_int, [c_i32, c_i64, c_p, c_p, c_p, c_p, c_p, c_i64, c_p]),
    "lxgb_bicgstab_update": (ctypes.c_int, [c_i32, c_i64, c_p, c_p, c_p, c_p, c_p, c_p, c_p,
                                            c_f64, c_f64, c_i64, c_i32, c_p, c_i64, c_p]),
    "lxgb_bicgstab_status": (ctypes.c_int, [c_i32, c_i64, c_p, c_p, c_p, c_p, c_p, c_i64, c_p]),
    "lxgb_gmres_workspace_size": (c_i64, [c_i32, c_i64, c_i32]),
    "lxgb_gmres_basis_offset": (c_i64, [c_i32, c_i64, c_i32, c_i32]),
    "lxgb_gmres_init": (ctypes.c_int, [c_i32, c_i64, c_i32, c_p, c_i64, c_p]),
    "lxgb_gmres_cycle_begin": (ctypes.c_int, [c_i32, c_i64, c_i32, c_i32, c_p, c_p, c_i64, c_p]),
    "lxgb_gmres_arnoldi": (
        ctypes.c_int, [c_i32, c_i64, c_i32, c_i32, c_i32, c_p, c_p, c_p, c_i64, c_p]),
    "lxgb_gmres_cycle_end": (
        ctypes.c_int, [c_i32, c_i64, c_i32, c_i32, c_i32, c_p, c_p, c_p, c_i64, c_p]),
    "lxgb_gmres_outer": (
        ctypes.c_int,
        [c_i32, c_i64, c_i32, c_i32, c_i32, c_p, c_p, c_p, c_p, c_p, c_f64, c_f64, c_i64, c_i32,
         c_i32, c_p, c_i64, c_p]),
    "lxgb_gmres_status": (ctypes.c_int, [c_i32, c_i64, c_i32, c_i32, c_p, c_p, c_i64, c_p]),
    "lxgb_kreduce_workspace_size": (c_i64, [c_i32, c_i64]),
    "lxgb_kreduce_f64": (
        ctypes.c_int, [c_i32, c_i32, c_i64, c_p, c_i64, c_p, c_i64, c_p, c_p, c_i64, c_p]),
    "lxgb_poisson5_f64": (ctypes.c_int, [c_i64, c_i64, c_i32, c_f64, c_p, c_p, c_p]),
    "lxgb_gemm_tf32_nt": (
        ctypes.c_int,
        [c_i32, c_i32, c_i32, c_p, c_i64, c_p, c_i64, c_p, c_i64, ctypes.c_float, ctypes.c_float,
         c_p, c_p]),
    "lxgb_getrf_f32_tc_workspace_size": (c_i64, [c_i32, c_i32]),
    "lxgb_getrf_f32_tc": (ctypes.c_int, [c_i32, c_p, c_p, c_p, c_p, c_i32, c_p, c_p, c_i64, c_p]),
    "lxgb_gemm_3xtf32_nt": (
        ctypes.c_int,
        [c_i32, c_i32, c_i32, c_p, c_p, c_i64, c_p, c_p, c_i64, c_p, c_i64, ctypes.c_float,
         ctypes.c_float, c_p, c_p]),
    "lxgb_getrs_f32": (ctypes.c_int, [c_i32, c_i32, c_p, c_p, c_p, c_p, c_p]),
    "lxgb_geqrf_f32_tc_workspace_size": (c_i64, [c_i64, c_i64]),
    "lxgb_geqrf_f32_tc": (ctypes.c_int, [c_i64, c_i64, c_p, c_p, c_p, c_p, c_p, c_p, c_i64, c_p]),
    "lxgb_cg32_workspace_size": (c_i64, [c_i32]),
    "lxgb_cg32_init": (ctypes.c_int, [c_i32, c_i64, c_i64, c_i64, c_p, c_i64, c_p]),
    "lxgb_cg32_refresh": (ctypes.c_int, [c_i32, c_i64, c_i64, c_p, c_p, c_p, c_p, ctypes.c_double,
                                         ctypes.c_double, c_i64, c_p, c_i64, c_p]),
    "lxgb_cg32_start_direction": (ctypes.c_int, [c_i32, c_i64, c_p, c_p, c_p]),
    "lxgb_cg32_iterate": (ctypes.c_int, [c_i32, c_i64, c_i64, c_i32, c_p, c_p, c_p, c_p, c_p,
                                         c_i64, c_p]),
    "lxgb_cg32_status": (ctypes.c_int, [c_i32, c_p, c_p, c_i64, c_p]),
    "lxgb_lu32_inverse_workspace_size": (c_i64, [c_i32, c_i32]),
    "lxgb_potrf_f32_tc_workspace_size": (c_i64, [c_i64]),
    "lxgb_potrf_f32_tc": (ctypes.c_int, [c_i64, c_p, c_p, c_p, c_p, c_p, c_i64, c_p]),
    "lxgb_chol32_to_lu32": (ctypes.c_int, [c_i64, c_p, c_p, c_p, c_p]),
    "lxgb_chol32_uinv": (ctypes.c_int, [c_i64, c_p, c_p, c_p, c_p]),
    "lxgb_lu32_inverse": (ctypes.c_int, [c_i32, c_p, c_p, c_p, c_p, c_p, c_i32, c_p, c_p, c_i64,
                                         c_p]),
    "lxgb_lu32_apply_workspace_size": (c_i64, [c_i32, c_i32]),
    "lxgb_lu32_apply": (ctypes.c_int, [c_i32, c_i32, c_p, c_p, c_p, c_i32, c_p, c_p, c_p, c_i64,
                                       c_p]),
    "lxgb_split_f64": (ctypes.c_int, [c_i64, c_i64, c_p, c_i64, c_p, c_p, c_i64, c_p]),
    "lxgb_gemv_df_workspace_size": (c_i64, [c_i32, c_i32]),
    "lxgb_gemv_df": (ctypes.c_int, [c_i32, c_i32, c_p, c_p, c_i64, c_i32, c_p, c_i64, c_p, c_p,
                                    c_i64, c_i32, c_p, c_i64, c_p]),
    "lxgb_trsm_f64": (ctypes.c_int, [c_i32, c_i32, c_p, c_i64, c_i32, c_i32, c_i32, c_p, c_p]),
    "lxgb_gemv_f64": (
        ctypes.c_int,
        [c_i64, c_i64, c_p, c_i64, c_i32, c_i32, c_p, c_i64, c_p, c_i64, c_f64, c_f64, c_p],
    ),
    "lxgb_nonfinite_f64": (ctypes.c_int, [c_i64, c_p, c_p, c_p]),
    "lxgb_reduce_workspace_size": (c_i64, [c_i64]),
    "lxgb_reduce_f64": (ctypes.c_int, [c_i32, c_i64, c_p, c_p, c_p, c_p, c_i64, c_p]),
    "lxgb_rows_scale_f64": (ctypes.c_int, [c_i32, c_i64, c_p, c_i32, c_p, c_p]),
    "lxgb_rows_axpy_f64": (ctypes.c_int, [c_i32, c_i64, c_p, c_p, c_p, c_p]),
    "lxgb_norm_inf_workspace_size": (c_i64, [c_i64]),
    "lxgb_norm_inf_f64": (ctypes.c_int, [c_i64, c_i64, c_p, c_i64, c_p, c_p, c_i64, c_p]),
    "lxgb_diag_solve_f64": (ctypes.c_int, [c_i64, c_p, c_i64, c_p, c_p, c_i32, c_p]),
}


class LxgbError(RuntimeError):
    """A library call failed with an argument or CUDA error (status >= 100)."""

    def __init__(self, name: str, status: int, text: str):
        super().__init__(f"{name} failed with status {status}: {text}")
        self.status = status


class LinearOperatorDesc(ctypes.Structure):
    """struct lxgb_linear_operator (include/lxgb.h)."""

    _fields_ = [("kind", c_i32), ("reserved", c_i32), ("n", c_i64), ("a", c_p),
                ("lda", c_i64), ("nx", c_i64), ("ny", c_i64), ("scale", c_f64),
                ("hi", c_p), ("lo", c_p), ("perm", c_p)]


OP_DENSE, OP_POISSON5, OP_SPLIT_DF, OP_LU32_INV, OP_QR32 = 0, 1, 2, 3, 4


def lib_path() -> pathlib.Path:
    return _LIB_PATH


def load() -> ctypes.CDLL:
    """Load liblxgb.so and declare its signatures (raises if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not _LIB_PATH.exists():
            raise ImportError(
                f"{_LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; "
                "g.build()\"` (the solve engine has no CPU fallback)"
            )
        # torch first, so the process shares one CUDA runtime with it.
        import torch  # noqa: F401

        lib = ctypes.CDLL(str(_LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def call(name: str, *args) -> int:
    """Call an entry point; statuses 0..6 are returned, >= 100 raise."""
    lib = load()
    status = getattr(lib, name)(*args)
    if status >= 100:
        text = (lib.lxgb_last_error() or b"").decode()
        raise LxgbError(name, status, text)
    return status


def ptr(t) -> int:
    """Device pointer of a torch tensor (0 for None)."""
    return 0 if t is None else t.data_ptr()


def stream_handle(device=None) -> int:
    import torch

    return torch.cuda.current_stream(device).cuda_stream
