"""CPU: the C-ABI library builds, loads, and exports every declared symbol;
host-side argument validation (no device work is launched)."""

import pathlib
import re

import pytest

HEADER = pathlib.Path(__file__).resolve().parent.parent / "include" / "lxgb.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(lxgb_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(lib_built):
    from lineax_gb300 import _ffi

    lib = _ffi.load()
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_ffi_signatures_cover_header():
    from lineax_gb300 import _ffi

    assert set(declared_symbols()) <= set(_ffi.SIGNATURES), (
        set(declared_symbols()) - set(_ffi.SIGNATURES))


def test_status_strings(lib_built):
    from lineax_gb300 import _ffi

    lib = _ffi.load()
    assert lib.lxgb_status_string(0) == b"successful"
    assert lib.lxgb_status_string(6) == b"nonfinite_input"
    assert lib.lxgb_version() >= 100


def test_invalid_arguments_rejected_on_host(lib_built):
    """Argument checks run before any launch, so they work without a GPU."""
    from lineax_gb300 import _ffi

    with pytest.raises(_ffi.LxgbError) as e:
        _ffi.call("lxgb_getrf_batched_f64", 1, -3, 0, 0, 0, 0, 0, 0)
    assert e.value.status == 100
    with pytest.raises(_ffi.LxgbError):
        _ffi.call("lxgb_getrs_batched_f64", 1, 4, 1, 1, 16, 1, 4, 1, 4, 7, 0)
    with pytest.raises(_ffi.LxgbError):
        _ffi.call("lxgb_reduce_f64", 9, 10, 1, 1, 1, 1, 8, 0)


def test_empty_problems_are_no_ops(lib_built):
    from lineax_gb300 import _ffi

    assert _ffi.call("lxgb_getrf_batched_f64", 0, 5, 0, 25, 0, 5, 0, 0) == 0
    assert _ffi.call("lxgb_trsm_f64", 0, 3, 0, 0, 1, 0, 0, 0, 0) == 0
    assert _ffi.call("lxgb_posv_ragged_mixed", 0, 16, 1, 0, 0, 0, 0, 0, 0, 0, 1e-12, 10, 0, 0, 0,
                     0, 0, 0) == 0
    assert _ffi.call("lxgb_syrk_f64", 0, 0, 5, 0, 5, 0, 0, 0, 0, 0) == 0


def test_mixed_workspace_size_grows_with_n(lib_built):
    from lineax_gb300 import _ffi

    lib = _ffi.load()
    small = lib.lxgb_posv_ragged_mixed_workspace_size(100, 200, 8)
    large = lib.lxgb_posv_ragged_mixed_workspace_size(100, 512, 8)
    assert small >= 256 and large > small
