"""The ragged mixed solve's autotune table: loading, validation, the library
entry that holds it, and (GPU) correctness at every threshold."""

import json

import numpy as np
import pytest
import torch

from lineax_gb300 import _ffi, autotune


def test_table_validation(tmp_path):
    good = tmp_path / "t.json"
    good.write_text(json.dumps({"X sm_103": {"posv_mixed_small_max": 96}}))
    assert autotune.load_table(good)["X sm_103"]["posv_mixed_small_max"] == 96
    bad = tmp_path / "b.json"
    bad.write_text(json.dumps({"X sm_103": {"posv_mixed_small_max": 500}}))
    with pytest.raises(ValueError):
        autotune.load_table(bad)
    assert autotune.load_table(tmp_path / "missing.json") == {}


def test_committed_table_is_valid():
    table = autotune.load_table()
    for entry in table.values():
        assert 0 <= entry["posv_mixed_small_max"] <= autotune.DEFAULT_SMALL_MAX


def test_library_threshold_and_workspace(lib_built):
    lib = _ffi.load()
    before = lib.lxgb_posv_mixed_small_max()
    try:
        assert _ffi.call("lxgb_posv_mixed_set_small_max", 144) == 0
        ws144 = lib.lxgb_posv_ragged_mixed_workspace_size(100, 128, 4)
        assert _ffi.call("lxgb_posv_mixed_set_small_max", 64) == 0
        assert lib.lxgb_posv_mixed_small_max() == 64
        ws64 = lib.lxgb_posv_ragged_mixed_workspace_size(100, 128, 4)
        assert ws64 > ws144  # order-128 systems now need factor slices
        with pytest.raises(_ffi.LxgbError):
            _ffi.call("lxgb_posv_mixed_set_small_max", 145)
    finally:
        _ffi.call("lxgb_posv_mixed_set_small_max", before)


@pytest.mark.gpu
@pytest.mark.parametrize("small_max", [0, 64, 96, 144])
def test_mixed_solve_correct_at_every_threshold(dev, small_max):
    from lineax_gb300 import batched
    from oracle import dense

    rng = np.random.default_rng(small_max + 5)
    ns = [16, 40, 64, 65, 100, 144, 145, 300]
    mats, rhs = [], []
    for n in ns:
        g = rng.standard_normal((n, n))
        mats.append(torch.tensor(g @ g.T / n + 1e-2 * np.eye(n)))
        rhs.append(torch.tensor(rng.standard_normal((3, n))))
    lib = _ffi.load()
    before = lib.lxgb_posv_mixed_small_max()
    try:
        autotune.ensure_applied(dev)
        _ffi.call("lxgb_posv_mixed_set_small_max", small_max)
        rb = batched.RaggedBatch.from_lists(mats, rhs, device=dev)
        res = batched.spd_solve_ragged_mixed(rb, tol=1e-12)
        torch.cuda.synchronize()
        assert int(res.info.abs().sum()) == 0
        for s in range(len(ns)):
            xs = rb.system_b(res.x, s).cpu().numpy()
            for k in range(3):
                assert dense.backward_error(mats[s].numpy(), xs[k], rhs[s][k].numpy()) <= 1e-12
    finally:
        _ffi.call("lxgb_posv_mixed_set_small_max", before)


def test_choose_small_max_rule():
    b = (48, 64, 80)
    fast = {"shared_ms": 1.0, "slice_ms": 2.0}
    slow = {"shared_ms": 2.0, "slice_ms": 1.0}
    assert autotune.choose_small_max({48: fast, 64: fast, 80: fast}, b) == \
        autotune.DEFAULT_SMALL_MAX
    assert autotune.choose_small_max({48: fast, 64: slow, 80: fast}, b) == 48
    assert autotune.choose_small_max({48: slow, 64: fast, 80: fast}, b) == autotune.FLOOR
    # ties keep shared memory
    tie = {"shared_ms": 1.0, "slice_ms": 1.0}
    assert autotune.choose_small_max({48: tie, 64: fast, 80: slow}, b) == 64


def test_committed_gb300_entry_matches_its_measurements():
    table = autotune.load_table()
    for entry in table.values():
        timings = {int(n): v for n, v in entry["measured"].items()}
        buckets = tuple(sorted(timings))
        assert autotune.choose_small_max(timings, buckets) == entry["posv_mixed_small_max"]
