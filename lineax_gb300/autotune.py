"""Autotune table of the ragged mixed-precision SPD solve.

The persistent kernel factors a system in shared memory when its order is at
most `small_max`, otherwise in a per-CTA workspace slice through L2; which is
faster around the crossover depends on the GPU model.  `tune()` measures it per
size bucket: for each candidate order n it times uniform batches of order-n
systems through both paths and returns the largest n up to which the shared-
memory path is not slower.  The result is kept in `autotune_table.json`
(committed, one entry per GPU model) and applied once per process, before the
first mixed solve, through lxgb_posv_mixed_set_small_max — the library holds
that one value as its immutable tuning table.

Run ``python -m lineax_gb300.autotune --write`` on a new GPU model to add its
entry.
"""

from __future__ import annotations

import json
import pathlib
import threading

TABLE = pathlib.Path(__file__).resolve().with_name("autotune_table.json")
BUCKETS = (48, 64, 80, 96, 112, 128, 144)
DEFAULT_SMALL_MAX = 144
FLOOR = 32   # orders up to this always use shared memory (not timed)
_lock = threading.Lock()
_applied: set = set()


def device_key(device=None) -> str:
    import torch

    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else \
        torch.device(device)
    name = torch.cuda.get_device_name(dev)
    major, minor = torch.cuda.get_device_capability(dev)
    return f"{name} sm_{major}{minor}"


def load_table(path: pathlib.Path = TABLE) -> dict:
    if not path.exists():
        return {}
    table = json.loads(path.read_text())
    for key, entry in table.items():
        v = entry.get("posv_mixed_small_max")
        if not isinstance(v, int) or not 0 <= v <= DEFAULT_SMALL_MAX:
            raise ValueError(f"autotune table entry {key!r}: bad posv_mixed_small_max {v!r}")
    return table


def apply(device=None, path: pathlib.Path = TABLE) -> int:
    """Set the library's tuning from the table entry of this GPU model (the
    default when there is none); returns the value in effect."""
    from . import _ffi

    entry = load_table(path).get(device_key(device))
    value = DEFAULT_SMALL_MAX if entry is None else entry["posv_mixed_small_max"]
    _ffi.call("lxgb_posv_mixed_set_small_max", value)
    return value


def ensure_applied(device=None) -> None:
    """apply() once per process (before the first mixed solve)."""
    if "done" in _applied:
        return
    with _lock:
        if "done" not in _applied:
            apply(device)
            _applied.add("done")


def _time_bucket(n: int, small_max: int, dev, systems: int, reps: int) -> float:
    import torch

    from . import _ffi, batched

    g = torch.Generator(device=dev).manual_seed(1000 + n)
    gm = torch.randn(systems, n, n, dtype=torch.float64, device=dev, generator=g)
    a = gm @ gm.transpose(1, 2) / n + 1e-2 * torch.eye(n, dtype=torch.float64, device=dev)
    b = torch.randn(systems, 4, n, dtype=torch.float64, device=dev, generator=g)
    rb = batched.RaggedBatch.from_packed(a.reshape(-1), b.reshape(-1), [n] * systems,
                                         [4] * systems, dev)
    _ffi.call("lxgb_posv_mixed_set_small_max", small_max)
    ws = batched.MixedWorkspace(rb.batch, rb.max_n, rb.max_nrhs, dev)
    for _ in range(2):
        batched.spd_solve_ragged_mixed(rb, 1e-12, 10, ws)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        batched.spd_solve_ragged_mixed(rb, 1e-12, 10, ws)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def choose_small_max(timings: dict, buckets=BUCKETS) -> int:
    """The largest bucket up to which (contiguously from FLOOR) the shared-
    memory path is not slower; DEFAULT_SMALL_MAX when that is every bucket."""
    small_max = FLOOR
    for i, n in enumerate(buckets):
        t = timings[n]
        if t["shared_ms"] <= t["slice_ms"] and small_max == (buckets[i - 1] if i else FLOOR):
            small_max = n
    if small_max == buckets[-1]:
        small_max = DEFAULT_SMALL_MAX
    return small_max


def tune(device=None, buckets=BUCKETS, systems: int = 608, reps: int = 5) -> dict:
    """Time the shared-memory and the slice path on uniform batches of each
    bucket's order; small_max = the largest bucket up to which the shared-
    memory path is never slower."""
    import torch

    from . import _ffi

    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else \
        torch.device(device)
    before = int(_ffi.load().lxgb_posv_mixed_small_max())
    timings = {}
    try:
        for n in buckets:
            t_smem = _time_bucket(n, DEFAULT_SMALL_MAX, dev, systems, reps)
            t_slice = _time_bucket(n, n - 1, dev, systems, reps)
            timings[n] = {"shared_ms": t_smem, "slice_ms": t_slice}
    finally:
        _ffi.call("lxgb_posv_mixed_set_small_max", before)
    small_max = choose_small_max(timings, buckets)
    return {"posv_mixed_small_max": small_max,
            "measured": {str(n): v for n, v in timings.items()},
            "systems_per_bucket": systems, "nrhs": 4}


def save(entry: dict, device=None, path: pathlib.Path = TABLE) -> None:
    table = load_table(path)
    table[device_key(device)] = entry
    path.write_text(json.dumps(table, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    import argparse

    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("--write", action="store_true", help="store the entry in the table")
    p.add_argument("--out", default=str(TABLE), help="table file to write")
    args = p.parse_args()
    entry = tune()
    print(json.dumps({device_key(): entry}, indent=1))
    if args.write:
        save(entry, path=pathlib.Path(args.out))
