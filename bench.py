"""Benchmark of the solve engine on the ragged batched Cholesky workload.

Workload (one "step"): 4096 SPD systems, n log-uniform in [16, 512],
A = G Gᵀ/n + 1e-2·I, 1..8 right-hand sides each, solved to a normwise backward
error <= 1e-12 by the mixed-precision path (FP32 factor, FP64 refinement) in
one persistent launch.  Metric: solves/s (systems with all their right-hand
sides solved per second), with per-step p50/p99 latency and, beside it, the
plain FP64 GPU path (FP64 potrf + potrs) on the same inputs.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference's CPU path on the host cores: lineax's
Cholesky solve lowers to LAPACK potrf/potrs (lineax/_solver/cholesky.py:60,74),
which JAX's CPU backend takes from SciPy, so SciPy's FP64 cho_factor/cho_solve
run in a spawn-started process pool over a sample of the same workload.
Under torchrun every rank solves its own 4096 systems (weak scaling, no
collective on the data path).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

TOL = 1e-12
COUNT = 4096
SEED = 0
METRIC = "solves/s and p50/p99 latency at <=1e-12 backward error vs plain FP64 GPU"
UNIT = "solves/s"
WORKLOAD = "ragged_spd_cholesky_4096"


# ---------------------------------------------------------------------------
# CPU side (reference arm and cpu_baseline): SciPy LAPACK in worker processes
# ---------------------------------------------------------------------------
_W = {}


def _cpu_worker_init(seed, picks):
    import numpy as np

    from lineax_gb300 import workloads

    n, k = workloads.ragged_spd_sizes(seed, COUNT)
    _W["systems"] = [workloads.spd_system(seed, s, n[s], k[s]) for s in picks]
    _W["np"] = np


def _cpu_worker_solve(_):
    import scipy.linalg as sl

    worst = 0.0
    for a, b in _W["systems"]:
        c = sl.cho_factor(a, lower=False, check_finite=False)
        x = sl.cho_solve(c, b.T, check_finite=False)
        worst = max(worst, float(abs(x[0, 0])))
    return len(_W["systems"]), worst


def _cpu_pool(seed, sample, cores):
    """A spawn pool whose workers hold disjoint parts of `sample`."""
    import multiprocessing as mp

    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    ctx = mp.get_context("spawn")
    parts = [sample[i::cores] for i in range(cores)]
    pools = [ctx.Pool(1, initializer=_cpu_worker_init, initargs=(seed, p)) for p in parts]
    return pools


def _cpu_step(pools):
    rs = [p.apply_async(_cpu_worker_solve, (0,)) for p in pools]
    return sum(r.get()[0] for r in rs)


def cpu_sample(seed, size):
    import numpy as np

    rng = np.random.default_rng([seed, 77])
    return sorted(rng.choice(COUNT, size=size, replace=False).tolist())


def run_cpu_baseline(seed, size=1024, min_seconds=10.0, cores=None):
    """Solve a random sample of the workload repeatedly for >= min_seconds."""
    cores = cores or len(os.sched_getaffinity(0))
    pools = _cpu_pool(seed, cpu_sample(seed, size), cores)
    try:
        _cpu_step(pools)  # warm-up (imports, first-touch)
        done, t0 = 0, time.perf_counter()
        while True:
            done += _cpu_step(pools)
            el = time.perf_counter() - t0
            if el >= min_seconds:
                break
    finally:
        for p in pools:
            p.terminate()
    return {
        "value": done / el,
        "unit": UNIT,
        "cores": cores,
        "kind": "port",
        "sample": f"{size} systems drawn uniformly from the {COUNT}-system workload, "
                  f"solved repeatedly for {el:.1f} s with SciPy LAPACK FP64 "
                  "cho_factor(lower=False)+cho_solve, one process per core",
    }


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = len(os.sched_getaffinity(0))
    size = 1024
    pools = _cpu_pool(SEED, cpu_sample(SEED, size), cores)
    times = []
    try:
        for _ in range(args.warmup):
            _cpu_step(pools)
        for _ in range(args.steps):
            t0 = time.perf_counter()
            _cpu_step(pools)
            times.append(time.perf_counter() - t0)
    finally:
        for p in pools:
            p.terminate()
    total = sum(times)
    value = size * len(times) / total
    lat = sorted(t * 1e3 for t in times)
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded numpy PCG64)",
        "config": {"workload": WORKLOAD, "systems": COUNT, "n": "log-uniform [16,512]",
                   "nrhs": "1..8", "tol": TOL, "step": f"{size}-system sample"},
        "latency_ms": {"p50": _pct(lat, 50), "p99": _pct(lat, 99)},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{size} of {COUNT} systems per step, SciPy LAPACK FP64 "
                                   "potrf/potrs (the routines lineax's Cholesky reaches on "
                                   "JAX-CPU), one process per core"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------
def _pct(sorted_vals, p):
    if not sorted_vals:
        return None
    i = min(len(sorted_vals) - 1, max(0, int(round(p / 100 * (len(sorted_vals) - 1)))))
    return sorted_vals[i]


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        rows = []
        for line in (self.out or "").strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, flags in rows for i, f in enumerate(flags)
                          if f.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows),
                "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows)}


def max_over_ranks(values, world, device):
    """Element-wise maximum of per-rank timings over all ranks (one all-reduce;
    the identity for a single process).  The whole-job rate of a step is the
    units of every rank over the slowest rank's time."""
    vals = [float(v) for v in values]
    if world <= 1:
        return vals
    import torch
    import torch.distributed as dist

    t = torch.tensor(vals, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu().tolist()]


def _bind_near_gpu(index):
    """Restrict this process to the host CPUs attached to GPU `index` (sysfs
    local_cpulist of its PCI function), when that leaves at least one allowed
    CPU, so that pinned host buffers are first touched on the GPU's own
    memory node.  Returns the CPUs used, or None when nothing was changed."""
    try:
        bus = subprocess.run(["nvidia-smi", f"--id={index}", "--query-gpu=pci.bus_id",
                              "--format=csv,noheader"], capture_output=True, text=True,
                             timeout=30).stdout.strip().splitlines()[0].strip()
        dom, rest = bus.split(":", 1)
        path = f"/sys/bus/pci/devices/{int(dom, 16):04x}:{rest.lower()}/local_cpulist"
        with open(path) as f:
            spec = f.read().strip()
        cpus = set()
        for part in spec.split(","):
            lo, _, hi = part.partition("-")
            cpus.update(range(int(lo), int(hi or lo) + 1))
        allowed = os.sched_getaffinity(0)
        near = cpus & allowed
        if not near or near == allowed:
            return None
        os.sched_setaffinity(0, near)
        return sorted(near)
    except Exception:  # noqa: BLE001 - best effort (no nvidia-smi, no sysfs entry)
        return None


def run_gpu(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    from lineax_gb300 import batched, workloads

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    def barrier():
        if world > 1:
            dist.barrier()

    # cpu baseline first (spawned workers, rank 0 only, every allowed core)
    cpu = run_cpu_baseline(SEED) if (rank == 0 and not args.no_cpu) else None

    near = _bind_near_gpu(local)
    wl = workloads.ragged_spd(SEED + rank, COUNT)
    a_host = torch.from_numpy(wl.a).pin_memory()
    b_host = torch.from_numpy(wl.b).pin_memory()
    rb = batched.RaggedBatch.from_packed(a_host.to(dev), b_host.to(dev), wl.n, wl.nrhs, dev)
    ws = batched.MixedWorkspace(rb.batch, rb.max_n, rb.max_nrhs, dev)
    # one persistent launch per step, replayed from a captured CUDA graph
    graphed = batched.CapturedMixedSolve(rb, TOL, workspace=ws)
    out = graphed.out
    stream = torch.cuda.current_stream(dev)

    def step():
        graphed.replay()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        barrier()
        t_all0 = torch.cuda.Event(enable_timing=True)
        t_all1 = torch.cuda.Event(enable_timing=True)
        t_all0.record(stream)
        for s0, s1 in ev:
            s0.record(stream)
            step()
            s1.record(stream)
        t_all1.record(stream)
        torch.cuda.synchronize()
        barrier()
    total_ms = t_all0.elapsed_time(t_all1)
    per_step = sorted(s0.elapsed_time(s1) for s0, s1 in ev)

    # correctness of the timed results
    info = out.info.cpu().numpy()
    berr = out.berr.cpu().numpy()
    iters = out.iters.cpu().numpy()
    ok = bool((info == 0).all() and (berr <= TOL).all())
    x_host = out.x.cpu().numpy()
    check = []
    for s in (0, len(wl.n) // 2, len(wl.n) - 1):
        n, k = wl.n[s], wl.nrhs[s]
        a_s = rb.system_a(s).cpu().numpy()
        xs = x_host[rb.b_off_host[s]: rb.b_off_host[s] + n * k].reshape(k, n)
        bs = wl.b[rb.b_off_host[s]: rb.b_off_host[s] + n * k].reshape(k, n)
        # normwise backward error ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf), in
        # extended precision so the check resolves 1e-12
        al, xl, bl = (v.astype(np.longdouble) for v in (a_s, xs, bs))
        check.append(max(float(np.abs(bl[j] - al @ xl[j]).max()
                               / (np.abs(al).sum(1).max() * np.abs(xl[j]).max()
                                  + np.abs(bl[j]).max())) for j in range(k)))
    ok = ok and max(check) <= TOL

    # plain FP64 GPU path on the same inputs (factor + solve)
    fp64_steps = max(2, min(args.steps, 5))
    u, _ = batched.cholesky_factor_ragged(rb)
    batched.cholesky_solve_ragged(rb, u)
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(fp64_steps):
        u, finfo = batched.cholesky_factor_ragged(rb)
        x64, _ = batched.cholesky_solve_ragged(rb, u)
    f1.record(stream)
    torch.cuda.synchronize()
    fp64_ms = f0.elapsed_time(f1) / fp64_steps
    fp64_ok = bool((finfo.cpu().numpy() == 0).all())
    del u, x64

    # end to end through the public host-buffer API
    hs = batched.HostRaggedSPDSolver(wl.n, wl.nrhs, TOL, device=dev)
    x_h = torch.empty(hs.out.x.numel(), dtype=torch.float64).pin_memory()
    i_h = torch.empty(rb.batch, dtype=torch.int32).pin_memory()
    it_h = torch.empty(rb.batch, dtype=torch.int32).pin_memory()
    be_h = torch.empty(rb.batch, dtype=torch.float64).pin_memory()
    for _ in range(max(1, args.warmup)):
        hs(a_host, b_host, x_h, i_h, it_h, be_h)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        hs(a_host, b_host, x_h, i_h, it_h, be_h)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    e2e_ok = bool((i_h.numpy() == 0).all() and (be_h.numpy() <= TOL).all())
    # the host-to-device rate of one plain copy of the matrices (explains e2e)
    a_chk = torch.empty_like(rb.a)
    c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    c0.record(stream)
    a_chk.copy_(a_host, non_blocking=True)
    c1.record(stream)
    torch.cuda.synchronize()
    h2d_gbs = a_host.numel() * 8 / (c0.elapsed_time(c1) * 1e-3) / 1e9
    del a_chk
    total_ms, e2e_ms, fp64_ms = max_over_ranks([total_ms, e2e_ms, fp64_ms], world, dev)

    if rank != 0:
        return
    ns = np.array(wl.n, dtype=np.float64)
    ks = np.array(wl.nrhs, dtype=np.float64)
    it = iters.astype(np.float64)
    hbm_bytes = float((8 * ns * ns).sum() + (16 * ns * ks).sum())  # A read once, b in, x out
    fp32_flops = float((ns ** 3 / 3).sum() + (4 * ns * ns * ks * it).sum())
    fp64_flops = float((2 * ns * ns * ks * it).sum())
    ms = total_ms / args.steps
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = hbm_bytes / (ms * 1e-3) / 1e9
    line = {
        "metric": METRIC,
        "value": COUNT * world / (ms * 1e-3),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 factor + f64 refinement",
        "data": "synthetic (seeded numpy PCG64, per-system streams)",
        "config": {
            "workload": WORKLOAD, "systems_per_gpu": COUNT, "n": "log-uniform [16,512]",
            "nrhs": "1..8", "A": "G G^T/n + 1e-2 I", "tol": TOL,
            "l2": "inputs larger than L2 (%.2f GB of matrices per step)" % (8 * (ns * ns).sum() / 1e9),
            "parallelism": f"replicas x{world}",
            "launch": "one persistent posv_mixed_kernel launch per step, replayed from a "
                      "captured CUDA graph",
            "trailing_update": "tcgen05 TF32 split" if args.tensor_core_update else "FP32 cores",
        },
        "latency_ms": {"p50": _pct(per_step, 50), "p99": _pct(per_step, 99)},
        "correct": {"all_berr_le_tol": ok, "max_berr": float(berr.max()),
                    "iters_mean": float(it.mean()), "iters_max": int(it.max())},
        "fp64_plain_gpu": {"value": COUNT * world / (fp64_ms * 1e-3), "unit": UNIT,
                           "ms_per_step": fp64_ms, "info_ok": fp64_ok,
                           "speedup_of_mixed": fp64_ms / ms},
        "e2e": {"value": COUNT * world / (e2e_ms * 1e-3), "unit": UNIT, "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": hs.h2d_bytes, "d2h_bytes_per_step": hs.d2h_bytes,
                "ok": e2e_ok, "api": "batched.HostRaggedSPDSolver",
                "h2d_gbs_plain_copy": h2d_gbs,
                "host_cpus": "near the GPU: %s" % (f"{near[0]}-{near[-1]}" if near else
                                                   "unchanged"),
                "overlap": f"{len(hs.sets)} device buffer sets: the host-to-device copy of "
                           "step k+1 (side stream) overlaps the solve of step k; every step "
                           "copies its inputs in and its results out inside the timed region"},
        "gpu_launches": 2 * args.steps,
        "roofline": {
            "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
            "frac": achieved / hbm_peak,
            # DRAM bytes per launch from one ncu capture of this 4096-system
            # launch: 3964.1 MB read + 930.3 MB written (A is read by the
            # FP32 copy and by each refinement residual; factor slices of
            # large systems spill from L2); scaled by the algorithmic bytes
            # when --systems changes the workload.
            "traffic": 4894.4e6 * hbm_bytes / 1215167544.0,
            "kernel": "posv_mixed_kernel",
            "note": "HBM roofline of the algorithmic bytes (A read once, b, x); the kernel is "
                    "latency-bound (barriers, shared-memory and FP latency at 16 warps per "
                    "SM), see compute",
            "compute": {"fp32_flops": fp32_flops, "fp64_flops": fp64_flops,
                        "fp32_tflops": fp32_flops / (ms * 1e-3) / 1e12,
                        "fp64_tflops": fp64_flops / (ms * 1e-3) / 1e12},
        },
        "clocks": clk.summary(),
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if not args.no_serve and world == 1:
        # the served mixed request stream against the plain FP64 server
        # (the metric's stream), with its own clock record
        line["serving"] = serve_suite(args, dev, loads=(0.5,))
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Secondary workload: mixed-precision LU + GMRES-IR (dense n×n, 16 RHS)
# ---------------------------------------------------------------------------
def haar_conditioned(n, cond, seed, dev):
    """A = U diag(sigma) Vᵀ, U and V Haar-orthogonal (QR of a Gaussian with the
    sign fix), sigma log-spaced from 1 to 1/cond.  Generated on the GPU with
    torch (input preparation, not part of any timed region)."""
    import torch

    g = torch.Generator(device=dev).manual_seed(seed)

    def haar():
        q, r = torch.linalg.qr(torch.randn(n, n, dtype=torch.float64, device=dev, generator=g))
        return q * torch.sign(torch.diagonal(r))

    u, v = haar(), haar()
    sig = torch.logspace(0, -float(__import__("math").log10(cond)), n, dtype=torch.float64,
                         device=dev)
    a = (u * sig) @ v.T
    del u, v
    return a.contiguous()


def run_gmres_ir(args):
    """Dense n×n, 16 right-hand sides, cond in {1e2, 1e6, 1e10}: FP32 LU with
    BF16, TF32 or 3xTF32 tensor-core updates + GMRES-IR to backward error <= 1e-12
    (a stalled factor escalates to the next precision before the FP64 LU),
    against the plain FP64 LU of this library.  One JSON line per case."""
    import time

    import torch

    from lineax_gb300 import _dense, mixed

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    n, k = args.n, 16
    g = torch.Generator(device=dev).manual_seed(11)
    b = torch.randn(k, n, dtype=torch.float64, device=dev, generator=g)
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def emit(obj):
        obj.update({"workload": f"gmres_ir_dense_n{n}_16rhs", "n": n, "nrhs": k})
        print(json.dumps(obj), flush=True)

    # warm-up: module load and first-call costs of every kernel used below
    a0 = haar_conditioned(256, 1e2, 1, dev)
    for prec in ("bf16", "tf32", "3xtf32"):
        mixed.gmres_ir(a0, b[:, :256].contiguous(), precision=prec, restart=args.restart)
    lu0, piv0 = _dense.lu_factor(a0)
    _dense.lu_solve(lu0, piv0, b[:, :256].contiguous())
    torch.cuda.synchronize()
    for cond in [float(c) for c in args.conds.split(",")]:
        a = haar_conditioned(n, cond, 5, dev)
        anorm = float(mixed.norm_inf(a).item())
        bn = b.abs().amax(dim=1)
        if (cond == 1e2 or args.fp64_all) and not args.no_fp64:
            e0, e1, e2 = ev(), ev(), ev()
            e0.record()
            lu, piv = _dense.lu_factor(a)
            e1.record()
            x = _dense.lu_solve(lu, piv, b)
            e2.record()
            torch.cuda.synchronize()
            r = b - (a @ x.T).T
            berr = (r.abs().amax(dim=1) / (anorm * x.abs().amax(dim=1) + bn)).max().item()
            emit({"case": "fp64_lu", "cond": cond, "factor_ms": e0.elapsed_time(e1),
                  "solve_ms": e1.elapsed_time(e2), "total_ms": e0.elapsed_time(e2),
                  "max_berr": berr, "solves_per_s": k / (e0.elapsed_time(e2) * 1e-3)})
            if not args.no_cpu:
                import scipy.linalg as sl

                ah, bh = a.cpu().numpy(), b.cpu().numpy()
                cpu_s, reps = _cpu_time(lambda: sl.lu_solve(sl.lu_factor(ah), bh.T),
                                        min_seconds=1.0, max_reps=3)
                emit({"case": "cpu_baseline", "cond": cond, "value": k / cpu_s,
                      "unit": "solves/s", "cores": _host_cores(), "kind": "port",
                      "sample": f"SciPy LAPACK lu_factor + lu_solve of the same n={n} "
                                f"system, 16 right-hand sides, {reps} repetitions",
                      "ms": cpu_s * 1e3})
            del lu, x
            torch.cuda.empty_cache()
        for prec in args.precisions.split(","):
            t0 = time.perf_counter()
            e = [ev() for _ in range(5)]
            e[0].record()
            f = mixed.lu_factor_tf32(a, prec)
            e[1].record()
            inv = mixed.lu_inverse(f, prec)
            e[2].record()
            sp = mixed.split_matrix(a)
            e[3].record()
            res = mixed.gmres_ir(a, b, tol=1e-12, restart=args.restart, max_outer=20,
                                 inner_max_steps=args.inner_max_steps, factor=f, inverse=inv,
                                 split=sp, precision=prec, arith=args.arith, fallback=True,
                                 escalate=args.arith == "auto")
            e[4].record()
            torch.cuda.synchronize()
            total = e[0].elapsed_time(e[4])
            emit({"case": f"gmres_ir_{prec}", "cond": cond, "restart": args.restart,
                  "arith": args.arith,
                  "factor_ms": e[0].elapsed_time(e[1]), "inverse_ms": e[1].elapsed_time(e[2]),
                  "split_ms": e[2].elapsed_time(e[3]), "refine_ms": e[3].elapsed_time(e[4]),
                  "total_ms": total, "outer": res.outer, "inner_cycles": res.inner_steps,
                  "max_berr": max(res.berr), "converged": res.converged,
                  "fp64_fallback": res.fallback,
                  "tiers": [{"factor": t[0], "outer": t[1], "converged": t[2]}
                            for t in res.tiers],
                  "solves_per_s": k / (total * 1e-3), "wall_s": time.perf_counter() - t0})
            del f, inv, sp, res
            torch.cuda.empty_cache()
        del a
        torch.cuda.empty_cache()


def _events(n):
    import torch

    return [torch.cuda.Event(enable_timing=True) for _ in range(n)]


def _cpu_time(fn, min_seconds=3.0, max_reps=1000):
    """Host-core timing of fn (all threads the BLAS uses): repeats until
    min_seconds have passed; returns (seconds per call, calls)."""
    fn()  # warm (imports, first touch)
    t0, reps = time.perf_counter(), 0
    while True:
        fn()
        reps += 1
        el = time.perf_counter() - t0
        if el >= min_seconds or reps >= max_reps:
            return el / reps, reps


def _host_cores():
    return len(os.sched_getaffinity(0))


def _fp64_peak():
    """Measured FP64 DGEMM rate on this GPU type (TFLOP/s), the FP64 roofline."""
    return 1.10


def run_lu_batch(args):
    """Plain FP64 LU: 64 systems, n = 128, A = G/sqrt(n) + I, one right-hand
    side each, factor + solve per step through lineax_gb300's batched LU."""
    import numpy as np
    import torch

    import scipy.linalg as sl

    from lineax_gb300 import _dense, workloads

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    batch, n = 64, 128
    a_h, b_h = workloads.lu_batch(0, batch, n)
    a = torch.tensor(a_h, device=dev)
    b = torch.tensor(b_h, device=dev)
    a_pin = torch.tensor(a_h).pin_memory()
    b_pin = torch.tensor(b_h).pin_memory()
    x_pin = torch.empty_like(b_pin).pin_memory()

    def step():
        lu, piv, _ = _dense.lu_factor_batched(a)
        return _dense.lu_solve_batched(lu, piv, b)

    def step_e2e():
        a_d = a_pin.to(dev, non_blocking=True)
        b_d = b_pin.to(dev, non_blocking=True)
        lu, piv, _ = _dense.lu_factor_batched(a_d)
        x_pin.copy_(_dense.lu_solve_batched(lu, piv, b_d), non_blocking=True)

    from lineax_gb300 import _ffi

    # The 8 MB of matrices fit in L2: a 256 MB buffer is written between
    # timed steps (outside the events) so every step starts from HBM.
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        total = 0.0
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0, e1 = _events(2)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1)
        return total / args.steps

    ms = timed(step)
    ms_factor = timed(lambda: _dense.lu_factor_batched(a))
    ms_e2e = timed(step_e2e)
    try:
        _ffi.call("lxgb_getrf_set_pair", 1)
        ms_pair = timed(step)
        ms_factor_pair = timed(lambda: _dense.lu_factor_batched(a))
    finally:
        _ffi.call("lxgb_getrf_set_pair", 0)
    x = step().cpu().numpy()
    berr = max(float(np.abs(b_h[i] - a_h[i] @ x[i]).max()
                     / (np.abs(a_h[i]).sum(1).max() * np.abs(x[i]).max() + np.abs(b_h[i]).max()))
               for i in range(batch))
    lu_ref = [sl.lu_factor(a_h[i]) for i in range(4)]
    flops = batch * (2 / 3 * n ** 3 + 2 * n * n)

    def cpu_step():
        for i in range(batch):
            sl.lu_solve(sl.lu_factor(a_h[i]), b_h[i])

    cpu_s, cpu_reps = _cpu_time(cpu_step)
    print(json.dumps({
        "workload": "lu_batch_64x128_f64", "metric": "LU solves/s (factor + solve)",
        "unit": "solves/s", "value": batch / (ms * 1e-3), "ms_per_step": ms,
        "e2e": {"value": batch / (ms_e2e * 1e-3), "unit": "solves/s",
                "h2d_bytes_per_step": int(a_pin.numel() * 8 + b_pin.numel() * 8),
                "d2h_bytes_per_step": int(x_pin.numel() * 8)},
        "max_berr": berr, "pivots_match_lapack": bool(all(
            np.array_equal(_dense.lu_factor_batched(a[i:i + 1])[1].cpu().numpy()[0], lu_ref[i][1])
            for i in range(4))),
        "roofline": {"bound": "fp64", "achieved": flops / (ms * 1e-3) / 1e12,
                     "peak": _fp64_peak(), "unit": "TFLOP/s",
                     "frac": flops / (ms * 1e-3) / 1e12 / _fp64_peak(),
                     "factor_only": {"ms": ms_factor,
                                     "frac": batch * 2 / 3 * n ** 3 / (ms_factor * 1e-3) / 1e12
                                     / _fp64_peak()}},
        "two_cta_cluster_per_matrix": {"ms_per_step": ms_pair, "factor_ms": ms_factor_pair,
                                       "value": batch / (ms_pair * 1e-3)},
        "l2": "256 MB written between timed steps (the inputs fit in L2)",
        "kernel": "getrf_small_kernel (one CTA per matrix, lookahead pivot search) + "
                  "getrs_small_kernel",
        "cpu_baseline": {"value": batch / cpu_s, "unit": "solves/s", "cores": _host_cores(),
                         "kind": "port", "sample": f"the same 64 systems, SciPy LAPACK "
                         f"lu_factor + lu_solve, {cpu_reps} repetitions"},
        "steps": args.steps, "warmup": args.warmup}), flush=True)


def run_qr_ls(args):
    """Least squares with Householder QR: A 16384×2048 (FP32-valued, N(0,1)),
    b = A x* + 1e-3 eps, through lx.linear_solve(..., lx.QR()) in FP64 and
    through lx.QR(precision="mixed") (TF32 tensor-core QR + corrected
    semi-normal equations refined to FP64 accuracy)."""
    import torch

    import lineax_gb300 as lx

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    m, n = args.qr_m, args.qr_n
    g = torch.Generator(device=dev).manual_seed(3)
    a = torch.randn(m, n, device=dev, generator=g).double()
    xs = torch.randn(n, dtype=torch.float64, device=dev, generator=g)
    b = a @ xs + 1e-3 * torch.randn(m, dtype=torch.float64, device=dev, generator=g)
    op = lx.MatrixLinearOperator(a)
    flops = 2 * m * n * n - 2 * n ** 3 / 3
    out = {"workload": f"qr_least_squares_{m}x{n}", "metric": "least-squares solves/s",
           "unit": "solves/s"}
    xref = None
    for name, solver in (("fp64", lx.QR()), ("mixed", lx.QR(precision="mixed")),
                         ("normal_cholesky", lx.Normal(lx.Cholesky()))):
        def step():
            return lx.linear_solve(op, b, solver).value

        for _ in range(args.warmup):
            x = step()
        torch.cuda.synchronize()
        e0, e1 = _events(2)
        e0.record()
        for _ in range(args.steps):
            x = step()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        r = b - a @ x
        opt = float((a.T @ r).abs().max() / (a.abs().sum(0).max() * r.abs().max()))
        if xref is None:
            xref = x
        out[name] = {
            "solves_per_s": 1e3 / ms, "ms_per_step": ms, "normal_equations_residual": opt,
            "max_abs_diff_vs_fp64_qr": float((x - xref).abs().max()),
            "roofline": ({"bound": "fp64", "achieved": flops / (ms * 1e-3) / 1e12,
                          "peak": _fp64_peak(), "unit": "TFLOP/s",
                          "frac": flops / (ms * 1e-3) / 1e12 / _fp64_peak()}
                         if name == "fp64" else
                         {"bound": "tensor (TF32 updates)", "effective_tflops":
                          flops / (ms * 1e-3) / 1e12} if name == "mixed" else
                         {"bound": "fp64 (Gram m n² + Cholesky n³/3)",
                          "achieved": (m * n * n + n ** 3 / 3) / (ms * 1e-3) / 1e12,
                          "peak": _fp64_peak(), "unit": "TFLOP/s",
                          "frac": (m * n * n + n ** 3 / 3) / (ms * 1e-3) / 1e12 / _fp64_peak()})}
    out["value"] = out["mixed"]["solves_per_s"]
    if not args.no_cpu:
        import scipy.linalg as sl

        ah, bh = a.cpu().numpy(), b.cpu().numpy()

        def cpu_step():
            q, r = sl.qr(ah, mode="economic")
            sl.solve_triangular(r, q.T @ bh)

        cpu_s, reps = _cpu_time(cpu_step, min_seconds=2.0, max_reps=3)
        out["cpu_baseline"] = {"value": 1.0 / cpu_s, "unit": "solves/s", "cores": _host_cores(),
                               "kind": "port", "sample": f"SciPy LAPACK economic QR + "
                               f"triangular solve of the same {m}×{n} problem, {reps} "
                               "repetitions"}
    out["steps"], out["warmup"] = args.steps, args.warmup
    print(json.dumps(out), flush=True)


def run_cholesky_large(args):
    """FP64 Cholesky solves of single large SPD matrices (A = G Gᵀ/n + I)
    through lx.linear_solve(..., lx.Cholesky()): the multi-CTA factorisation
    (lxgb_potrf_f64) plus the solve, and the factorisation alone."""
    import torch

    import lineax_gb300 as lx
    from lineax_gb300 import _dense

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    g = torch.Generator(device=dev).manual_seed(4)
    out = {"workload": "cholesky_large_f64", "metric": "factorisation ms", "unit": "ms",
           "cases": []}
    for n in (1024, 2048, 4096):
        gm = torch.randn(n, n, dtype=torch.float64, device=dev, generator=g)
        a = gm @ gm.T / n + torch.eye(n, dtype=torch.float64, device=dev)
        b = torch.randn(n, dtype=torch.float64, device=dev, generator=g)
        op = lx.MatrixLinearOperator(a, lx.positive_semidefinite_tag)
        case = {"n": n}
        for name, fn in (("factor", lambda: _dense.cho_factor(a)),
                         ("solve", lambda: lx.linear_solve(op, b, lx.Cholesky()).value)):
            for _ in range(args.warmup):
                fn()
            torch.cuda.synchronize()
            e0, e1 = _events(2)
            e0.record()
            for _ in range(args.steps):
                fn()
            e1.record()
            torch.cuda.synchronize()
            case[name + "_ms"] = e0.elapsed_time(e1) / args.steps
        fl = n ** 3 / 3
        case["roofline"] = {"bound": "fp64", "achieved": fl / (case["factor_ms"] * 1e-3) / 1e12,
                            "peak": _fp64_peak(), "unit": "TFLOP/s",
                            "frac": fl / (case["factor_ms"] * 1e-3) / 1e12 / _fp64_peak()}
        x = lx.linear_solve(op, b, lx.Cholesky()).value
        case["backward_error"] = float((b - a @ x).abs().max() /
                                       (a.abs().sum(1).max() * x.abs().max() + b.abs().max()))
        if not args.no_cpu:
            import scipy.linalg as sl

            ah = a.cpu().numpy()
            cpu_s, reps = _cpu_time(lambda: sl.cho_factor(ah, lower=False), min_seconds=1.0,
                                    max_reps=5)
            case["cpu_baseline"] = {"value": cpu_s * 1e3, "unit": "ms", "cores": _host_cores(),
                                    "kind": "port", "sample": f"SciPy LAPACK cho_factor of the "
                                    f"same matrix, {reps} repetitions"}
        out["cases"].append(case)
    out["steps"], out["warmup"] = args.steps, args.warmup
    print(json.dumps(out), flush=True)


def run_cg_poisson(args):
    """CG on the 5-point -Laplacian of a 2048×2048 interior grid (zero
    Dirichlet boundary, matrix-free FunctionLinearOperator), 64 right-hand
    sides, rtol = atol = 1e-10: a timed block of iterations of the FP64 CG
    (lineax's iteration statement for statement) and of the mixed-precision CG
    (FP32 iterations, FP64 residual replacement every 16), plus the full
    mixed-precision solve with --cg-full."""
    import torch

    from lineax_gb300 import _krylov
    from lineax_gb300._operator import Poisson2DOperator

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    nx = ny = args.grid
    k = args.cg_rhs
    op = Poisson2DOperator(nx, ny)
    g = torch.Generator(device=dev).manual_seed(9)
    b = torch.randn(k, nx * ny, dtype=torch.float64, device=dev, generator=g)
    rtol, atol = 1e-10, 1e-10
    points = nx * ny * k
    e0, e1 = _events(2)
    out = {"workload": f"cg_poisson_{nx}x{ny}_{k}rhs", "metric": "CG iterations/s (64 RHS)",
           "unit": "iterations/s", "rtol": rtol, "atol": atol}
    # FP64 vectors: p, Ap read/written by the stencil (16), the alpha step reads
    # Ap, p, x, r and writes x, r (48), the beta step reads r, p and writes p
    # (24), the true residual every 10th iteration adds b, Ax, r (2.4)
    for name, fn, bpp in (
            ("fp64", lambda m: _krylov.cg_block(op, b, rtol=rtol, atol=atol, max_steps=m),
             16 + 48 + 24 + 2.4),
            # FP32 vectors: stencil reads p, writes Ap (8); update reads p, Ap,
            # x_lo, r and writes x_lo, r (24); direction reads r, p, writes p
            # (12); the FP64 replacement every 16 iterations: fold x += x_lo (24)
            # and r = b - A x (20), 44 / 16 = 2.75
            ("mixed", lambda m: _krylov.cg_poisson_mixed(op, b, rtol=rtol, atol=atol,
                                                         max_steps=m), 8 + 24 + 12 + 2.75)):
        fn(args.warmup)
        torch.cuda.synchronize()
        e0.record()
        res = fn(args.cg_iters)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        iters = max(res.steps)
        gbs = bpp * points * iters / (ms * 1e-3) / 1e9
        out[name] = {"iterations_per_s": iters / (ms * 1e-3), "ms_per_iteration": ms / iters,
                     "iterations_timed": iters, "bytes_per_point_iteration": bpp,
                     "roofline": {"bound": "hbm", "achieved": gbs, "unit": "GB/s",
                                  "peak": 6784.0, "frac": gbs / 6784.0}}
    out["value"] = out["mixed"]["iterations_per_s"]
    if not args.no_cpu:
        import numpy as np
        import scipy.sparse as sp

        t1 = sp.diags([-np.ones(nx - 1), 2 * np.ones(nx), -np.ones(nx - 1)], [-1, 0, 1])
        lap = (sp.kron(sp.identity(ny), t1) + sp.kron(t1, sp.identity(nx))).tocsr()
        kb = min(k, 8)
        bh = b[:kb].cpu().numpy().T.copy()
        st = {"x": np.zeros_like(bh), "r": bh.copy(), "p": bh.copy(),
              "g": (bh * bh).sum(0)}

        def cpu_iter():  # one CG iteration on kb right-hand sides (matvec, dots, axpys)
            ap = lap @ st["p"]
            alpha = st["g"] / (st["p"] * ap).sum(0)
            st["x"] += alpha * st["p"]
            st["r"] -= alpha * ap
            gn = (st["r"] * st["r"]).sum(0)
            st["p"] = st["r"] + (gn / st["g"]) * st["p"]
            st["g"] = gn

        cpu_s, reps = _cpu_time(cpu_iter, min_seconds=3.0, max_reps=50)
        out["cpu_baseline"] = {"value": (kb / k) / cpu_s, "unit": "iterations/s (64 RHS)",
                               "cores": _host_cores(), "kind": "port",
                               "sample": f"{reps} FP64 CG iterations on {kb} of the 64 "
                               "right-hand sides with a SciPy CSR 5-point Laplacian, scaled to "
                               "64"}
    if args.cg_full:
        e0.record()
        res = _krylov.cg_poisson_mixed(op, b, rtol=rtol, atol=atol)
        e1.record()
        torch.cuda.synchronize()
        r = b - op.mv_block(res.y)
        scale = atol + rtol * b.abs()
        out["full_solve_mixed"] = {
            "ms": e0.elapsed_time(e1), "iterations": max(res.steps),
            "results": sorted(set(res.results)),
            "max_residual_over_tolerance": float((r.abs() / scale).max())}
    print(json.dumps(out), flush=True)


SERVE_ROUTES = ("chol_ragged", "lu_small", "lu_mixed", "chol_mixed", "qr_mixed", "qr_f64",
                "lu_f64", "chol_f64")


def serve_suite(args, dev, loads=(0.25, 0.5, 0.75), emit=None):
    """Serving mix (50% LU / 30% Cholesky / 20% QR, n log-uniform [32, 4096],
    1-16 right-hand sides, 30% on a resident operator): saturation throughput
    of the mixed-precision server and of the plain FP64 server on the same
    requests, then open-loop Poisson arrivals at fractions `loads` of each
    server's saturation rate for p50/p99 latency.  Clocks are sampled over the
    whole suite.  Returns a summary dict; `emit` receives each result line."""
    import torch

    from lineax_gb300 import serve

    count = args.serve_requests
    warm = serve.synthetic_requests(24, seed=99, nmax=1024)

    def pct(v, p):
        v = sorted(v)
        return v[min(len(v) - 1, int(round(p / 100.0 * (len(v) - 1))))]

    def one(mode, rate, seed):
        reqs = serve.synthetic_requests(count, seed=seed, nmax=args.serve_nmax, rate=rate,
                                        device=dev)
        for r in reqs:
            if r.a is not None:
                r.a = r.a.pin_memory()
            r.b = r.b.pin_memory()
        torch.cuda.synchronize()
        srv = serve.SolveServer(dev, mode=mode, hbm_budget=int(args.serve_budget_gb * 2**30))
        t0 = time.perf_counter()
        out = srv.run(reqs, realtime=True)
        wall = time.perf_counter() - t0
        lat = [c.latency * 1e3 for c in out]
        return {"mode": mode, "streams": srv.streams, "offered_rate": rate, "requests": len(out),
                "solves_per_s": len(out) / wall,
                "rhs_per_s": sum(r.nrhs for r in reqs) / wall, "wall_s": wall,
                "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99),
                "max_berr": max(c.berr for c in out),
                "all_berr_le_tol": all(c.berr <= TOL for c in out),
                "fallbacks": sum(c.fallback for c in out),
                "reused": sum(c.reused for c in out),
                "routes": {k: sum(c.route == k for c in out) for k in SERVE_ROUTES
                           if any(c.route == k for c in out)}}

    emit = emit or (lambda obj: None)
    tag = f"serve_{count}req_n32-{args.serve_nmax}"
    with ClockSampler(dev.index or 0) as clk:
        # warm-up: one untimed pass of each server over the timed request
        # stream itself, so neither pays first-use costs (kernel loading, the
        # allocator's first blocks of large orders) inside its timing
        for mode in ("mixed", "fp64"):
            serve.SolveServer(dev, mode=mode).run(warm, realtime=False)
            one(mode, None, 5)
        torch.cuda.synchronize()
        # three saturation passes per server, the servers alternating; each
        # server's median pass is its result (single passes of the same
        # stream have moved by up to 8 % between runs, with the host's timing)
        passes = {"fp64": [], "mixed": []}
        for _ in range(3):
            for m in ("fp64", "mixed"):
                passes[m].append(one(m, None, 5))
        sat = {}
        for m in ("fp64", "mixed"):
            runs = sorted(passes[m], key=lambda r: r["solves_per_s"])
            sat[m] = {**runs[1], "passes_solves_per_s": [r["solves_per_s"] for r in passes[m]]}
        for m in ("fp64", "mixed"):
            emit({"workload": tag, "phase": "saturation", **sat[m]})
        ratio = sat["mixed"]["solves_per_s"] / sat["fp64"]["solves_per_s"]
        emit({"workload": tag, "phase": "speedup", "mixed_over_fp64_solves_per_s": ratio})
        sweep = []
        for m in ("fp64", "mixed"):
            for frac in loads:
                row = {"load": frac, **one(m, frac * sat[m]["solves_per_s"], 6)}
                sweep.append(row)
                emit({"workload": tag, "phase": "open_loop", **row})
    keep = ("solves_per_s", "p50_ms", "p99_ms", "max_berr", "all_berr_le_tol", "fallbacks",
            "reused", "routes", "streams", "passes_solves_per_s")
    return {
        "workload": tag, "requests": count,
        "mix": f"50% LU / 30% Cholesky / 20% QR, n log-uniform [32, {args.serve_nmax}], "
               "1-16 RHS, 30% reuse",
        "saturation": {m: {k: sat[m][k] for k in keep} for m in ("mixed", "fp64")},
        "mixed_over_fp64_solves_per_s": ratio,
        "open_loop": [{k: r[k] for k in ("mode", "load", "offered_rate", "solves_per_s",
                                         "p50_ms", "p99_ms")} for r in sweep],
        "clocks": clk.summary(),
    }


def run_serve(args):
    """The serving suite alone, one JSON line per result, plus the SciPy
    CPU baseline on the same request stream."""
    import torch

    from lineax_gb300 import serve

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    summary = serve_suite(args, dev, emit=lambda o: print(json.dumps(o), flush=True))
    print(json.dumps({"workload": summary["workload"], "phase": "clocks",
                      "clocks": summary["clocks"]}), flush=True)
    if not args.no_cpu:
        # the same request stream solved one request at a time on the host
        # cores with SciPy LAPACK (Cholesky, QR or LU as the request asks)
        import scipy.linalg as sl

        reqs = serve.synthetic_requests(60, seed=5, nmax=args.serve_nmax)
        mats = {r.op_id: r.a.numpy() for r in reqs if r.a is not None}

        def cpu_stream():
            for r in reqs:
                a = mats[r.op_id]
                bb = r.b.numpy().T
                if r.kind == "cholesky":
                    sl.cho_solve(sl.cho_factor(a), bb)
                elif r.kind == "qr":
                    q, rr = sl.qr(a)
                    sl.solve_triangular(rr, q.T @ bb)
                else:
                    sl.lu_solve(sl.lu_factor(a), bb)

        cpu_s, reps = _cpu_time(cpu_stream, min_seconds=1.0, max_reps=2)
        print(json.dumps({"workload": summary["workload"], "phase": "cpu_baseline",
                          "value": len(reqs) / cpu_s, "unit": "solves/s",
                          "cores": _host_cores(), "kind": "port",
                          "sample": "the first 60 requests of the stream (no resident "
                                    "factors), SciPy LAPACK, one request at a time"}),
              flush=True)


def run_peaks(args):
    """Arithmetic reference points on this GPU: library GEMMs (torch.matmul,
    FP64 / FP32 / TF32 / BF16, a sanity line) and this library's tcgen05 TF32,
    3xTF32 and BF16 GEMMs (persistent kernel, and the one-tile-per-CTA kernel
    beside it) on the same square shape and on the rank-64 update shape of the
    LU factorisations.  Best of 5 CUDA-event timings after 2 warm-ups."""
    import torch

    from lineax_gb300 import _blas

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    n = args.peaks_n
    out = {"workload": f"gemm_peaks_{n}"}

    def best(fn, flops):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(5):
            e0, e1 = _events(2)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return flops / (min(ts) * 1e-3) / 1e12

    g = torch.Generator(device=dev).manual_seed(0)
    a32 = torch.randn(n, n, device=dev, generator=g)
    b32 = torch.randn(n, n, device=dev, generator=g)
    c32 = torch.zeros(n, n, device=dev)
    fl = 2.0 * n ** 3
    if not args.peaks_ours_only:
        a64, b64 = a32.double(), b32.double()
        out["torch_fp64_tflops"] = best(lambda: a64 @ b64, fl)
        torch.backends.cuda.matmul.allow_tf32 = False
        out["torch_fp32_tflops"] = best(lambda: a32 @ b32, fl)
        torch.backends.cuda.matmul.allow_tf32 = True
        out["torch_tf32_tflops"] = best(lambda: a32 @ b32, fl)
        torch.backends.cuda.matmul.allow_tf32 = False
        del a64, b64
    from lineax_gb300 import _ffi

    a16 = a32.to(torch.bfloat16)
    b16 = b32.to(torch.bfloat16)
    err = torch.zeros(1, dtype=torch.int32, device=dev)

    def bf16_gemm(a, b, c, alpha=1.0, beta=0.0):
        _ffi.call("lxgb_gemm_bf16_nt", a.shape[0], b.shape[0], a.shape[1], _ffi.ptr(a),
                  a.stride(0), _ffi.ptr(b), b.stride(0), _ffi.ptr(c), c.stride(0), alpha, beta,
                  _ffi.ptr(err), _ffi.stream_handle(dev))

    if not args.peaks_ours_only:
        out["torch_bf16_tflops"] = best(lambda: a16 @ b16.T, fl)
    # the LU trailing update: C (n×n) -= A (n×64) Bᵀ (n×64), C read and written
    a_k = a32[:, :64].contiguous()
    b_k = b32[:, :64].contiguous()
    for tag, on in (("", 1), ("_tile", 0)):
        # "" = the persistent kernel (default), "_tile" = one CTA per 128×128 tile
        _ffi.call("lxgb_gemm_set_persistent", on)
        out[f"lxgb_tf32{tag}_tflops"] = best(lambda: _blas.gemm_tf32_nt(a32, b32, c32), fl)
        out[f"lxgb_3xtf32{tag}_tflops"] = best(lambda: _blas.gemm_3xtf32_nt(a32, b32, c32), fl)
        out[f"lxgb_bf16{tag}_tflops"] = best(lambda: bf16_gemm(a16, b16, c32), fl)
        t = best(lambda: _blas.gemm_tf32_nt(a_k, b_k, c32, alpha=-1.0, beta=1.0),
                 2.0 * n * n * 64)
        out[f"lxgb_tf32{tag}_rank64_tflops"] = t
        out[f"lxgb_tf32{tag}_rank64_gbs"] = t * 1e12 / (2.0 * n * n * 64) * (8.0 * n * n) / 1e9
    _ffi.call("lxgb_gemm_set_persistent", 1)
    torch.cuda.synchronize()
    out["pipeline_timeouts"] = int(err.item())
    print(json.dumps(out), flush=True)


def main():
    global COUNT
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline measurement")
    p.add_argument("--no-serve", action="store_true",
                   help="skip the serving suite in the default line")
    p.add_argument("--tensor-core-update", action="store_true",
                   help="ragged factor: trailing updates on the tensor cores (TF32 split)")
    p.add_argument("--systems", type=int, default=COUNT,
                   help="systems per GPU (smaller values are for profiling runs only)")
    p.add_argument("--workload", default="ragged_cholesky",
                   choices=["ragged_cholesky", "gmres_ir", "lu_batch", "qr_ls", "cg_poisson",
                            "serve", "peaks", "cholesky_large"],
                   help="gmres_ir: the dense mixed-precision LU + GMRES-IR workload")
    p.add_argument("--n", type=int, default=8192, help="order for --workload gmres_ir")
    p.add_argument("--restart", type=int, default=8, help="GMRES restart for --workload gmres_ir")
    p.add_argument("--inner-max-steps", type=int, default=5,
                   help="GMRES restart cycles per refinement step before falling back to FP64")
    p.add_argument("--conds", default="1e2,1e6,1e10", help="condition numbers (gmres_ir)")
    p.add_argument("--qr-m", type=int, default=16384, help="rows for --workload qr_ls")
    p.add_argument("--qr-n", type=int, default=2048, help="columns for --workload qr_ls")
    p.add_argument("--grid", type=int, default=2048, help="grid side for --workload cg_poisson")
    p.add_argument("--cg-rhs", type=int, default=64, help="right-hand sides (cg_poisson)")
    p.add_argument("--cg-iters", type=int, default=200, help="timed CG iterations (cg_poisson)")
    p.add_argument("--cg-full", action="store_true", help="also run CG to rtol 1e-10")
    p.add_argument("--serve-requests", type=int, default=300, help="requests (serve)")
    p.add_argument("--peaks-n", type=int, default=8192, help="GEMM order (peaks)")
    p.add_argument("--peaks-ours-only", action="store_true",
                   help="time only this library's GEMMs (peaks)")
    p.add_argument("--serve-nmax", type=int, default=4096, help="largest order (serve)")
    p.add_argument("--serve-budget-gb", type=float, default=64.0, help="HBM budget (serve)")
    p.add_argument("--arith", default="auto", choices=["auto", "df", "fp32"],
                   help="inner GMRES arithmetic (gmres_ir)")
    p.add_argument("--precisions", default="bf16,tf32,3xtf32",
                   help="first factor precision of each case (gmres_ir; a stalled factor "
                        "escalates bf16 -> tf32 -> 3xtf32 -> FP64)")
    p.add_argument("--no-fp64", action="store_true", help="skip the FP64 LU line (gmres_ir)")
    p.add_argument("--fp64-all", action="store_true",
                   help="time the plain FP64 LU at every condition number (gmres_ir)")
    args = p.parse_args()
    COUNT = args.systems
    if args.tensor_core_update:
        from lineax_gb300 import _ffi
        _ffi.call("lxgb_posv_mixed_set_tensor_cores", 1)
    modes = {"gmres_ir": run_gmres_ir, "lu_batch": run_lu_batch, "qr_ls": run_qr_ls,
             "cg_poisson": run_cg_poisson, "serve": run_serve, "peaks": run_peaks,
             "cholesky_large": run_cholesky_large}
    if args.workload in modes:
        # every secondary workload's lines come with the clocks sampled while it ran
        with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
            modes[args.workload](args)
        print(json.dumps({"workload": args.workload, "phase": "clocks",
                          "clocks": clk.summary()}), flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
