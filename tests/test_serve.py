"""Serving loop: admission and residency logic on the CPU; on the GPU, every
request solved to FP64 backward error, results independent of the batch a
request was served in, and resident factors reused."""

import pytest
import torch

from lineax_gb300 import serve


def req(rid, kind, n, k=1, op=None, arrival=0.0, with_a=True):
    b = torch.zeros(k, n, dtype=torch.float64)
    a = torch.eye(n, dtype=torch.float64) if with_a else None
    return serve.Request(rid, kind, b, rid if op is None else op, a, arrival)


def test_routes():
    assert serve.route_of("cholesky", 1024, "mixed") == "chol_ragged"
    assert serve.route_of("cholesky", 1025, "mixed") == "chol_mixed"
    assert serve.route_of("cholesky", 1025, "fp64") == "chol_f64"
    assert serve.route_of("qr", 100, "mixed") == "qr_f64"   # QR requests are served by QR
    assert serve.route_of("qr", 169, "mixed") == "qr_f64"     # FP64 is faster below 512
    assert serve.route_of("qr", 512, "mixed") == "qr_mixed"
    assert serve.route_of("lu", 511, "mixed") == "lu_f64"
    assert serve.route_of("lu", 512, "mixed") == "lu_mixed"
    assert serve.route_of("qr", 4096, "fp64") == "qr_f64"
    assert serve.route_of("lu", 100, "mixed") == "lu_small"
    assert serve.route_of("lu", 169, "fp64") == "lu_f64"
    with pytest.raises(ValueError):
        serve.route_of("svd", 10, "mixed")


def test_admission_is_fifo_and_respects_arrival_and_budget():
    s = serve.Scheduler(budget_bytes=serve.footprint("lu_mixed", 2000, 1) * 2, mode="mixed")
    for r in (req(0, "lu", 2000), req(1, "lu", 2000), req(2, "lu", 2000), req(3, "lu", 50,
                                                                                arrival=5.0)):
        s.submit(r)
    first = s.admit(now=1.0)
    assert [r.rid for r in first] == [0, 1]          # the third does not fit beside them
    assert s.admit(now=1.0) == []                    # still in flight: no room
    s.release(first)                                 # they finished
    second = s.admit(now=1.0)
    assert [r.rid for r in second] == [2]            # request 3 has not arrived yet
    assert s.admit(now=1.0) == [] and s.next_arrival() == 5.0
    assert [r.rid for r in s.admit(now=5.0)] == [3]  # small: fits beside request 2
    s.release(second)
    assert s.inflight > 0                             # request 3 still charged


def test_residents_are_charged_and_evicted_lru():
    per = serve.resident_bytes("lu_mixed", 1000)
    s = serve.Scheduler(budget_bytes=int(per * 2.5), mode="mixed")
    s.remember("a", per, "A")
    s.remember("b", per, "B")
    assert s.lookup("a") == "A"                      # a becomes most recently used
    s.remember("c", per, "C")                        # evicts b, the least recently used
    assert s.lookup("b") is None and s.lookup("a") == "A" and s.lookup("c") == "C"
    assert s.resident_total == 2 * per
    # an arriving request that needs room evicts residents it does not use
    s.submit(req(9, "lu", 1000, op="c"))
    got = s.admit(now=0.0)
    assert [r.rid for r in got] == [9] and s.lookup("c") == "C"


def test_request_larger_than_budget_is_rejected():
    s = serve.Scheduler(budget_bytes=1 << 20, mode="mixed")
    s.submit(req(0, "lu", 4096))
    s.submit(req(1, "lu", 40))
    assert [r.rid for r in s.admit(now=0.0)] == [1]
    assert [r.rid for r in s.rejected] == [0]


class _HostOnlyServer(serve.SolveServer):
    """The serving loop's host side (admission, worker threads, completion
    bookkeeping) with jobs that touch no device: each job records whether its
    operator's matrix is known when it runs and waits `delay[rid]` seconds."""

    def __init__(self, delay, **kw):
        super().__init__(torch.device("cuda", 0), mode="mixed", hbm_budget=1 << 34, **kw)
        self.delay, self.seen = delay, {}

    def _jobs(self, batch):
        return [(self._fake, [r]) for r in batch]

    def _fake(self, reqs):
        import time

        r = reqs[0]
        time.sleep(self.delay.get(r.rid, 0.0))
        self.seen[r.rid] = r.a is not None or r.op_id in self.registry
        return [serve.Completion(r.rid, r.b, 0.0, "host", False, r.a is None)]

    def _work(self, fn, reqs, t0):
        import time

        out = fn(reqs)
        for c in out:
            c.finished = time.perf_counter() - t0
        return out


def test_reuse_request_finds_its_matrix_when_it_runs_first():
    # Request 0 defines operator 7 and is slow; request 1 reuses operator 7,
    # arrives right after it and, on another worker, runs first.  The matrix
    # must be known from the moment request 0 was sent.
    reqs = [req(0, "lu", 600, op=7), req(1, "lu", 600, op=7, arrival=0.001, with_a=False),
            req(2, "cholesky", 1200), req(3, "qr", 800, arrival=0.002)]
    srv = _HostOnlyServer({0: 0.2}, streams=3)
    out = srv.run(reqs, realtime=True)
    assert [c.rid for c in out] == [0, 1, 2, 3]
    assert all(srv.seen[r.rid] for r in reqs)
    assert srv.seen and out[1].finished < out[0].finished   # the reuse really ran first
    assert all(c.latency >= 0.0 for c in out)
    assert srv.sched.inflight == 0                          # every job returned its footprint


def test_synthetic_mix_shapes():
    reqs = serve.synthetic_requests(60, seed=1, nmax=600, rate=100.0)
    assert all(r.kind in serve.KINDS and 32 <= r.n <= 600 and 1 <= r.nrhs <= 16 for r in reqs)
    assert all(b.arrival >= a.arrival for a, b in zip(reqs, reqs[1:]))
    reused = [r for r in reqs if r.a is None]
    assert reused and all(any(o.op_id == r.op_id and o.a is not None for o in reqs) for r in reused)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_serve_mix_backward_error_and_batch_independence(dev, mode):
    reqs = serve.synthetic_requests(40, seed=3, nmax=1400)   # every route up to chol_mixed
    srv = serve.SolveServer(dev, mode=mode)
    out = srv.run(reqs, realtime=False)
    assert len(out) == len(reqs)
    for c, r in zip(out, reqs):
        assert c.rid == r.rid and c.berr <= 1e-12, (c.route, c.berr)
        assert c.x.shape == (r.nrhs, r.n)
    assert any(c.reused for c in out) or mode == "mixed" and not any(
        c.route == "lu_mixed" for c in out)
    # each request again on a fresh server, alone: bit-identical results
    for r in reqs[:12]:
        alone = serve.SolveServer(dev, mode=mode)
        for o in reqs:
            if o.a is not None:
                alone.register(o.op_id, o.a)
        c = alone.run([serve.Request(r.rid, r.kind, r.b, r.op_id, r.a, 0.0)], realtime=False)[0]
        assert torch.equal(c.x, out[r.rid].x), (r.kind, r.n, c.route)


def test_pipeline_flag_is_checked_once_per_request():
    serve._check_pipeline(None)
    serve._check_pipeline(torch.zeros(1, dtype=torch.int32))
    with pytest.raises(RuntimeError, match="pipeline timed out"):
        serve._check_pipeline(torch.ones(1, dtype=torch.int32))


def test_resident_of_a_timed_out_factor_is_dropped():
    srv = _HostOnlyServer({})
    per = serve.resident_bytes("lu_mixed", 512)
    srv.sched.remember(7, per, "factor")
    srv._check_or_forget(torch.zeros(1, dtype=torch.int32), 7)     # flag clear: kept
    assert srv.sched.lookup(7) == "factor"
    with pytest.raises(RuntimeError, match="pipeline timed out"):
        srv._check_or_forget(torch.ones(1, dtype=torch.int32), 7)
    assert srv.sched.lookup(7) is None and srv.sched.resident_total == 0
    srv.sched.forget(7)                                            # absent: no effect
    assert srv.sched.resident_total == 0
