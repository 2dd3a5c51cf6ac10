"""Serving loop admission on the host (no GPU): slots and the HBM budget
bound the concurrency, arrivals are served in order, oversize jobs are
refused, and the latency statistics come out of a stream of arrivals."""
import threading
import time

import pytest

from orthoroute_gb300.serve import RouteJob, RouteServer, job_footprint, poisson_arrivals


class _Probe:
    def __init__(self, dur=0.05):
        self.dur = dur
        self.lock = threading.Lock()
        self.active = 0
        self.peak = 0
        self.order = []

    def __call__(self, job):
        with self.lock:
            self.active += 1
            self.peak = max(self.peak, self.active)
            self.order.append(job.name)
        time.sleep(self.dur)
        with self.lock:
            self.active -= 1
        return {"name": job.name, "paths": {}}


def _jobs(n, size=10):
    return [RouteJob(f"J{i}", size, size, 4, [("N0", 0, 5)], max_iterations=1) for i in range(n)]


def test_slots_bound_concurrency():
    probe = _Probe()
    srv = RouteServer(slots=3, hbm_budget_bytes=1 << 40, executor=probe, footprint=lambda j: 1)
    futs = [srv.submit(j) for j in _jobs(9)]
    res = [f.result(timeout=30) for f in futs]
    srv.close()
    assert probe.peak == 3 and srv.peak_running == 3
    assert [r.name for r in res] == [f"J{i}" for i in range(9)]
    assert all(r.error is None and r.latency >= 0 for r in res)
    assert probe.order == [f"J{i}" for i in range(9)]   # FIFO admission


def test_hbm_budget_bounds_concurrency():
    probe = _Probe()
    srv = RouteServer(slots=8, hbm_budget_bytes=250, executor=probe, footprint=lambda j: 100)
    futs = [srv.submit(j) for j in _jobs(6)]
    [f.result(timeout=30) for f in futs]
    srv.close()
    assert probe.peak == 2 and srv.peak_bytes <= 250


def test_oversize_job_is_refused():
    srv = RouteServer(slots=2, hbm_budget_bytes=50, executor=_Probe(), footprint=lambda j: 100)
    fut = srv.submit(_jobs(1)[0])
    with pytest.raises(MemoryError):
        fut.result(timeout=5)
    srv.close()


def test_executor_errors_are_reported_per_job():
    def boom(job):
        if job.name == "J1":
            raise ValueError("bad board")
        return {}
    srv = RouteServer(slots=2, executor=boom, footprint=lambda j: 1)
    res = [f.result(timeout=10) for f in [srv.submit(j) for j in _jobs(3)]]
    srv.close()
    assert [r.error is None for r in res] == [True, False, True]


def test_stream_of_arrivals_reports_latency_percentiles():
    jobs = _jobs(12)
    for j, t in zip(jobs, poisson_arrivals(len(jobs), 200.0, seed=7)):
        j.arrival = float(t)
    srv = RouteServer(slots=4, executor=_Probe(0.02), footprint=lambda j: 1)
    out = srv.run_stream(jobs)
    srv.close()
    assert out["errors"] == 0 and len(out["results"]) == 12
    assert 0.0 < out["p50_s"] <= out["p99_s"] and out["jobs_per_s"] > 0


def test_footprint_grows_with_the_board():
    small = job_footprint(100, 100, 6, 279_200, 200)
    big = job_footprint(600, 400, 12, 21_110_000, 2000)
    assert 0 < small < big < 160 * (1 << 30)
