"""Serving loop: continuous batching of routing jobs on one GB300.

Jobs (a lattice, its requests and an iteration cap) arrive over time.  The
server admits a waiting job as soon as a job slot is free and the job's HBM
footprint fits the budget next to the jobs already running.  Each admitted
job gets a worker thread, its own CUDA stream and its own device-resident
router state (CSR, congestion arrays, path store and workspaces) for the
whole job, so jobs overlap on the device: one job's kernels run while
another job's host policy runs (the ctypes calls release the interpreter
lock), single-CTA kernels of different jobs share the SMs, and each job's
whole-lattice searches use a 1/slots share of the resident CTAs, so the
cooperative searches of concurrent jobs fit on the GPU together.  Every
kernel is deterministic, so a job's result is the same alone and in the mix.

The reference has no serving loop; its unit of work is one
``route_multiple_nets`` call, which is what a job runs.
"""
from __future__ import annotations

import heapq
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np


@dataclass
class RouteJob:
    """One routing job: a lattice (nx, ny, nz and the allowed via spans), its
    board bounds, the requests and the negotiation iteration cap."""
    name: str
    nx: int
    ny: int
    nz: int
    requests: Sequence[Tuple[str, int, int]]
    max_iterations: int = 40
    bounds: Optional[Tuple[float, float, float, float]] = None
    allowed_via_spans: Optional[Sequence[Tuple[int, int]]] = None
    arrival: float = 0.0          # seconds after the server start (used by run_stream)
    ors_path: Optional[str] = None  # when set, the job's solution is also written there as .ORS


@dataclass
class JobResult:
    name: str
    arrival: float
    admitted: float
    finished: float
    result: Dict = field(default_factory=dict)
    error: Optional[str] = None

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def job_footprint(nx: int, ny: int, nz: int, num_edges: int, num_nets: int, window_slots: int = 32,
                  max_roi_nodes: int = 50_000, slot_cap: int = 8192, bfs_slots: int = 64) -> int:
    """HBM bytes of one job's device state (the allocations of a router):
    CSR, congestion arrays, search workspaces, path store, ROI pool."""
    N, E = nx * ny * nz, int(num_edges)
    R = min(max_roi_nodes, N)
    csr = 4 * (N + 1) + E * (4 + 4 + 1 + 1 + 4 + 4)
    state = E * 4 * 7 + N * 4 * 4 + 4 * nz
    roi_ws = 72 * N + 2 * 4 * min(N, 65536) * 32 + 4 * min(N, 65536)
    full_ws = 44 * N + 4 * E
    qcap = min(N, max(4 * max_roi_nodes, 1 << 18))
    bfs = min(bfs_slots, max(1, num_nets)) * (4 * N + 4 * 4 * qcap)
    window = window_slots * (4 * N + 48 * R + 8 * min(R, 65536) * 32 + slot_cap * 4)
    store = num_nets * (slot_cap * 12 + R * 4 + 24)
    return int(csr + state + roi_ws + full_ws + bfs + window + store + (64 << 20))


def _percentile(v: List[float], q: float) -> float:
    if not v:
        return float("nan")
    return float(np.percentile(np.asarray(v, dtype=np.float64), q))


class RouteServer:
    """Admits jobs into at most `slots` concurrent workers under an HBM budget.

    ``submit(job)`` returns a Future of a JobResult.  ``executor(job)`` runs a
    job and returns its result dict; the default builds a PathFinderRouter on
    the worker's own CUDA stream (tests substitute a host-only executor)."""

    def __init__(self, slots: int = 4, hbm_budget_bytes: int = 160 * (1 << 30), device: str = "cuda",
                 window_slots: int = 32, executor: Optional[Callable[[RouteJob], Dict]] = None,
                 footprint: Optional[Callable[[RouteJob], int]] = None, sm_share: bool = True):
        self.slots = max(1, int(slots))
        self.sm_share = bool(sm_share)
        self.budget = int(hbm_budget_bytes)
        self.device = device
        self.window_slots = int(window_slots)
        self.executor = executor or self._run_on_gpu
        self.footprint = footprint or self._footprint
        self._lock = threading.Condition()
        self._queue: List[Tuple[float, int, RouteJob, Future]] = []
        self._seq = 0
        self._running = 0
        self._used = 0
        self._threads: List[threading.Thread] = []
        self._closed = False
        self.t0 = time.perf_counter()
        self.peak_running = 0
        self.peak_bytes = 0
        self._sched = threading.Thread(target=self._schedule, daemon=True)
        self._sched.start()

    # -- sizing -------------------------------------------------------------------
    def _footprint(self, job: RouteJob) -> int:
        from .lattice import Lattice
        lat = Lattice(job.nx, job.ny, job.nz, allowed_via_spans=job.allowed_via_spans)
        E = _num_edges(lat)
        return job_footprint(job.nx, job.ny, job.nz, E, len(job.requests), self.window_slots)

    # -- API ----------------------------------------------------------------------
    def now(self) -> float:
        return time.perf_counter() - self.t0

    def submit(self, job: RouteJob) -> Future:
        fut: Future = Future()
        need = self.footprint(job)
        if need > self.budget:
            fut.set_exception(MemoryError(f"job {job.name} needs {need} B of HBM, budget is {self.budget} B"))
            return fut
        with self._lock:
            if self._closed:
                raise RuntimeError("server closed")
            arrival = self.now()
            heapq.heappush(self._queue, (arrival, self._seq, job, fut))
            self._seq += 1
            job._need = need           # noqa: SLF001
            job._arrival_abs = arrival   # noqa: SLF001
            self._lock.notify_all()
        return fut

    def close(self, wait: bool = True):
        with self._lock:
            self._closed = True
            self._lock.notify_all()
        if wait:
            self._sched.join()
            for t in list(self._threads):
                t.join()

    # -- scheduling ---------------------------------------------------------------
    def _schedule(self):
        while True:
            with self._lock:
                while True:
                    head = self._queue[0] if self._queue else None
                    fits = head is not None and self._running < self.slots and \
                        self._used + head[2]._need <= self.budget
                    if fits or (self._closed and not self._queue):
                        break
                    self._lock.wait(timeout=0.05)
                if head is None or not fits:
                    return
                _, _, job, fut = heapq.heappop(self._queue)
                self._running += 1
                self._used += job._need
                self.peak_running = max(self.peak_running, self._running)
                self.peak_bytes = max(self.peak_bytes, self._used)
                t = threading.Thread(target=self._work, args=(job, fut), daemon=True)
                self._threads.append(t)
                t.start()

    def _work(self, job: RouteJob, fut: Future):
        admitted = self.now()
        res = JobResult(job.name, job._arrival_abs, admitted, admitted)
        try:
            res.result = self.executor(job)
        except Exception as e:  # reported through the future, the server keeps running
            res.error = f"{type(e).__name__}: {e}"
        res.finished = self.now()
        with self._lock:
            self._running -= 1
            self._used -= job._need
            self._lock.notify_all()
        fut.set_result(res)

    def _run_on_gpu(self, job: RouteJob) -> Dict:
        import torch
        from .lattice import Lattice
        from .router import PathFinderConfig, PathFinderRouter
        stream = torch.cuda.Stream(device=self.device)
        with torch.cuda.device(self.device), torch.cuda.stream(stream):
            if self.sm_share:
                # this job's whole-lattice searches take a 1/slots share of the
                # resident CTAs (the grid knob is per host thread), so
                # cooperative searches of concurrent jobs fit on the GPU together
                from .autotune import full_grid
                _, limit = full_grid(0)
                full_grid(max(1, limit // self.slots))
            r = PathFinderRouter(PathFinderConfig(max_iterations=job.max_iterations), device=self.device,
                                 window_slots=self.window_slots)
            r.initialize_lattice(Lattice(job.nx, job.ny, job.nz, allowed_via_spans=job.allowed_via_spans),
                                 job.bounds)
            t0 = time.perf_counter()
            out = r.route_multiple_nets(list(job.requests))
            stream.synchronize()
            if job.ors_path:
                write_job_ors(r, out, job.name, job.ors_path, time.perf_counter() - t0)
        return {"paths": {k: list(v) for k, v in out["paths"].items()},
                **{k: out.get(k) for k in ("success", "converged", "iterations", "overuse_sum",
                                           "barrel_conflicts", "failed_nets")}}

    # -- streams of arrivals --------------------------------------------------------
    def run_stream(self, jobs: Sequence[RouteJob]) -> Dict:
        """Submit every job at its `arrival` time (seconds from now) and wait
        for all: per-job results plus p50 / p99 latency and jobs per second."""
        start = self.now()
        futs = []
        for job in sorted(jobs, key=lambda j: j.arrival):
            delay = start + job.arrival - self.now()
            if delay > 0:
                time.sleep(delay)
            futs.append(self.submit(job))
        results = [f.result() for f in futs]
        lat = [r.latency for r in results if r.error is None]
        span = max(r.finished for r in results) - start if results else 0.0
        return {"results": results, "p50_s": _percentile(lat, 50), "p99_s": _percentile(lat, 99),
                "jobs_per_s": (len(results) / span) if span > 0 else float("nan"),
                "errors": sum(r.error is not None for r in results),
                "peak_concurrent": self.peak_running, "peak_hbm_bytes": self.peak_bytes}


def write_job_ors(router, result: Dict, name: str, path: str, seconds: float) -> None:
    """The job's geometry, per-iteration metrics and outcome as a .ORS file
    (the layout of the reference's headless export, main.py:594-662)."""
    from .ors import export_solution_to_ors
    router.emit_geometry()
    metrics = [{"iteration": m.get("iter", 0), "overuse": m.get("overuse_edges", 0),
                "nets_routed": m.get("nets_routed", 0), "overflow": m.get("overuse_sum", 0),
                "time": m.get("iter_time_s", 0.0)} for m in result.get("iteration_metrics", [])]
    metadata = {"total_iterations": result.get("iterations", len(metrics)), "converged": bool(result.get("converged")),
                "total_time": seconds, "nets_routed": result.get("nets_routed", 0), "board_name": name,
                "notes": f"barrel_conflicts={result.get('barrel_conflicts', 0)} failed_nets={result.get('failed_nets', 0)}"}
    export_solution_to_ors(router.get_geometry_payload(), metrics, metadata, path, compress=True)


def _num_edges(lat) -> int:
    import ctypes as C
    from . import _lib
    desc, keep = lat.descriptor()
    E = C.c_int64(0)
    _lib.check(_lib.load().ogr_csr_num_edges(C.byref(desc), C.byref(E)), "ogr_csr_num_edges")
    del keep
    return int(E.value)


def poisson_arrivals(n: int, rate_per_s: float, seed: int) -> np.ndarray:
    """Arrival times of a seeded Poisson process (exponential gaps)."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate_per_s, size=n))
