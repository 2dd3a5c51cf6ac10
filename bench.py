"""Benchmark: PathFinder time-to-zero-overuse and SSSP GTEPS on one GB300.

A step is one complete negotiated-congestion routing job over a seeded
synthetic board: build the congestion state, run the negotiation loop until
the reference's success predicate holds or the iteration cap is reached, and
return every path.  ``value`` is seconds per job with the lattice CSR already
resident in HBM; ``e2e`` is the same job through the public router API
starting from host requests (CSR build, state upload and the path read-back
inside the timed region).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--config c1|c0|c2|c4]
                    [--impl ours|reference]

``--impl reference`` times the CPU restatement of the reference's routing
path (the oracle with its C heap Dijkstra) on the host cores, on a bounded
sample of the same job.  Under torchrun only rank 0 reports; the other ranks
route independent replicas (a route job does not shard).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

CONFIGS = {
    # the CPU-runnable case: 100x100x6, 200 two-pin nets on layer 0, length 5-80, 10 iterations
    "c0": dict(nx=100, ny=100, nz=6, nets=200, iters=10, seed=1234, clusters=False, plain_iters=None),
    # the headline case: 600x400x12, 2,000 nets, 30% from two 20x20 clusters, <= 40 iterations
    # plain_iters: the plain one-net-per-launch form is compared with the batched form on the
    # job's first iterations (all nets, same search engine)
    "c1": dict(nx=600, ny=400, nz=12, nets=2000, iters=40, seed=4321, clusters=True, via_span=4,
               plain_iters=3,
               # DRAM bytes / algorithmic bytes of full_sssp_kernel, ncu on a 300x200x8 search
               traffic_ratio=0.6655),
    # multi-pin batching: 600x400x12, 1,500 multi-pin nets (2-16 pins, 1 + geometric(0.35)) with
    # pins inside a seeded 50x50 box per net, as star two-pin requests p0 -> pi (multipin.py)
    "c2": dict(nx=600, ny=400, nz=12, nets=1500, iters=40, seed=2468, multipin=True, via_span=4,
               plain_iters=3),
    # BGA escape + backplane: 1000x800x32 (25.6 M nodes; 32 layers allow adjacent vias only), a 40x40
    # BGA at 1 mm (2.5 cells) in the centre and four edge-connector rows; reconciled to 1,600 BGA
    # escape nets (ball -> seeded-random connector pin) + 3,200 backplane nets pairing the other
    # 6,400 connector pins, every pin used once (bga_requests); iterations capped for a run
    "c3": dict(nx=1000, ny=800, nz=32, nets=4800, iters=2, seed=1357, bga=True,
               plain_iters=None),
}


# serving stream: jobs arrive as a seeded Poisson process; each job's board is
# one of three sizes with nets generated as in c0 (100x100x6) or c1 (larger)
SERVE = dict(jobs=256, rate=4.0, seed=99, slots=4, budget_gb=160,
             sizes=[dict(nx=100, ny=100, nz=6, nets=200, iters=10, clusters=False),
                    dict(nx=300, ny=200, nz=8, nets=800, iters=40, clusters=True, via_span=4),
                    dict(nx=600, ny=400, nz=12, nets=2000, iters=40, clusters=True, via_span=4)])


def serve_jobs(n_jobs, iter_cap=None):
    """The first n_jobs of the seeded serving stream (arrival times, boards, nets)."""
    from orthoroute_gb300.serve import RouteJob, poisson_arrivals
    arr = poisson_arrivals(SERVE["jobs"], SERVE["rate"], SERVE["seed"])
    rng = np.random.default_rng(SERVE["seed"] + 1)
    kinds = rng.integers(0, len(SERVE["sizes"]), size=SERVE["jobs"])
    jobs = []
    for i in range(n_jobs):
        size = dict(SERVE["sizes"][int(kinds[i])])
        size["seed"] = int(SERVE["seed"] * 1000 + i)
        its = size["iters"] if iter_cap is None else min(size["iters"], iter_cap)
        jobs.append(RouteJob(f"job{i}", size["nx"], size["ny"], size["nz"], make_requests(size),
                             max_iterations=its, bounds=board_bounds(size["nx"], size["ny"]),
                             allowed_via_spans=via_spans(size), arrival=float(arr[i])))
    return jobs


def via_spans(cfg):
    """allowed_via_spans of the lattice: the reference's default legal via
    pairs (layers 0..Nz-2, Lattice3D.get_legal_via_pairs) whose span |dz|
    (unified_pathfinder.py:1872) is at most via_span; None = all legal pairs."""
    k = cfg.get("via_span")
    if k is None:
        return None
    from orthoroute_gb300 import Lattice
    return [(a, b) for a, b in Lattice(2, 2, cfg["nz"]).via_pairs() if b - a <= k]


def make_lattice(cfg):
    from orthoroute_gb300 import Lattice
    return Lattice(cfg["nx"], cfg["ny"], cfg["nz"], allowed_via_spans=via_spans(cfg))


def make_requests(cfg):
    """Seeded two-pin nets with endpoints on layer 0 (numpy default_rng); for a
    multi-pin config, the star requests of seeded multi-pin nets."""
    nx, ny, n = cfg["nx"], cfg["ny"], cfg["nets"]
    if cfg.get("multipin"):
        from orthoroute_gb300.multipin import seeded_multipin_nets, star_requests
        return star_requests(seeded_multipin_nets(nx, ny, n, cfg["seed"]))
    if cfg.get("bga"):
        return bga_requests(nx, ny, cfg["seed"])
    rng = np.random.default_rng(cfg["seed"])
    out = []
    if not cfg["clusters"]:
        while len(out) < n:
            x0, x1 = rng.integers(0, nx, size=2)
            y0, y1 = rng.integers(0, ny, size=2)
            d = abs(int(x1) - int(x0)) + abs(int(y1) - int(y0))
            if 5 <= d <= 80:
                out.append((f"N{len(out)}", int(y0) * nx + int(x0), int(y1) * nx + int(x1)))
        return out
    centres = [(int(rng.integers(20, nx - 40)), int(rng.integers(20, ny - 40))) for _ in range(2)]
    n_cluster = int(round(0.3 * n))
    while len(out) < n:
        if len(out) < n_cluster:
            cx, cy = centres[len(out) % 2]
            x0, y0 = cx + int(rng.integers(0, 20)), cy + int(rng.integers(0, 20))
        else:
            x0, y0 = int(rng.integers(0, nx)), int(rng.integers(0, ny))
        x1, y1 = int(rng.integers(0, nx)), int(rng.integers(0, ny))
        if (x0, y0) == (x1, y1):
            continue
        out.append((f"N{len(out)}", y0 * nx + x0, y1 * nx + x1))
    return out


def connector_pins(nx, ny, per_row=2000):
    """Four edge-connector rows of per_row pins on layer 0: the top and bottom
    rows fill two cell rows along their edge, the left and right rows three
    cell columns (evenly spread)."""
    rows = []
    for y0 in (0, ny - 2):                       # top / bottom: 2 x nx cells
        cells = [(x, y0 + d) for x in range(nx) for d in range(2)]
        rows.append(cells)
    for x0 in (0, nx - 3):                       # left / right: 3 x ny cells
        cells = [(x0 + d, y) for y in range(2, ny - 2) for d in range(3)]
        rows.append(cells)
    pins = []
    for cells in rows:
        idx = np.linspace(0, len(cells) - 1, per_row).round().astype(int)
        pins.extend(cells[i] for i in idx)
    return [y * nx + x for x, y in pins]


def bga_requests(nx, ny, seed, balls=40, pitch_cells=2.5):
    """c3's nets (see CONFIGS): BGA escapes then backplane pairs, seeded."""
    rng = np.random.default_rng(seed)
    cx, cy = nx / 2.0, ny / 2.0
    off = (balls - 1) / 2.0
    bga = [int(round(cy + (j - off) * pitch_cells)) * nx + int(round(cx + (i - off) * pitch_cells))
           for j in range(balls) for i in range(balls)]
    conn = connector_pins(nx, ny)
    perm = rng.permutation(len(conn))
    out = [(f"B{k}", bga[k], conn[perm[k]]) for k in range(len(bga))]
    rest = perm[len(bga):]
    for k in range(len(rest) // 2):
        out.append((f"P{k}", conn[rest[2 * k]], conn[rest[2 * k + 1]]))
    return out


def workload_config(name, cfg):
    """The workload as both arms print it."""
    return {"workload": name, "lattice": [cfg["nx"], cfg["ny"], cfg["nz"]], "nets": cfg["nets"],
            "max_iterations": cfg["iters"]}


def trajectory_fixture(name):
    """The oracle's committed trajectory of a workload (per-iteration path
    fingerprints, searches, wall time of the CPU run), or None."""
    path = os.path.join(ROOT, "tests", "golden", f"{name}_trajectory.json.gz")
    if not os.path.exists(path):
        return None
    from orthoroute_gb300.trajectory import load
    return load(path)


def host_cpu():
    """Model and online cores of the host CPU."""
    model = None
    try:
        r = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10)
        for ln in r.stdout.splitlines():
            if ln.split(":")[0].strip() in ("Model name", "Model"):
                model = ln.split(":", 1)[1].strip()
                if ln.startswith("Model name"):
                    break
    except Exception:
        pass
    return {"model": model, "nproc": os.cpu_count()}


def board_bounds(nx, ny, pitch=0.4):
    sx = (nx - 1) * pitch - 6.0 + 1e-6
    sy = (ny - 1) * pitch - 6.0 + 1e-6
    return (7.0, 7.0, 10.0 + sx + 3.0, 10.0 + sy + 3.0)


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons while running."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        def run():
            while not self._stop.is_set():
                try:
                    r = subprocess.run(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                        "-i", os.environ.get("LOCAL_RANK", "0")],
                                       capture_output=True, text=True, timeout=5)
                    if r.returncode == 0 and r.stdout.strip():
                        self.rows.append([c.strip() for c in r.stdout.strip().split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)
        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=6)
        sm = [float(r[0]) for r in self.rows if r[0].replace('.', '', 1).isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace('.', '', 1).isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if len(r) > 3 + i and r[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# ----------------------------------------------------------------- replicas
def replica_max(ms: float, device: str) -> float:
    """Max over ranks of one replica's time per job (a route job does not
    shard: every rank routes its own copy, with no exchange on the data path)."""
    import torch
    import torch.distributed as tdist
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def replica_value(ms: float, world: int) -> float:
    """Whole-job throughput of N replicas expressed in the metric's unit
    (seconds per job): N jobs finish every `ms`."""
    return ms / 1e3 / max(1, world)


# --------------------------------------------------------------------- our arm
def run_ours(args, cfg, rank, world):
    import ctypes as C

    import torch
    from orthoroute_gb300 import _lib
    from orthoroute_gb300.router import PathFinderConfig, PathFinderRouter

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    reqs = make_requests(cfg)
    nx, ny, nz = cfg["nx"], cfg["ny"], cfg["nz"]
    bounds = board_bounds(nx, ny)

    def job(router):
        router.config = PathFinderConfig(max_iterations=cfg["iters"])
        router.initialize_state()
        return router.route_multiple_nets(reqs)

    router = PathFinderRouter(PathFinderConfig(max_iterations=cfg["iters"]), mode=args.mode,
                              full_engine=args.full_engine)
    router.initialize_lattice(make_lattice(cfg), bounds)
    parity = None
    for w in range(args.warmup):
        fixture = trajectory_fixture(args.config) if w == 0 else None
        if fixture is not None:
            # the first warm-up job is fingerprinted (untimed) against the oracle's run
            from orthoroute_gb300.trajectory import TrajectoryRecorder, first_difference
            router.trace = TrajectoryRecorder()
            job(router)
            diff = first_difference(router.trace.records, fixture["records"])
            parity = {"oracle_trajectory": f"tests/golden/{args.config}_trajectory.json.gz",
                      "iterations_compared": len(fixture["records"]),
                      "paths_match_every_iteration": diff is None,
                      "first_difference": None if diff is None else {"record": diff[0], "nets": diff[1]}}
            router.trace = None
        else:
            job(router)
    dist = world > 1
    if dist:
        import torch.distributed as tdist
        tdist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler()
    sampler.start()
    router.profile_reset()
    full_prof = (C.c_int64 * 8)()
    _lib.check(_lib.load().ogr_full_profile(full_prof, 1), "ogr_full_profile")   # reset the in-kernel counters
    start_ev = torch.cuda.Event(enable_timing=True)
    end_ev = torch.cuda.Event(enable_timing=True)
    start_ev.record()
    t0 = time.perf_counter()
    results = []
    for _ in range(args.steps):
        results.append(job(router))
    end_ev.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    dev_ms = start_ev.elapsed_time(end_ev)
    clocks = sampler.stop()
    prof = router.profile_snapshot()
    # whole-lattice searches: count, settle phases and in-kernel time (globaltimer, CTA 0)
    _lib.check(_lib.load().ogr_full_profile(full_prof, 1), "ogr_full_profile")
    full_n, full_phases, full_ns = int(full_prof[0]), int(full_prof[1]), int(full_prof[2])
    # end-to-end through the public API from host requests (fresh CSR build + state + read-back)
    e2e_t = []
    for _ in range(max(1, min(args.steps, 2))):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        r2 = PathFinderRouter(PathFinderConfig(max_iterations=cfg["iters"]), mode=args.mode,
                              full_engine=args.full_engine)
        r2.initialize_lattice(make_lattice(cfg), bounds)
        res2 = r2.route_multiple_nets(reqs)
        _ = {k: list(v) for k, v in res2["paths"].items()}
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t1)
        del r2
    plain = None
    if args.mode == "persistent" and args.compare_plain:
        # plain form: one launch per net with a host round trip per net, the same search engine
        # and tuning as the batched form; compared on the whole job, or on its first
        # iterations (all nets) for the large boards
        k_it = cfg.get("plain_iters") or cfg["iters"]
        preqs = reqs
        whole = k_it == cfg["iters"]

        def timed(r, iters):
            r.config = PathFinderConfig(max_iterations=iters)
            r.initialize_state()
            torch.cuda.synchronize()
            t = time.perf_counter()
            out = r.route_multiple_nets(preqs)
            torch.cuda.synchronize()
            return time.perf_counter() - t, out

        rp = PathFinderRouter(PathFinderConfig(max_iterations=k_it), mode="plain", full_engine=args.full_engine)
        rp.initialize_lattice(make_lattice(cfg), bounds)
        t_plain, resp = timed(rp, k_it)
        del rp
        if whole:
            t_batched, resb = None, results[-1]
        else:
            t_batched, resb = timed(router, k_it)
        same = {k: list(v) for k, v in resp["paths"].items()} == {k: list(v) for k, v in resb["paths"].items()}
        plain = {"iterations": k_it, "nets": len(preqs), "plain_s": round(t_plain, 4), "identical_paths": bool(same),
                 "engine": "same as the batched form (" + str(router.full_engine) +
                           (", tile windows" if getattr(router, "full_tile_delta", 0) else "") + ")"}
        if t_batched is not None:
            plain["batched_s"] = round(t_batched, 4)
    ms = max(dev_ms, wall * 1e3) / args.steps
    if dist:
        ms = replica_max(ms, "cuda")
    res = results[-1]
    pk, pk_kind = peaks()
    search_ms = prof["search_kernel_ms"]
    launches = prof["search_launches"]
    alg_bytes = prof["arcs"] * 24 + prof["pops"] * 20
    achieved = (alg_bytes / launches) / (search_ms / launches * 1e-3) / 1e9 if launches and search_ms > 0 else 0.0
    gteps = prof["arcs"] / (search_ms * 1e-3) / 1e9 if search_ms > 0 else 0.0
    line = {
        "metric": "PathFinder time-to-zero-overuse (s per routing job; capped iterations when not converged)",
        "value": round(replica_value(ms, world), 6),
        "unit": "s/job",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": False, "scaling": "weak" if world > 1 else "weak",
        "vs_baseline": None, "dtype": "f32 costs / f64 labels / int32 indices",
        "data": "synthetic seeded board (seeded nets of the named workload; no dataset)",
        "config": workload_config(args.config, cfg),
        "workload_info": {"arcs": router.E, "nodes": router.N,
                          "replicas": "independent per rank" if world > 1 else "single",
                          "l2": "working set per search < L2; no flush (searches are latency-bound)"},
        "result": {k: res.get(k) for k in ("success", "converged", "iterations", "overuse_sum", "barrel_conflicts",
                                           "failed_nets")},
        "sssp_gteps": round(gteps, 4),
        # device time of the search launches (CUDA events on the routing stream) vs the whole job
        "time_split": {"search_kernels_s": round(search_ms / 1e3 / max(1, args.steps), 3),
                       # wall time of the routing passes (launch to sync) and everything else: the host
                       # negotiation policy, tallies, cost updates and their transfers
                       "routing_passes_s": round(prof["search_wall_s"] / max(1, args.steps), 3),
                       "host_policy_and_rest_s": round((ms / 1e3) - prof["search_wall_s"] / max(1, args.steps), 3),
                       "job_s": round(ms / 1e3, 3),
                       # of the search kernels: the whole-lattice searches (in-kernel clock) and their phases
                       "whole_lattice_searches_s": round(full_ns / 1e9 / max(1, args.steps), 3),
                       "whole_lattice_searches": full_n // max(1, args.steps),
                       "phases_per_whole_lattice_search": round(full_phases / max(1, full_n), 1),
                       "us_per_phase": round(full_ns / 1e3 / max(1, full_phases), 3)},
        "searches_per_job": prof["searches"] // max(1, args.steps),
        # window searches whose results were undone (an earlier member of their window failed);
        # their nets were searched again and that search is the one counted above
        "discarded_window_searches_per_job": prof["discarded_searches"] // max(1, args.steps),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 3), "peak": pk.get("hbm_gbs"), "unit": "GB/s",
                     "frac": round(achieved / pk.get("hbm_gbs", 1.0), 6),
                     "traffic": (round(cfg["traffic_ratio"] * alg_bytes / max(1, prof["searches"])) if
                                 cfg.get("traffic_ratio") else None),
                     "traffic_unit": "bytes per search (ncu DRAM bytes of full_sssp_kernel on a smaller "
                                     "lattice, scaled by the algorithmic bytes)" if cfg.get("traffic_ratio")
                                     else None,
                     "kernel": "search launches of the routing pass (full_sssp_kernel on all SMs for "
                               "full-graph nets, route_pass_kernel / roi_batch_kernel for ROI nets)",
                     "peak_kind": pk_kind,
                     "algorithmic_bytes": "24 B per arc scanned + 20 B per node popped by the sequential search"},
        "e2e": {"value": round(float(np.median(e2e_t)), 6), "unit": "s/job",
                "h2d_bytes_per_step": prof["h2d_bytes"] // max(1, args.steps),
                "d2h_bytes_per_step": prof["d2h_bytes"] // max(1, args.steps)},
        "gpu_launches": prof["launches"] // max(1, args.steps),
        "clocks": clocks,
        "mode": args.mode,
        "full_engine": {"requested": args.full_engine, "used": router.full_engine,
                        "tuning": (None if router.tuning is None else
                                   {"ctas": router.tuning.full_ctas, "full_lanes": router.tuning.full_lanes,
                                    "full_reuse": router.tuning.full_reuse,
                                    "roi_lanes": router.tuning.roi_lanes,
                                    "ms_per_search": router.tuning.ms_per_search,
                                    "cached": router.tuning.cached})},
    }
    if parity is not None:
        line["parity"] = parity
    if plain is not None:
        if "batched_s" not in plain:
            plain["batched_s"] = round(ms / 1e3, 4)
        plain["speedup"] = round(plain["plain_s"] / max(plain["batched_s"], 1e-9), 3)
        line["plain_one_net_per_launch"] = plain
    return line


# ---------------------------------------------------------------- CPU baseline
class CpuSample:
    """The CPU restatement of the reference's routing path (the oracle with its
    C heap Dijkstra), timed on this host's cores on a bounded, stratified
    sample of a workload.

    Boards of up to 400 nets route the whole job.  Larger boards: the first
    step routes one stratified chunk of nets through a whole negotiation
    iteration (the host policy's time per iteration is that step's time minus
    its searches); every later step routes the next chunk through the
    routing pass alone (rip-up, search, commit), timing searches.  The job
    time is the time per search x the searches of the whole job plus the
    policy time x its iterations, both counts taken from the oracle's own
    run of the same job (its committed trajectory) when there is one."""

    def __init__(self, name, cfg, chunk=3):
        from oracle.lattice import LatticeSpec
        from oracle.loop import Config, OracleRouter
        self.name, self.cfg = name, cfg
        reqs = make_requests(cfg)
        self.tasks = {n: (a, b) for n, a, b in reqs if a != b}
        nx, ny, nz = cfg["nx"], cfg["ny"], cfg["nz"]
        self.small = cfg["nets"] <= 400
        self.R = OracleRouter(LatticeSpec(nx, ny, nz, allowed_via_spans=via_spans(cfg)), board_bounds(nx, ny),
                              Config(max_iterations=cfg["iters"] if self.small else 1), fast=True)
        find = self.R._find
        self.search_s = 0.0

        def timed_find(*a, **k):
            t = time.perf_counter()
            try:
                return find(*a, **k)
            finally:
                self.search_s += time.perf_counter() - t
        self.R._find = timed_find
        # stratified order: every net of the name order, interleaved from evenly spaced starts
        names = list(self.tasks)
        stride = 40
        self.order = [names[i] for off in range(stride) for i in range(off, len(names), stride)]
        self.chunk = chunk
        self.pos = 0
        self.policy_s = None
        self.timed_searches = 0
        self.timed_search_s = 0.0
        self.full_job_s = None

    def step(self):
        if self.small:
            self.R = self.R.__class__(self.R.spec, self.R.bounds, self.R.cfg.__class__(max_iterations=self.cfg["iters"]),
                                      fast=True)
            t = time.perf_counter()
            res = self.R.route(self.tasks)
            self.full_job_s = time.perf_counter() - t
            self.small_desc = f"full job ({res['iterations']} iterations, {self.R.stats['searches']} searches)"
            return
        sub_names = self.order[self.pos:self.pos + self.chunk]
        self.pos = (self.pos + self.chunk) % max(1, len(self.order))
        sub = {n: self.tasks[n] for n in sub_names}
        s0, n0 = self.search_s, self.R.stats["searches"]
        t = time.perf_counter()
        if self.policy_s is None:
            self.R.route(sub)                                  # one whole iteration
            self.policy_s = (time.perf_counter() - t) - (self.search_s - s0)
        else:
            self.R._route_all(sub, self.tasks)                 # the routing pass alone
        self.timed_searches += self.R.stats["searches"] - n0
        self.timed_search_s += self.search_s - s0

    def estimate(self, gpu_counts=None):
        """(s per job, description)."""
        if self.small:
            return self.full_job_s, self.small_desc
        fx = trajectory_fixture(self.name)
        if fx is not None:
            searches, iters = fx["searches"], fx["result"]["iterations"]
            src = f"the oracle's own run of the job: {searches} searches, {iters} iterations"
        elif gpu_counts:
            searches, iters = gpu_counts
            src = f"this GPU run of the bit-identical job: {searches} searches, {iters} iterations"
        else:
            # no measured count: later iterations reroute an unmeasured subset of the nets, so
            # only the first iteration's searches (every net once) are counted -- a lower bound
            searches, iters = len(self.tasks), self.cfg["iters"]
            src = ("no measured count: the first iteration's searches only (every net once), a lower bound "
                   "of the job's searches")
        per = self.timed_search_s / max(1, self.timed_searches)
        v = per * searches + (self.policy_s or 0.0) * iters
        return v, (f"stratified sample of iteration 1: {self.timed_searches} searches ({per:.3f} s each) and one "
                   f"iteration's host policy ({self.policy_s:.1f} s), scaled by {src}")


def cpu_job_sample(name, cfg, steps=8, gpu_counts=None):
    cs = CpuSample(name, cfg)
    for _ in range(1 if cs.small else steps):
        cs.step()
    v, desc = cs.estimate(gpu_counts)
    return v, desc, 1


def run_reference(args, cfg):
    """The reference arm: the oracle (the CPU restatement of the reference's
    routing path, pinned to its own runs) on this host's cores.  Warm-up
    steps route chunks untimed; each timed step is one more stratified chunk
    (see CpuSample)."""
    cs = CpuSample(args.config, cfg)
    t_steps = []
    for i in range(args.warmup + args.steps):
        t = time.perf_counter()
        cs.step()
        if i >= args.warmup:
            t_steps.append(time.perf_counter() - t)
        if cs.small and i >= args.warmup:
            break
    v, desc = cs.estimate()
    fx = trajectory_fixture(args.config)
    cpu = {"value": round(v, 4), "unit": "s/job", "cores": 1, "kind": "port", "sample": desc,
           "host_cpu": host_cpu()}
    if fx is not None and fx.get("wall_s"):
        cpu["full_job_measured_on_build_host_s"] = fx["wall_s"]
    return {"metric": "PathFinder time-to-zero-overuse (s per routing job; capped iterations when not converged)",
            "value": round(v, 4), "unit": "s/job", "impl": "reference", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": False,
            "config": workload_config(args.config, cfg),
            "cpu_baseline": cpu,
            "e2e": {"value": round(v, 4), "unit": "s/job", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_engine_compare(args):
    """Whole-lattice searches on one lattice with uncongested costs (base 0.12
    plus the reference's index jitter), timed per engine: the phase-settled
    search and the tile-window search at several window widths.  The paths
    must be identical; the line gives ms per search and the engines' own
    counters (phases / grid rounds, windows, per-stage time)."""
    import ctypes as C
    import torch
    from orthoroute_gb300 import Lattice, _lib, autotune
    from orthoroute_gb300.device import DeviceGraph, DeviceState, Ops
    cfg = CONFIGS[args.config]
    if args.lattice:
        nx, ny, nz = (int(v) for v in args.lattice.lower().split("x"))
        lat = Lattice(nx, ny, nz, allowed_via_spans=[(a, b) for a, b in Lattice(2, 2, nz).via_pairs() if b - a <= 4])
    else:
        lat = make_lattice(cfg)
    g = DeviceGraph(lat)
    s = DeviceState(g)
    s.enable_rcost()
    ops = Ops(g, s)
    jit = (np.arange(g.E) % 9973).astype(np.float32) * np.float32(1e-6)
    s.total_cost.copy_(torch.from_numpy((np.float32(0.12) + jit).astype(np.float32)))
    ops.sync_rcost()
    nx, ny = lat.nx, lat.ny
    rng = np.random.default_rng(5)
    pairs = [(5 + (ny // 10) * nx, nx * ny - 7 - (ny // 13) * nx)]
    pairs += [(int(rng.integers(0, nx * ny)), int(rng.integers(0, nx * ny))) for _ in range(2)]

    def prof(fn, n):
        out = (C.c_int64 * n)()
        _lib.check(getattr(_lib.load(), fn)(out, 1), fn)
        return list(out)

    engines = [("phase", 0.0)] + [(f"tile_delta{d}", d) for d in (0.5, 1.0, 2.0, 4.0)]
    res = {}
    paths = {}
    for name, delta in engines:
        autotune.full_tile(1 if delta else 0, delta)
        ops.find_path(ops.net_args(0, pairs[0][0], pairs[0][1], full_graph=True, penalty=False), engine="grid")
        prof("ogr_full_profile", 8)
        prof("ogr_tile_profile", 24)
        torch.cuda.synchronize()
        t0 = ops.counters["search_ms"]
        got = [ops.find_path(ops.net_args(0, a, b, full_graph=True, penalty=False), engine="grid") for a, b in pairs]
        ms = (ops.counters["search_ms"] - t0) / len(pairs)
        fp, tp = prof("ogr_full_profile", 8), prof("ogr_tile_profile", 24)
        paths[name] = got
        r = {"ms_per_search": round(ms, 3)}
        if delta:
            r.update(rounds=tp[1] // len(pairs), windows=tp[2] // len(pairs), handed_over=tp[4],
                     stage_ns_per_cta={"structure": tp[8] // len(pairs), "labels": tp[9] // len(pairs),
                                       "iterations": tp[10] // len(pairs), "write_back": tp[11] // len(pairs),
                                       "barrier_wait": tp[12] // len(pairs)},
                     local_iterations_per_tile=round(tp[6] / max(1, tp[7]), 2), tiles_processed=tp[7] // len(pairs))
        else:
            r.update(phases=fp[1] // len(pairs))
        res[name] = r
    autotune.full_tile(0)
    same = all(paths[k] == paths["phase"] for k in paths)
    return {"metric": "whole-lattice search time by engine (ms per search)", "unit": "ms",
            "config": {"workload": args.config, "lattice": [lat.nx, lat.ny, lat.nz], "arcs": int(g.E),
                       "costs": "0.12 + index jitter (uncongested)", "searches": len(pairs),
                       "path_lengths": [len(p or []) for p in paths["phase"]]},
            "identical_paths": bool(same), "engines": res}


def run_serving(args):
    """A bounded prefix of the serving stream through RouteServer: p50 / p99
    job latency (arrival to completion) and jobs per second."""
    import torch
    from orthoroute_gb300.serve import RouteServer
    warm = RouteServer(slots=1)
    warm.run_stream(serve_jobs(1, iter_cap=2))      # loads the kernels once
    warm.close()
    torch.cuda.synchronize()
    jobs = serve_jobs(args.serve_jobs, iter_cap=args.serve_iters)
    srv = RouteServer(slots=SERVE["slots"], hbm_budget_bytes=SERVE["budget_gb"] << 30)
    sampler = ClockSampler()
    sampler.start()
    t0 = time.perf_counter()
    out = srv.run_stream(jobs)
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    srv.close()
    kinds = {}
    for j in jobs:
        kinds[f"{j.nx}x{j.ny}x{j.nz}"] = kinds.get(f"{j.nx}x{j.ny}x{j.nz}", 0) + 1
    return {"metric": "serving stream: p99 job latency (arrival to completion)", "value": round(out["p99_s"], 4),
            "unit": "s", "higher_is_better": False, "n_gpus": 1,
            "p50_s": round(out["p50_s"], 4), "p99_s": round(out["p99_s"], 4),
            "jobs_per_s": round(out["jobs_per_s"], 4), "errors": out["errors"],
            "error_messages": sorted({r.error for r in out["results"] if r.error}),
            "peak_concurrent_jobs": out["peak_concurrent"], "peak_hbm_gb": round(out["peak_hbm_bytes"] / 2 ** 30, 2),
            "wall_s": round(wall, 3), "clocks": clocks, "data": "synthetic seeded job stream",
            "config": {"workload": "c4", "jobs": len(jobs), "of_stream": SERVE["jobs"], "rate_per_s": SERVE["rate"],
                       "iteration_cap": args.serve_iters, "slots": SERVE["slots"], "budget_gb": SERVE["budget_gb"],
                       "boards": kinds,
                       "sample": f"first {len(jobs)} jobs of the seeded {SERVE['jobs']}-job stream, "
                                 f"negotiation capped at {args.serve_iters} iterations per job"}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed jobs (default: 1 for c1, 3 for c0)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--config", default="c1", choices=sorted(CONFIGS) + ["c4"])
    ap.add_argument("--serve-jobs", type=int, default=16, help="c4: jobs of the stream to run")
    ap.add_argument("--serve-iters", type=int, default=5, help="c4: iteration cap per job")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode", default="persistent", choices=["persistent", "plain"])
    ap.add_argument("--full-engine", default="auto", choices=["auto", "grid", "cta"],
                    help="engine of full-graph nets; auto = autotuned per lattice")
    ap.add_argument("--compare-engines", action="store_true",
                    help="time the whole-lattice search engines on the workload's lattice and exit")
    ap.add_argument("--lattice", default=None, help="with --compare-engines: NXxNYxNZ instead of the workload's")
    ap.add_argument("--compare-plain", action="store_true", default=True)
    ap.add_argument("--no-compare-plain", dest="compare_plain", action="store_false")
    args = ap.parse_args()
    if args.config == "c4":
        if int(os.environ.get("RANK", "0")) == 0 and args.impl == "ours":
            print(json.dumps(run_serving(args)), flush=True)
        elif args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no serving loop"}), flush=True)
        return
    if args.compare_engines:
        if int(os.environ.get("RANK", "0")) == 0:
            print(json.dumps(run_engine_compare(args)), flush=True)
        return
    cfg = CONFIGS[args.config]
    if args.steps is None:
        args.steps = 1 if args.config == "c1" else 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args, cfg)), flush=True)
        return
    if world > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
    line = run_ours(args, cfg, rank, world)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, sample, cores = cpu_job_sample(args.config, cfg,
                                          gpu_counts=(line["searches_per_job"], line["result"]["iterations"]))
        line["cpu_baseline"] = {"value": round(v, 4), "unit": "s/job", "cores": cores, "kind": "port",
                                "sample": sample, "host_cpu": host_cpu()}
        fx = trajectory_fixture(args.config)
        if fx is not None and fx.get("wall_s"):
            line["cpu_baseline"]["full_job_measured_on_build_host_s"] = fx["wall_s"]
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as tdist
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
