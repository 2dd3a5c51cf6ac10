"""Write the oracle's trajectory of a benchmark workload as a fixture.

Runs the CPU oracle loop (``oracle.loop.OracleRouter`` with the C heap
Dijkstra), which is pinned to the reference's own routing runs by
``tests/golden/make_golden.py``, on one of the seeded workloads that
``bench.py`` times, and writes per-iteration path fingerprints, the
iteration metrics and the final tallies (``orthoroute_gb300/trajectory.py``):

    python tests/golden/make_c1_trajectory.py                 # c1 -> tests/golden/c1_trajectory.json.gz
    python tests/golden/make_c1_trajectory.py --config c0     # c0 -> tests/golden/c0_trajectory.json.gz

c1 (600x400x12, 2,000 nets, 40 iterations) takes hours on one core: the
whole-lattice searches settle about a million nodes each.  A partial file
(``.partial``) is rewritten after every iteration.  The run fixes
``PYTHONHASHSEED`` (the detail pass picks nets in string-hash order).
"""
from __future__ import annotations

import argparse
import hashlib
import os
import platform
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

HASH_SEED = "0"


class _Recorder:
    def __init__(self, on_record):
        from orthoroute_gb300.trajectory import TrajectoryRecorder
        self.rec = TrajectoryRecorder()
        self.on_record = on_record
        self.t0 = time.perf_counter()
        self.times = []

    def append(self, paths):
        self.rec.append(paths)
        self.times.append(round(time.perf_counter() - self.t0, 1))
        self.on_record(self)

    def __len__(self):
        return len(self.rec)


def run(config: str, out: str, iters=None, router_cls=None, log=print) -> dict:
    import bench
    from orthoroute_gb300 import trajectory
    from oracle.lattice import LatticeSpec
    from oracle.loop import Config, OracleRouter

    cfg = dict(bench.CONFIGS[config])
    if iters is not None:
        cfg["iters"] = int(iters)
    reqs = bench.make_requests(cfg)
    tasks = {n: (s, d) for n, s, d in reqs if s != d}
    nx, ny, nz = cfg["nx"], cfg["ny"], cfg["nz"]
    cls = router_cls or OracleRouter
    t0 = time.perf_counter()
    R = cls(LatticeSpec(nx, ny, nz, allowed_via_spans=bench.via_spans(cfg)), bench.board_bounds(nx, ny),
            Config(max_iterations=cfg["iters"]), fast=True)
    for n, s, d in reqs:
        if s == d:
            R.net_paths[n] = [s]
    doc = {"workload": config, "lattice": [nx, ny, nz], "nets": len(reqs), "max_iterations": cfg["iters"],
           "via_spans": bench.via_spans(cfg), "seed": cfg["seed"], "pythonhashseed": os.environ.get("PYTHONHASHSEED"),
           "generator": "oracle.loop.OracleRouter(fast=True)", "host": platform.machine()}

    def on_record(r):
        doc["records"] = r.rec.records
        doc["record_wall_s"] = r.times
        doc["searches"] = R.stats.get("searches")
        trajectory.save(out + ".partial", doc)
        log(f"[{config}] record {len(r)} at {r.times[-1]} s, searches {R.stats.get('searches')}")

    R.trace = _Recorder(on_record)
    res = R.route(tasks)
    doc["records"] = R.trace.rec.records
    doc["record_wall_s"] = R.trace.times
    doc["searches"] = R.stats.get("searches")
    doc["scanned"] = R.stats.get("scanned")
    doc["settled"] = R.stats.get("settled")
    doc["wall_s"] = round(time.perf_counter() - t0, 1)
    doc["result"] = {k: (bool(v) if isinstance(v, bool) else v) for k, v in res.items()
                     if k in ("success", "converged", "iterations", "overuse_sum", "overuse_edges",
                              "barrel_conflicts", "failed_nets", "path_node_overuse_sum", "best_iteration")}
    doc["iteration_metrics"] = [{k: int(v) for k, v in m.items()} for m in res.get("iteration_metrics", [])]
    doc["final_sha256"] = hashlib.sha256(trajectory.flat_paths(R.net_paths).tobytes()).hexdigest()
    trajectory.save(out, doc)
    if os.path.exists(out + ".partial"):
        os.remove(out + ".partial")
    return doc


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c1")
    ap.add_argument("--iters", type=int, default=None, help="iteration cap (default: the workload's)")
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    if os.environ.get("PYTHONHASHSEED") != HASH_SEED:
        os.environ["PYTHONHASHSEED"] = HASH_SEED
        os.execv(sys.executable, [sys.executable] + sys.argv)
    out = a.out or os.path.join(os.path.dirname(os.path.abspath(__file__)), f"{a.config}_trajectory.json.gz")
    doc = run(a.config, out, a.iters)
    print(f"wrote {out}: {len(doc['records'])} records, {doc['searches']} searches, {doc['wall_s']} s, "
          f"result {doc['result']}")


if __name__ == "__main__":
    main()
