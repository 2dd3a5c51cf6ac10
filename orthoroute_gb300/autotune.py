"""Autotuner: search engine, CTA grid and lanes per node, per lattice size.

Full-graph nets (Manhattan length >= 125, ``_route_all`` :8219-8262) are
searched either by ``full_sssp_kernel`` on a cooperative grid of CTAs (one
grid step per settle phase), by the tile-window engine on a grid of one CTA
per SM, or by a single 1024-thread CTA.  Which one is faster, and with how
many CTAs, depends on the lattice: a grid step costs a grid-wide barrier
(more CTAs, dearer barrier) and spreads the phase's front over the CTAs
(more CTAs, less work each).  The phase engine has no bucket width to tune
(each phase's threshold is the least tentative label and the settle rule is
fixed by exactness); the tile-window engine's window width is one.  So the
tuner sweeps

* the engine: "grid" or "cta";
* the lanes per examined frontier node of the "grid" engine (4, 8, 16) and
  whether waiting frontier nodes keep their last pull (on / off), timed on
  the full grid;
* then the grid of the "grid" engine: 1/4, 1/2, 3/4 and all of the resident
  CTAs (SMs x CTAs per SM);
* then the tile-window engine (label windows over lattice tiles in shared
  memory, tilesearch.cu) at window widths delta of 2, 4, 8, 16 and 32
  uncongested lateral hops: the delta of a delta-stepping search;

on a few full-graph searches of the job's own long nets over the current
costs, and keeps the fastest.  For ROI nets (one 1024-thread CTA per search)
it sweeps the lanes that serve one node (2, 4, 8, 16: the CTA's tile of
nodes in flight is 1024 / lanes), timing a spread of the job's ROI nets; the
best width follows the lattice's arcs per node.  Every setting returns the
same paths (the searches are exact and independent of the schedule), so
tuning changes only time.  Results are cached per (lattice, GPU) in a JSON
file.
"""
from __future__ import annotations

import ctypes as C
import json
import os
from dataclasses import asdict, dataclass, field
from typing import Dict, List, Sequence, Tuple

import torch

from . import _lib


@dataclass
class Tuning:
    key: str
    full_engine: str
    full_ctas: int
    ms_per_search: Dict[str, float] = field(default_factory=dict)
    roi_lanes: int = 4
    full_lanes: int = 16
    full_reuse: int = 0
    full_tile_delta: float = 0.0     # > 0: tile-window engine with this window width
    samples: int = 0
    cached: bool = False


def full_grid(ctas: int = 0) -> Tuple[int, int]:
    """Set (ctas > 0) or read the whole-lattice search's grid: (current, limit)."""
    cur, lim = C.c_int32(0), C.c_int32(0)
    _lib.check(_lib.load().ogr_full_grid(int(ctas), C.byref(cur), C.byref(lim)), "ogr_full_grid")
    return int(cur.value), int(lim.value)


def search_lanes(lanes: int = 0) -> int:
    """Set (lanes > 0) or read the ROI search's lanes per node."""
    cur = C.c_int32(0)
    _lib.check(_lib.load().ogr_search_lanes(int(lanes), C.byref(cur)), "ogr_search_lanes")
    return int(cur.value)


LANES = (2, 4, 8, 16)
FULL_LANES = (4, 8, 16)


def full_lanes(lanes: int = 0) -> int:
    """Set (lanes > 0) or read the whole-lattice search's lanes per frontier node."""
    cur = C.c_int32(0)
    _lib.check(_lib.load().ogr_full_lanes(int(lanes), C.byref(cur)), "ogr_full_lanes")
    return int(cur.value)


def full_reuse(mode: int = -1) -> int:
    """Set (0 / 1) or read (-1) the whole-lattice search's reuse of clean pulls."""
    cur = C.c_int32(0)
    _lib.check(_lib.load().ogr_full_reuse(int(mode), C.byref(cur)), "ogr_full_reuse")
    return int(cur.value)


TILE_DELTA_HOPS = (2, 4, 8, 16, 32)


def full_tile(enable: int = -1, delta: float = 0.0, tx: int = 0, ty: int = 0) -> Tuple[int, float]:
    """Select (enable 1 with window width delta > 0), deselect (0) or read (-1)
    the tile-window engine of whole-lattice searches: (enabled, delta)."""
    cur, d = C.c_int32(0), C.c_double(0.0)
    _lib.check(_lib.load().ogr_full_tile(int(enable), float(delta), int(tx), int(ty), C.byref(cur), C.byref(d)),
               "ogr_full_tile")
    return int(cur.value), float(d.value)


def hop_cost(lattice, base_cost_weight: float = 0.3) -> float:
    """One uncongested lateral hop of the cost update (pitch x base weight):
    the unit of the tile engine's window widths."""
    return float(lattice.pitch) * float(base_cost_weight)


def window_lookahead(nets: int = -1) -> int:
    """Set (0..16) or read (-1) how many clashing nets a disjoint-ROI window may skip."""
    cur = C.c_int32(0)
    _lib.check(_lib.load().ogr_window_lookahead(int(nets), C.byref(cur)), "ogr_window_lookahead")
    return int(cur.value)


def cache_path() -> str:
    return os.environ.get("ORTHOROUTE_GB300_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "orthoroute_gb300", "autotune.json"))


def lattice_key(lattice, device) -> str:
    props = torch.cuda.get_device_properties(device)
    spans = getattr(lattice, "allowed_via_spans", None)
    spans = "all" if spans is None else ",".join(f"{a}-{b}" for a, b in sorted(spans))
    return f"{props.name}/{props.multi_processor_count}sm/{lattice.nx}x{lattice.ny}x{lattice.nz}/{spans}"


def _load_cache(path: str) -> Dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store_cache(path: str, key: str, t: Tuning) -> None:
    data = _load_cache(path)
    data[key] = asdict(t)
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = f"{path}.{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass    # a read-only home only loses the cache


def candidates(limit: int) -> List[Tuple[str, int]]:
    grids = sorted({max(1, (limit * k) // 4) for k in (1, 2, 3, 4)})
    return [("grid", c) for c in grids] + [("cta", 0)]


def _time_roi(ops, nets, lanes) -> float:
    search_lanes(lanes)
    t0 = ops.counters["search_ms"]
    for s, d in nets:
        ops.find_path(ops.net_args(0, s, d, full_graph=False, penalty=False), engine="cta")
    return (ops.counters["search_ms"] - t0) / max(1, len(nets))


def tune(ops, lattice, nets: Sequence[Tuple[int, int]], roi_nets: Sequence[Tuple[int, int]] = (), *,
         use_cache: bool = True, cta_max_nodes: int = 400_000, repeats: int = 1) -> Tuning:
    """Pick the engine and grid for full-graph searches of `lattice` by timing
    searches of `nets` ((src, dst) pairs, full-graph length), and the lanes
    per node of ROI searches by timing `roi_nets`, on `ops`'s current costs.
    Leaves the choices set and returns them."""
    key = lattice_key(lattice, ops.g.device)
    path = cache_path()
    if use_cache:
        hit = _load_cache(path).get(key)
        if hit:
            t = Tuning(**{**hit, "cached": True})
            if t.full_engine == "grid":
                full_grid(t.full_ctas)
                full_lanes(t.full_lanes)
                full_reuse(t.full_reuse)
            full_tile(1 if t.full_tile_delta > 0 else 0, t.full_tile_delta)
            search_lanes(t.roi_lanes)
            return t
    cur, limit = full_grid(0)
    full_tile(0)
    nets = list(nets)
    roi_nets = list(roi_nets)
    timings: Dict[str, float] = {}
    lanes0 = search_lanes(0)
    best_lanes = lanes0
    if roi_nets:
        _time_roi(ops, roi_nets[:1], lanes0)       # untimed: workspace and caches
        lane_ms = {lanes: _time_roi(ops, roi_nets, lanes) for lanes in LANES}
        best_lanes = min(LANES, key=lambda k: (lane_ms[k], k))
        timings.update({f"roi_lanes{k}": round(v, 4) for k, v in lane_ms.items()})
    search_lanes(best_lanes)
    best = ("grid", limit, float("inf"))
    stream = torch.cuda.current_stream()
    if not nets:
        t = Tuning(key=key, full_engine="grid", full_ctas=cur, ms_per_search=timings, roi_lanes=best_lanes,
                   samples=len(roi_nets))
        if use_cache:
            _store_cache(path, key, t)
        return t
    # one untimed search first: workspace, lazy module load and caches
    s0, d0 = nets[0]
    ops.find_path(ops.net_args(0, s0, d0, full_graph=True, penalty=False), engine="grid")

    def time_full(engine):
        ms = 0.0
        for _ in range(repeats):
            for s, d in nets:
                t0 = ops.counters["search_ms"]
                ops.find_path(ops.net_args(0, s, d, full_graph=True, penalty=False), engine=engine)
                ms += ops.counters["search_ms"] - t0
        return ms / max(1, repeats * len(nets))

    lanes_ms = {}
    full_grid(limit)
    for lanes in FULL_LANES:
        for reuse in (0, 1):
            full_lanes(lanes)
            full_reuse(reuse)
            lanes_ms[(lanes, reuse)] = time_full("grid")
            timings[f"full_lanes{lanes}_reuse{reuse}"] = round(lanes_ms[(lanes, reuse)], 4)
    best_full_lanes, best_reuse = min(lanes_ms, key=lambda k: (lanes_ms[k], -k[0], k[1]))
    full_lanes(best_full_lanes)
    full_reuse(best_reuse)
    try:
        for engine, ctas in candidates(limit):
            if engine == "cta" and ops.g.N > cta_max_nodes:
                continue        # one CTA over a lattice this large is never the faster engine
            if engine == "grid":
                full_grid(ctas)
            ms = lanes_ms[(best_full_lanes, best_reuse)] if (engine == "grid" and ctas == limit) else time_full(engine)
            name = f"grid{ctas}" if engine == "grid" else "cta"
            timings[name] = round(ms, 4)
            if ms < best[2]:
                best = (engine, ctas, ms)
    finally:
        stream.synchronize()
    engine, ctas, best_ms = best
    full_grid(ctas if engine == "grid" else cur)
    # the tile-window engine at each window width (it hands a net it cannot
    # take to the phase engine configured above)
    tile_delta = 0.0
    if engine == "grid":
        unit = hop_cost(lattice)
        try:
            for hops in TILE_DELTA_HOPS:
                full_tile(1, hops * unit)
                ms = time_full("grid")
                timings[f"tile_delta{hops}"] = round(ms, 4)
                if ms < best_ms:
                    best_ms, tile_delta = ms, hops * unit
        finally:
            full_tile(1 if tile_delta > 0 else 0, tile_delta)
            stream.synchronize()
    t = Tuning(key=key, full_engine=engine, full_ctas=ctas if engine == "grid" else cur, ms_per_search=timings,
               samples=len(nets) + len(roi_nets), roi_lanes=best_lanes, full_lanes=best_full_lanes,
               full_reuse=best_reuse, full_tile_delta=tile_delta)
    if use_cache:
        _store_cache(path, key, t)
    return t


def sample_roi_nets(tasks: Dict, distance, threshold: int, k: int = 16) -> List[Tuple[int, int]]:
    """Up to k ROI nets of a job spread evenly over its name order, for timing."""
    rows = sorted((str(n), s, d) for n, (s, d) in tasks.items() if 0 < distance(s, d) < threshold)
    if not rows:
        return []
    step = max(1, len(rows) // k)
    return [(s, d) for _, s, d in rows[::step][:k]]


def sample_full_nets(tasks: Dict, distance, threshold: int, k: int = 3) -> List[Tuple[int, int]]:
    """The k longest full-graph nets of a job (ties by name), for timing."""
    rows = []
    for name, (s, d) in tasks.items():
        dist = distance(s, d)
        if dist >= threshold:
            rows.append((-dist, str(name), s, d))
    rows.sort()
    return [(s, d) for _, _, s, d in rows[:k]]
