"""``PathFinderRouter`` — the reference's router API over the GB300 kernels.

Keeps the public surface of OrthoRoute's router
(orthoroute/algorithms/manhattan/unified_pathfinder.py):

* ``PathFinderRouter(config=None, use_gpu=None)``                 :2697
* ``initialize_graph(board) -> bool``                             :2800
* ``route_multiple_nets(requests, progress_cb=None, iteration_cb=None)``
  with tuple requests ``(name, src, dst)`` or nets with ``.pads``  :4335
* ``net_paths: Dict[str, List[int]]`` and the result dict keys   :7510-7534

The negotiation policy (net order, hotsets, pressure schedule, cleanup
gating, stagnation rip-up, best-state restore, detail pass) runs on the host
exactly as the reference sequences it (:6163-7534); every step that touches
per-arc or per-node arrays runs on the device: cost update, via-pool
penalties and hard block, live-present rebase, ROI BFS + exact SSSP +
backtrace per net, commit / rip-up scatter, history, present EMA and the
overuse / layer tallies.  Host mirrors hold only what the policy reads at
path granularity (path-node use, node history, via pools); barrel ownership,
shared nodes and via-pool use are recomputed from one flat numpy view of all
paths per change.  There is no CPU routing fallback: a missing CUDA device
raises.
"""
from __future__ import annotations

import heapq
import os
import random
import time
from collections import defaultdict
from typing import Dict, List, Optional, Set, Tuple

import numpy as np
import torch

from . import _lib
from .device import DeviceGraph, DeviceState, Ops, PathStore, require_cuda, route_pass
from .lattice import Lattice

ROI_THRESHOLD_STEPS = 125
MAX_ROI_NODES = 50_000


class PathFinderConfig:
    """Router parameters (the fields of the reference's PathFinderConfig the
    negotiation loop reads, with the same defaults, :570-782)."""

    def __init__(self, **kw):
        self.max_iterations = 40
        self.owner_penalty_base = 25.0
        self.path_node_penalty_base = 25.0
        self.node_history_penalty = 5.0
        self.node_history_increment = 1.0
        self.pres_fac_init = 1.0
        self.pres_fac_mult = 1.10
        self.pres_fac_max = 64.0
        self.hist_gain = 0.2
        self.base_cost_weight = 0.3
        self.grid_pitch = 0.4
        self.preferred_layer_directions: Optional[List[str]] = None
        self.wrong_way_cost_multiplier = float("inf")
        self.via_cost = 0.7
        self.via_pressure_threshold = 64
        self.via_pressure_multiplier = 1.5
        self.allow_any_layer_via: Optional[bool] = None
        self.adjacent_via_step_scale = 4.0
        self.via_diameter = 0.25
        self.clearance = 0.15
        self.via_drill = 0.15
        self.track_width = 0.24
        self.layer_names: List[str] = ['F.Cu', 'In1.Cu', 'In2.Cu', 'In3.Cu', 'In4.Cu', 'B.Cu']
        self.min_hole_to_hole = 0.25
        self.stagnation_patience = 5
        self.slow_progress_window = 5
        self.slow_progress_min_fraction = 0.025
        self.slow_progress_min_overuse = 2048
        self.slow_progress_hotset_cap = 512
        self.slow_progress_hotset_growth_after = 2
        self.slow_progress_hotset_cap_max = 1024
        self.slow_progress_pressure_after = 2
        self.slow_progress_pres_fac_max = 1024.0
        self.slow_progress_pressure_trial_min_ratio = 0.80
        self.slow_progress_pressure_trial_patience = 2
        self.pressure_reference_hotset = 100
        self.pressure_work_scale_max = 2.0
        self.hist_cost_weight = 10.0
        self.hotset_cap = 2048
        self.hotset_cap_floor = 0
        self.physical_hotset_cap = 1024
        self.physical_hotset_min = 64
        self.physical_conflicts_per_hotset_net = 50.0
        self.via_keeper_rotation_overuse_threshold = 8
        self.via_keeper_rotation_nets_per_step = 1024
        self.portal_cleanup_edge_threshold = 3
        self.portal_cleanup_node_penalty = 1_000_000.0
        self.physical_cleanup_overuse_threshold = None
        self.history_decay = None
        self.live_present_costs = True
        self.reroute_only_offenders = True
        self.portal_enabled = False
        self.use_gpu = True
        self.layer_count = 6
        self._explicit = set()
        for k, v in kw.items():
            setattr(self, k, v)

    def __setattr__(self, k, v):
        if k == "max_iterations" and hasattr(self, "_explicit"):
            self._explicit.add(k)
        object.__setattr__(self, k, v)


# ------------------------------------------------------------- policy helpers
def _history_hotset_cap(t):
    if t <= 8:
        return 16
    if t <= 32:
        return 32
    if t <= 128:
        return 64
    if t <= 2048:
        return 100
    if t <= 16384:
        return 180
    return 256


def _exploration_fraction(t):
    return 0.15 if t > 16384 else 0.25 if t > 2048 else 0.40


def _conflict_aware_hotset(ranked, pairs, cap, fraction, rng):
    """Greedy pair cover + exploration (``_select_conflict_aware_hotset`` :8912-9037)."""
    cap = max(0, int(cap))
    if cap == 0 or not ranked:
        return []
    cands = list(dict.fromkeys(ranked))
    cap = min(cap, len(cands))
    cset = set(cands)
    rank = {c: i for i, c in enumerate(cands)}
    adj = defaultdict(set)
    for a, b in pairs or ():
        if a != b and a in cset and b in cset:
            adj[a].add(b)
            adj[b].add(a)
    fraction = min(1.0, max(0.0, float(fraction)))
    primary = max(1, min(cap, int(round(cap * (1.0 - fraction)))))
    sel, sset = [], set()
    rem = {c: set(adj.get(c, ())) for c in cands}
    heap = [(-len(rem[c]), rank[c], c) for c in cands if rem[c]]
    heapq.heapify(heap)
    while len(sel) < primary and heap:
        nd, _, c = heapq.heappop(heap)
        if c in sset:
            continue
        live = len(rem[c])
        if -nd != live:
            heapq.heappush(heap, (-live, rank[c], c))
            continue
        if live == 0:
            break
        sel.append(c)
        sset.add(c)
        for nb in tuple(rem[c]):
            rem[nb].discard(c)
            heapq.heappush(heap, (-len(rem[nb]), rank[nb], nb))
        rem[c].clear()
    if len(sel) < primary:
        nonred = [c for c in cands if c not in sset and not (adj.get(c, set()) & sset)]
        nrs = set(nonred)
        for c in nonred + [c for c in cands if c not in sset and c not in nrs]:
            sel.append(c)
            sset.add(c)
            if len(sel) >= primary:
                break
    if len(sel) < cap:
        rest = [c for c in cands if c not in sset]
        rng.shuffle(rest)
        sel.extend(rest[:cap - len(sel)])
    return sel


def _sorted_unique(a):
    """``np.unique`` of an integer array by one sort (NumPy 2's hashing
    ``unique`` is many times slower on the path arrays here)."""
    a = np.sort(np.asarray(a).ravel())
    if a.size > 1:
        a = a[np.concatenate(([True], a[1:] != a[:-1]))]
    return a


def _expand_ranges(lo, hi):
    """Concatenation of arange(lo[i], hi[i]) over i."""
    cnt = hi - lo
    total = int(cnt.sum())
    if total == 0:
        return np.zeros(0, dtype=np.int64)
    return np.repeat(lo - (np.cumsum(cnt) - cnt), cnt) + np.arange(total, dtype=np.int64)


class _PathDict(dict):
    """``net_paths`` (net name -> node list, the reference's dict) plus a
    version that every assignment bumps and cached int64 node arrays per net,
    from which the router's vectorised policy steps build one flat view of
    all paths per version.  Paths are replaced, never edited in place."""

    def __init__(self, *args, **kw):
        super().__init__(*args, **kw)
        self.version = 0
        self._arrays: Dict[str, np.ndarray] = {}

    def _touch(self, key):
        self.version += 1
        self._arrays.pop(key, None)

    def __setitem__(self, key, value):
        dict.__setitem__(self, key, value)
        self._touch(key)

    def set_path(self, key, value, array):
        """Assign `value` together with its node array (int64, same nodes)."""
        dict.__setitem__(self, key, value)
        self._touch(key)
        self._arrays[key] = array

    def __delitem__(self, key):
        dict.__delitem__(self, key)
        self._touch(key)

    def pop(self, key, *default):
        out = dict.pop(self, key, *default)
        self._touch(key)
        return out

    def popitem(self):
        key, value = dict.popitem(self)
        self._touch(key)
        return key, value

    def clear(self):
        dict.clear(self)
        self.version += 1
        self._arrays.clear()

    def update(self, *args, **kw):
        for key, value in dict(*args, **kw).items():
            self[key] = value

    def setdefault(self, key, default=None):
        if key not in self:
            self[key] = default
        return self[key]

    def __ior__(self, other):
        self.update(other)
        return self

    def array(self, key) -> np.ndarray:
        a = self._arrays.get(key)
        if a is None:
            a = np.asarray(self.get(key) or (), dtype=np.int64)
            self._arrays[key] = a
        return a


class _FlatPaths:
    """Every non-empty path of one ``net_paths`` version, concatenated in dict
    order (one-node paths are the reference's trivially routed nets).
    ``owner[i]`` is the position in ``names`` of the net of node i, ``ids``
    the nets' router ids (-1 for a one-node path that never got one),
    ``same[i]`` whether nodes i and i+1 are one net's hop, ``hops`` the
    positions i where (i, i+1) is a via hop (same (x, y), different z)."""

    def __init__(self, paths: _PathDict, plane: int, net_id, known_id):
        self.version = paths.version
        self.plane = plane
        self.names = [n for n, p in paths.items() if p is not None and len(p) >= 1]
        arrs = [paths.array(n) for n in self.names]
        k = len(arrs)
        self.lens = np.fromiter((a.size for a in arrs), dtype=np.int64, count=k)
        self.nodes = np.concatenate(arrs) if k else np.zeros(0, dtype=np.int64)
        self.owner = np.repeat(np.arange(k, dtype=np.int64), self.lens)
        self.ids = np.fromiter((net_id(n) if a.size >= 2 else known_id(n) for n, a in zip(self.names, arrs)),
                               dtype=np.int64, count=k)
        self.z, self.r = np.divmod(self.nodes, plane)
        self.same = self.owner[:-1] == self.owner[1:]
        self.hops = np.flatnonzero(self.same & (self.r[:-1] == self.r[1:]) & (self.z[:-1] != self.z[1:]))
        self._via = None

    def via_members(self):
        """(node, net id) of every node spanned by a net's via hops (each
        layer of the barrel), unique, sorted by node then id."""
        if self._via is None:
            h = self.hops
            zu, zv = self.z[h], self.z[h + 1]
            lo = np.minimum(zu, zv)
            cnt = np.abs(zu - zv) + 1
            rep = np.repeat(np.arange(h.size), cnt)
            off = np.arange(int(cnt.sum()), dtype=np.int64) - np.repeat(np.cumsum(cnt) - cnt, cnt)
            node = (lo[rep] + off) * self.plane + self.r[h][rep]
            nid = self.ids[self.owner[h]][rep]
            K = int(self.ids.max()) + 1 if self.ids.size else 1
            key = _sorted_unique(node * K + nid)
            self._via = (key // K, key % K)
        return self._via


class _ArcCount:
    """Stands for a net's arc list where only its length is kept."""
    __slots__ = ("size",)

    def __init__(self, n):
        self.size = int(n)

    def __len__(self):
        return self.size


class _ViaPools:
    """Column / segment via pools on the host (small: Nx*Ny*(Nz-2))."""

    def __init__(self, nx, ny, nz, col_cap=4, seg_cap=2):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.segZ = nz - 2 if nz > 2 else 0
        self.has_seg = nz > 2
        self.col_cap = np.full((nx, ny), col_cap, dtype=np.int16)
        self.col_use = np.zeros((nx, ny), dtype=np.int16)
        self.col_pres = np.zeros((nx, ny), dtype=np.float32)
        self.device_spatial = None        # set when the use counts come from the device
        if self.has_seg:
            self.seg_cap = np.full((nx, ny, self.segZ), seg_cap, dtype=np.int8)
            self.seg_use = np.zeros((nx, ny, self.segZ), dtype=np.int16)
            self.seg_pres = np.zeros((nx, ny, self.segZ), dtype=np.float32)
            self.seg_prefix = np.zeros((nx, ny, self.segZ), dtype=np.float32)
            self.seg_pres_via = None

    def rebuild(self, flat: _FlatPaths):
        """One column count per contiguous via run; its hull of segments
        (``_accumulate_via_usage_for_path`` :4470-4546), over all paths at once."""
        nx, ny = self.nx, self.ny
        h = flat.hops
        if h.size == 0:
            self.col_use[:] = 0
            if self.has_seg:
                self.seg_use[:] = 0
            return
        r, z = flat.r, flat.z
        # run starts: a via hop whose previous hop is not a via hop in the same
        # column (adjacent hop positions always belong to one net)
        start = np.ones(h.size, dtype=bool)
        start[1:] = ~((h[1:] == h[:-1] + 1) & (r[h[1:]] == r[h[:-1]]))
        rs = r[h[start]]
        col = np.bincount(rs, minlength=nx * ny).reshape(ny, nx).T
        self.col_use[:] = col.astype(np.int16)
        if not self.has_seg:
            return
        zl = np.clip(np.minimum(z[h], z[h + 1]), 1, self.nz - 2)
        zh = np.clip(np.maximum(z[h], z[h + 1]), 1, self.nz - 2)
        first = np.flatnonzero(start)
        lo = np.minimum.reduceat(zl, first)
        hi = np.maximum.reduceat(zh, first)
        cnt = np.maximum(hi - lo, 0)
        rep = np.repeat(np.arange(first.size), cnt)
        zz = lo[rep] + (np.arange(int(cnt.sum()), dtype=np.int64) - np.repeat(np.cumsum(cnt) - cnt, cnt))
        s = zz - 1
        ok = (s >= 0) & (s < self.segZ)
        rr = rs[rep][ok]
        flat_idx = ((rr % nx) * ny + rr // nx) * self.segZ + s[ok]
        seg = np.bincount(flat_idx, minlength=nx * ny * self.segZ).reshape(nx, ny, self.segZ)
        self.seg_use[:] = seg.astype(np.int16)

    def set_from_device(self, over, spatial):
        """Host mirror after a device rebuild: use counts of the over-full
        pools only (rows {kind 0 column / 1 segment, x, y, s, use}; every other
        pool reads as within capacity) and the spatial overuse sum."""
        self.col_use[:] = 0
        if self.has_seg:
            self.seg_use[:] = 0
        for kind, x, y, sidx, use in over.tolist():
            if kind == 0:
                self.col_use[x, y] = use
            else:
                self.seg_use[x, y, sidx] = use
        self.device_spatial = int(spatial)

    def update_presence(self, alpha=0.6, beta=0.4):
        over = np.maximum(0, self.col_use - self.col_cap).astype(np.float32)
        self.col_pres = alpha * over + beta * self.col_pres
        if self.has_seg:
            over = np.maximum(0, self.seg_use - self.seg_cap).astype(np.float32)
            prev = self.seg_pres_via if self.seg_pres_via is not None else self.seg_pres
            self.seg_pres_via = alpha * over + beta * prev
            self.seg_pres = self.seg_pres_via.copy()
            np.cumsum(self.seg_pres, axis=2, out=self.seg_prefix)

    def spatial_overuse(self):
        if self.device_spatial is not None:
            return self.device_spatial
        t = int(np.maximum(0, self.col_use - self.col_cap).sum())
        if self.has_seg:
            t += int(np.maximum(0, self.seg_use - self.seg_cap).sum())
        return t


# ------------------------------------------------------------------- router
class PathFinderRouter:
    """GB300 PathFinder router with the reference's Python API."""

    def __init__(self, config: Optional[PathFinderConfig] = None, use_gpu: Optional[bool] = None,
                 device: str = "cuda", mode: str = "persistent", full_engine: str = "grid",
                 window_slots: int = 32):
        require_cuda()
        if mode not in ("persistent", "plain"):
            raise ValueError("mode must be 'persistent' (one launch per routing pass) or 'plain' (one per net)")
        if full_engine not in ("grid", "tile", "cta", "auto"):
            raise ValueError("full_engine must be 'grid' (phase-settled search on all SMs per full-graph net), "
                             "'tile' (tile-window search on all SMs), 'cta' (one CTA) or "
                             "'auto' (the autotuner picks per lattice)")
        self.config = config or PathFinderConfig()
        self.device = device
        self.mode = mode
        self.full_engine = "grid" if full_engine == "tile" else full_engine
        self.full_engine_request = full_engine
        self.full_tile_delta = 0.0       # > 0: whole-lattice searches use the tile-window engine
        self.tuning = None
        self.window_slots = int(window_slots)   # > 0: batched disjoint-ROI windows in persistent mode
        self.store: Optional[PathStore] = None
        self.lattice: Optional[Lattice] = None
        self.net_paths: Dict[str, List[int]] = {}
        self.iteration = 0
        self.trace = None
        self.search_log = None
        self.stats = {"searches": 0, "arcs": 0, "pops": 0, "search_s": 0.0}

    # ------------------------------------------------------------- set-up
    @staticmethod
    def board_bounds(board):
        """``_calc_bounds`` (:3266-3321): pads of nets with 2+ pads, +3 mm."""
        xs, ys = [], []
        for net in getattr(board, "nets", []) or []:
            pads = getattr(net, "pads", []) or []
            if len(pads) >= 2:
                for p in pads:
                    if getattr(p, "position", None) is not None:
                        xs.append(p.position.x)
                        ys.append(p.position.y)
        if not xs:
            if hasattr(board, "_kicad_bounds"):
                b = board._kicad_bounds
                return (b[0] - 3.0, b[1] - 3.0, b[2] + 3.0, b[3] + 3.0)
            return (0, 0, 100, 100)
        return (min(xs) - 3.0, min(ys) - 3.0, max(xs) + 3.0, max(ys) + 3.0)

    @staticmethod
    def assign_layer_axes(signal_layers, demand_h_pct, anchor_top_is_h=True):
        """``assign_layer_axes_by_demand`` (board_analyzer.py:17-62)."""
        n = len(signal_layers)
        if n == 0:
            return set(), set()
        if n == 1:
            return (set(signal_layers), set()) if demand_h_pct >= 0.5 else (set(), set(signal_layers))
        h_goal = max(1, min(n - 1, int(round(n * float(demand_h_pct)))))
        h, v = set(), set()
        want_h = anchor_top_is_h
        for layer in signal_layers:
            if want_h and len(h) < h_goal:
                h.add(layer)
            else:
                v.add(layer)
            want_h = not want_h
        while len(h) < h_goal and v:
            mid = sorted(v)[len(v) // 2]
            v.remove(mid)
            h.add(mid)
        while len(h) > h_goal and h:
            mid = sorted(h)[len(h) // 2]
            h.remove(mid)
            v.add(mid)
        return h, v

    @classmethod
    def demand_layer_directions(cls, board, layer_count):
        """``preferred_layer_directions_for_board`` (board_analyzer.py:65-105)."""
        ddx = ddy = 0.0
        for net in getattr(board, "nets", ()) or ():
            pads = getattr(net, "pads", ()) or ()
            if len(pads) < 2:
                continue
            a, b = pads[0].position, pads[1].position
            ddx += abs(float(b.x) - float(a.x))
            ddy += abs(float(b.y) - float(a.y))
        tot = ddx + ddy
        pct = ddx / tot if tot > 1e-9 else 0.5
        if os.environ.get("ORTHO_LATERAL_ALL", "0") == "1":
            sig = list(range(int(layer_count)))
        else:
            sig = list(range(1, max(1, int(layer_count) - 1)))
        h, _ = cls.assign_layer_axes(sig, pct)
        dirs = ["h" if z in h else "v" for z in range(int(layer_count))]
        if dirs:
            dirs[0] = "v"
        return dirs

    def initialize_graph(self, board) -> bool:
        cfg = self.config
        bounds = self.board_bounds(board)
        nz = int(getattr(board, "layer_count", None) or cfg.layer_count)
        cfg.layer_count = nz
        pitch = cfg.grid_pitch
        gx0 = round(bounds[0] / pitch) * pitch
        gy0 = round(bounds[1] / pitch) * pitch
        gx1 = round(bounds[2] / pitch) * pitch
        gy1 = round(bounds[3] / pitch) * pitch
        nx = int((gx1 - gx0) / pitch) + 1
        ny = int((gy1 - gy0) / pitch) + 1
        dirs = cfg.preferred_layer_directions or self.demand_layer_directions(board, nz)
        spacing = max(float(cfg.via_diameter) + float(cfg.clearance),
                      float(cfg.via_drill) + float(cfg.min_hole_to_hole))
        lat = Lattice(nx, ny, nz, pitch=pitch, layer_dirs=list(dirs), via_cost=cfg.via_cost,
                      allow_any_layer_via=cfg.allow_any_layer_via,
                      adjacent_via_step_scale=cfg.adjacent_via_step_scale, min_via_center_spacing=spacing,
                      wrong_way_cost_multiplier=float(os.environ.get("ORTHO_WRONG_WAY",
                                                                     cfg.wrong_way_cost_multiplier)))
        self.initialize_lattice(lat, bounds)
        return True

    def initialize_lattice(self, lattice: Lattice, bounds=None, layer_names: Optional[List[str]] = None):
        """Build the device CSR and congestion state for a lattice."""
        self.lattice = lattice
        self.tuning = None
        if self.full_engine_request == "auto":
            self.full_engine = "grid"
        from . import autotune
        self.full_tile_delta = (autotune.TILE_DELTA_HOPS[2] * autotune.hop_cost(lattice, self.config.base_cost_weight)
                                if self.full_engine_request == "tile" else 0.0)
        # copper layer names as initialize_graph derives them (:2883-2904)
        names = list(layer_names) if layer_names else list(getattr(self.config, "layer_names", []) or [])
        if len(names) != lattice.nz:
            names = ["F.Cu"] + [f"In{i}.Cu" for i in range(1, lattice.nz - 1)] + (["B.Cu"] if lattice.nz > 1 else [])
        self.config.layer_names = names
        self._geometry_payload = GeometryPayload([], [])
        self._provisional_geometry = GeometryPayload([], [])
        if bounds is None:
            p = lattice.pitch
            bounds = (0.0, 0.0, (lattice.nx - 1) * p, (lattice.ny - 1) * p)
        self.bounds = bounds
        self.g = DeviceGraph(lattice, device=self.device)
        self.s = DeviceState(self.g)
        self.s.enable_rcost()
        self.ops = Ops(self.g, self.s)
        L = lattice
        self.nx, self.ny, self.nz = L.nx, L.ny, L.nz
        self.plane = L.plane
        self.N = L.num_nodes
        self.E = self.g.E
        self.pools = _ViaPools(L.nx, L.ny, L.nz)
        self.node_use = np.zeros(self.N, dtype=np.int16)
        self._via_owner = np.full(self.N, -1, dtype=np.int64)
        self._via_owner_set = np.zeros(0, dtype=np.int64)
        self.node_history = np.zeros(self.N, dtype=np.float32)
        self._hist_iter = None
        self._hist_mask = np.zeros(self.N, dtype=bool)
        self._flat_view = None
        self.layer_bias = np.ones(self.nz, dtype=np.float32)
        self._layer_bias_ema = None
        self.net_paths = {}
        self.net_to_edges: Dict[str, np.ndarray] = {}
        self._eidx = None
        self.net_id_map: Dict[str, int] = {}
        dev = self.g.device
        self._d_col_pres = torch.zeros((L.nx, L.ny), dtype=torch.float32, device=dev)
        self._d_col_use = torch.zeros((L.nx, L.ny), dtype=torch.int16, device=dev)
        self._d_col_cap = torch.from_numpy(self.pools.col_cap).to(dev)
        if self.pools.has_seg:
            self._d_seg_prefix = torch.zeros((L.nx, L.ny, self.pools.segZ), dtype=torch.float32, device=dev)
            self._d_seg_use = torch.zeros((L.nx, L.ny, self.pools.segZ), dtype=torch.int16, device=dev)
            self._d_seg_cap = torch.from_numpy(self.pools.seg_cap).to(dev)
            self._d_seg_pres = torch.zeros((L.nx, L.ny, self.pools.segZ), dtype=torch.float32, device=dev)
        # device via pools (persistent mode): use counts rebuilt from the path store
        self._d_pool_scratch = torch.zeros(L.nx * L.ny * (1 + self.pools.segZ), dtype=torch.int32, device=dev)
        self._d_spatial = torch.zeros(1, dtype=torch.int64, device=dev)
        self._d_pool_over = torch.zeros(5 * 4096, dtype=torch.int32, device=dev)
        self._d_pool_over_n = torch.zeros(1, dtype=torch.int32, device=dev)
        self._d_disc = torch.zeros(self.nz * self.nz, dtype=torch.float64, device=dev)
        cap = max(1 << 16, min(self.E, 1 << 24))
        self._ov_idx = torch.empty(cap, dtype=torch.int32, device=dev)
        self._ov_val = torch.empty(cap, dtype=torch.float32, device=dev)
        self._ov_cnt = torch.zeros(1, dtype=torch.int32, device=dev)
        # device barrel scan (persistent mode): node marks with a stamp per call, output lists
        self._d_barrel_mark = torch.zeros(self.N, dtype=torch.int32, device=dev)
        self._barrel_stamp = 0
        self._barrel_cap = 0
        self._barrel_ids = None
        self._reset_policy_state()

    def initialize_state(self):
        """Reset the congestion state and policy for a new job on the same lattice."""
        s = self.s
        for t in (s.present, s.present_ema, s.history, s.total_cost, s.live_static, s.path_node_use,
                  s.owner_count, s.owner_xor, s.node_history):
            t.zero_()
        if s.rcost is not None:
            s.rcost.zero_()
        s.layer_bias.fill_(1.0)
        s.use_layer_bias = False
        self.pools = _ViaPools(self.nx, self.ny, self.nz)
        self._d_col_pres.zero_()
        if self.pools.has_seg:
            self._d_seg_pres.zero_()
            self._d_seg_prefix.zero_()
        self.node_use.fill(0)
        self.node_history.fill(0)
        self._hist_iter = None
        self._hist_mask.fill(False)
        self.layer_bias = np.ones(self.nz, dtype=np.float32)
        self._layer_bias_ema = None
        self.net_paths = {}
        self.net_to_edges = {}
        self._eidx = None
        self.net_id_map = {}
        self.iteration = 0
        self._reset_policy_state()

    def profile_reset(self):
        self.ops.reset_counters()
        self.ops.discarded.zero_()
        self.stats = {"searches": 0, "arcs": 0, "pops": 0, "search_s": 0.0}

    def profile_snapshot(self):
        """Counters since profile_reset.  `searches` counts accepted searches
        (the reference's); `discarded_searches` the window searches whose
        results were undone because an earlier member of their window failed
        (those nets were searched again, and that search is in `searches`)."""
        c = dict(self.ops.counters)
        disc = self.ops.discarded.cpu().numpy()
        return {"launches": int(c["launches"]), "h2d_bytes": int(c["h2d_bytes"]), "d2h_bytes": int(c["d2h_bytes"]),
                "search_launches": int(c["search_launches"]), "search_kernel_ms": float(c["search_ms"]),
                "searches": self.stats["searches"], "arcs": self.stats["arcs"], "pops": self.stats["pops"],
                "search_wall_s": float(self.stats["search_s"]),
                "discarded_searches": int(disc[0]), "discarded_arcs": int(disc[1]), "discarded_pops": int(disc[2])}

    def _reset_policy_state(self):
        self.stagnation_counter = 0
        self.full_graph_fallback_count = 0
        self._last_ripped: Set[str] = set()
        self._freeze_pres_fac_until = 0
        self._stagnation_victim_history: Set[str] = set()
        self._stagnation_victim_cursor = 0
        self._cleanup_move_counts = defaultdict(int)
        self.freeze = False
        self.physical_cleanup_started = False
        self.barrel_count = 0
        self.path_node_scores: Dict[str, int] = {}
        self.path_node_pairs = set()
        self.exact_pairs = set()
        self.barrel_conflict_nets: Set[str] = set()
        self.barrel_owner_nets: Set[str] = set()
        self.barrel_victim_nets: Set[str] = set()
        self.physical_scores = defaultdict(int)
        self._net_clean_iters: Dict[str, int] = {}
        self._last_reroute_iter: Dict[str, int] = {}
        self._via_pool_keepers = {}
        self._via_pool_member_state = {}
        self._via_pool_keeper_stagnation = {}
        self._last_hotset_size = 0
        self._pres_fac_now = 1.0
        self._present_pres_fac = 1.0

    # ------------------------------------------------------------- helpers
    def _net_id(self, name):
        if name not in self.net_id_map:
            self.net_id_map[name] = len(self.net_id_map)
        return self.net_id_map[name]

    def idx_to_coord(self, n):
        z, r = divmod(int(n), self.plane)
        y, x = divmod(r, self.nx)
        return x, y, z

    def _overused(self):
        """(arc ids, over values) of every arc with present > capacity (device compaction)."""
        lib = self.ops.lib
        cap = int(self._ov_idx.numel())
        _lib.check(lib.ogr_overused_arcs(self.E, self.s.present.data_ptr(), self.s.capacity.data_ptr(),
                                         self._ov_idx.data_ptr(), self._ov_val.data_ptr(), cap,
                                         self._ov_cnt.data_ptr(), self.ops._sp()), "ogr_overused_arcs")
        n = int(self._ov_cnt.item())
        if n > cap:
            raise RuntimeError("overused-arc buffer too small")
        idx = self._ov_idx[:n].cpu().numpy().astype(np.int64)
        val = self._ov_val[:n].cpu().numpy()
        self.ops.counters["d2h_bytes"] += 4 + 8 * n
        order = np.argsort(idx)
        return idx[order], val[order]

    def _arc_attrs(self, idx):
        """(src, dst, layer, is_via) of the given arcs, gathered on the device
        (the policy asks only about its few overused arcs)."""
        idx = np.asarray(idx, dtype=np.int64)
        if idx.size == 0:
            z = np.zeros(0, dtype=np.int64)
            return z, z, z, np.zeros(0, dtype=bool)
        g = self.g
        t = torch.from_numpy(idx).to(g.device)
        out = [x.index_select(0, t).cpu().numpy() for x in (g.edge_src, g.indices, g.edge_layer, g.edge_kind)]
        self.ops.counters["h2d_bytes"] += 8 * idx.size
        self.ops.counters["d2h_bytes"] += 10 * idx.size
        return (out[0].astype(np.int64), out[1].astype(np.int64), out[2].astype(np.int64), out[3].astype(bool))

    def _over_map(self):
        idx, val = self._overused()
        return dict(zip(idx.tolist(), val.tolist())), idx, val

    # host mirrors of node state ------------------------------------------------
    @property
    def net_paths(self) -> Dict[str, List[int]]:
        return self._net_paths

    @net_paths.setter
    def net_paths(self, value):
        self._net_paths = value if isinstance(value, _PathDict) else _PathDict(value)

    def _flat(self) -> _FlatPaths:
        """The flat view of the current paths (rebuilt after any change)."""
        f = self._flat_view
        if f is None or f.version != self._net_paths.version or f.src is not self._net_paths:
            f = _FlatPaths(self._net_paths, self.plane, self._net_id, lambda n: self.net_id_map.get(n, -1))
            f.src = self._net_paths
            self._flat_view = f
        return f

    def _mark_many(self, arrays, sign):
        """_mark_nodes of many paths at once: each path's distinct nodes count once."""
        arrays = [a for a in arrays if a.size]
        if not arrays:
            return
        P = len(arrays)
        key = _sorted_unique(np.concatenate(arrays) * P +
                             np.repeat(np.arange(P, dtype=np.int64), [a.size for a in arrays]))
        cnt = np.bincount(key // P, minlength=self.N)
        hit = np.flatnonzero(cnt)
        if sign > 0:
            self.node_use[hit] += cnt[hit].astype(self.node_use.dtype)
        else:
            self.node_use[hit] = np.maximum(self.node_use[hit].astype(np.int64) - cnt[hit], 0).astype(self.node_use.dtype)

    def _mark_nodes(self, name, path, sign, array=None):
        """path_node_use of one net's path (``_mark_path_node_use`` :4635);
        the via-barrel ownership is derived from the paths when read."""
        nodes = _sorted_unique(np.asarray(path, dtype=np.int64) if array is None else array)
        if sign > 0:
            self.node_use[nodes] += 1
        else:
            self.node_use[nodes] = np.maximum(self.node_use[nodes] - 1, 0)

    def _via_owner_of(self, flat: _FlatPaths):
        """Per-node barrel owner (``_mark_via_barrel_ownership_for_path``
        :4934): -1 no via of any net, the net id for one net, -2 for several.
        A dense node array of which only the nodes set last time are reset."""
        vn, vid = flat.via_members()
        own = self._via_owner
        own[self._via_owner_set] = -1
        if vn.size:
            first = np.ones(vn.size, dtype=bool)
            first[1:] = vn[1:] != vn[:-1]
            starts = np.flatnonzero(first)
            cnt = np.diff(np.append(starts, vn.size))
            un = vn[starts]
            own[un] = np.where(cnt == 1, vid[starts], -2)
            self._via_owner_set = un
        else:
            self._via_owner_set = np.zeros(0, dtype=np.int64)
        return own

    def _accumulate_history(self, nodes):
        """Node conflict history, once per node per iteration."""
        nodes = _sorted_unique(np.asarray(nodes if isinstance(nodes, np.ndarray) else list(nodes), dtype=np.int64))
        if nodes.size == 0:
            return
        if self._hist_iter != self.iteration:
            self._hist_iter = self.iteration
            self._hist_mask.fill(False)
        nodes = nodes[~self._hist_mask[nodes]]
        if nodes.size == 0:
            return
        self.node_history[nodes] += np.float32(self.config.node_history_increment)
        self._hist_mask[nodes] = True
        d = torch.from_numpy(nodes).to(self.g.device)
        self.s.node_history[d] = torch.from_numpy(self.node_history[nodes]).to(self.g.device)

    def _update_tracking(self, name, edges):
        """Track a committed net's arcs: the arc list itself (plain mode, whose
        per-net overuse is summed on the host), or only their count (persistent
        mode sums on the device from the path store)."""
        self.net_to_edges.pop(name, None)
        self.net_to_edges[name] = (_ArcCount(int(edges)) if isinstance(edges, (int, np.integer))
                                   else np.asarray(edges, dtype=np.int64))
        self._eidx = None

    def _clear_tracking(self, name):
        if self.net_to_edges.pop(name, None) is not None:
            self._eidx = None

    def _edge_index(self):
        """Flat (arc, net) view of net_to_edges, rebuilt after any change:
        (net names, arcs concatenated in net order, net position per arc)."""
        if self._eidx is None:
            names = [n for n, e in self.net_to_edges.items() if len(e)]
            if names:
                arrs = [self.net_to_edges[n] for n in names]
                lens = np.fromiter((a.size for a in arrs), dtype=np.int64, count=len(arrs))
                flat = np.concatenate(arrs)
                owner = np.repeat(np.arange(len(names), dtype=np.int64), lens)
            else:
                flat = np.zeros(0, dtype=np.int64)
                owner = np.zeros(0, dtype=np.int64)
            self._eidx = (names, flat, owner)
        return self._eidx

    def _edge_over(self, over_idx, over_val, canonical_only=False):
        """For every tracked net: (Σ over values of its arcs in its arc order —
        the left-to-right float sum of the reference's generator — and whether
        any of its arcs is in over_idx).  over_idx: sorted arc ids.  The
        overused arcs are looked up through a dense arc-indexed scratch array;
        the result is reused while neither the tracking nor the overuse
        changed (the hotset and the net order of one iteration ask the same)."""
        if getattr(self, "store", None) is not None:
            return self._edge_over_device(canonical_only)
        names, flat, owner = self._edge_index()
        k = len(names)
        oi = np.asarray(over_idx, dtype=np.int64)
        ov = np.asarray(over_val, dtype=np.float64)
        c = getattr(self, "_edge_over_cache", None)
        if c is not None and c[0] is self._eidx and np.array_equal(c[1], oi) and np.array_equal(c[2], ov):
            return c[3]
        if k == 0 or oi.size == 0:
            out = (names, np.zeros(k, dtype=np.float64), np.zeros(k, dtype=bool))
        else:
            dense = getattr(self, "_over_dense", None)
            if dense is None or dense.size != self.E:
                # the over values are float32 on the device: a float32 scratch holds them exactly
                dense = self._over_dense = np.zeros(self.E, dtype=np.float32)
                self._over_mask = np.zeros(self.E, dtype=bool)
            mask = self._over_mask
            dense[oi] = ov
            mask[oi] = True
            try:
                hit = mask[flat]
                w = dense[flat].astype(np.float64)
            finally:
                dense[oi] = 0.0
                mask[oi] = False
            sums = np.bincount(owner, weights=w, minlength=k)
            anyhit = np.bincount(owner, weights=hit.astype(np.float64), minlength=k) > 0
            out = (names, sums, anyhit)
        self._edge_over_cache = (self._eidx, oi.copy(), ov.copy(), out)
        return out

    def _edge_over_device(self, canonical_only):
        """The persistent mode's version of _edge_over: every net's overuse sum
        and hit flag over the arcs of its stored path, computed on the device
        from the present counts (ogr_nets_overuse) — the same whole-number
        sums, without the arcs on the host."""
        st = self.store
        k = st.num_nets
        dev = self.g.device
        if getattr(self, "_nets_over_out", None) is None or self._nets_over_out[0].numel() != k:
            self._nets_over_out = (torch.empty(k, dtype=torch.float64, device=dev),
                                   torch.empty(k, dtype=torch.uint8, device=dev))
        sums, hit = self._nets_over_out
        g = self.g
        _lib.check(self.ops.lib.ogr_nets_overuse(
            st.length.data_ptr(), st.arcs.data_ptr(), k, int(st.arcs.shape[1]), self.s.present.data_ptr(),
            self.s.capacity.data_ptr(), g.edge_src.data_ptr(), g.indices.data_ptr(), int(bool(canonical_only)),
            sums.data_ptr(), hit.data_ptr(), self.ops._sp()), "ogr_nets_overuse")
        lengths = st.length.cpu().numpy()
        s_h = sums.cpu().numpy()
        h_h = hit.cpu().numpy().astype(bool)
        self.ops.counters["launches"] += 1
        self.ops.counters["d2h_bytes"] += 13 * k
        rows = np.flatnonzero(lengths >= 2)
        names = [self._task_names[r] for r in rows.tolist()]
        return names, s_h[rows], h_h[rows]

    # ------------------------------------------------------------- tallies
    def _compute_overuse(self):
        over_sum, over_cnt, _, _, _ = self.ops.tally(canonical_only=True)
        return over_sum + self.pools.spatial_overuse(), over_cnt

    def _path_node_overuse(self):
        u = self.node_use[self.node_use > 1]
        return int(u.sum(dtype=np.int64)) - u.size, int(u.size)

    def _path_node_conflicts(self, shared_list=None):
        """Shared path nodes (``_detect_path_node_conflicts`` :10564-10606):
        (pairs of nets sharing a node, the shared nodes, shared-node count per net).
        In persistent mode the (node, slot) entries of the stored paths on
        shared nodes come from the device barrel scan (`shared_list`, or a
        scan made here); the trivially routed one-node nets are added on the
        host.  Otherwise the host flat view of all paths is filtered."""
        shared = self.node_use > 1
        if not shared.any():
            return set(), set(), {}
        if getattr(self, "store", None) is not None:
            if shared_list is None:
                shared_list = self._barrel_scan()[4]
            names = list(self._task_names)
            single = [(n, p[0]) for n, p in self.net_paths.items() if p and len(p) == 1]
            extra = [(len(names) + j, v) for j, (_, v) in enumerate(single) if shared[v]]
            names += [n for n, _ in single]
            nodes = shared_list[:, 0]
            owner = shared_list[:, 1]
            if extra:
                nodes = np.concatenate([nodes, np.fromiter((v for _, v in extra), dtype=np.int64, count=len(extra))])
                owner = np.concatenate([owner, np.fromiter((i for i, _ in extra), dtype=np.int64, count=len(extra))])
        else:
            F = self._flat()
            m = shared[F.nodes]
            names, nodes, owner = F.names, F.nodes[m], F.owner[m]
        K = max(1, len(names))
        key = _sorted_unique(nodes * K + owner)
        node, own = key // K, key % K
        cnt = np.bincount(own, minlength=K)
        scores = {names[i]: int(cnt[i]) for i in np.flatnonzero(cnt).tolist()}
        pairs = set()
        if node.size:
            first = np.ones(node.size, dtype=bool)
            first[1:] = node[1:] != node[:-1]
            starts = np.flatnonzero(first)
            size = np.diff(np.append(starts, node.size))
            pk = []
            for k in _sorted_unique(size[size > 1]).tolist():
                g = starts[size == k]
                ii, jj = np.triu_indices(k, 1)
                pk.append((own[g[:, None] + ii] * K + own[g[:, None] + jj]).ravel())
            if pk:
                for v in _sorted_unique(np.concatenate(pk)).tolist():
                    x, y = names[v // K], names[v % K]
                    pairs.add((x, y) if x <= y else (y, x))
            shared_nodes = set(node[starts].tolist())
        else:
            shared_nodes = set()
        return pairs, shared_nodes, scores

    def _barrel_scan(self):
        """The device barrel scan of the stored paths (ogr_barrel_scan):
        (conflicting hops, occ (node, net id)[], cnode (node, owner count,
        owner xor)[], member (node, net id)[], shared (node, slot)[]) as
        numpy arrays; the lists are grown and the scan repeated if a list
        outgrew them."""
        st, s = self.store, self.s
        k = st.num_nets
        dev = self.g.device
        if self._barrel_ids is None or self._barrel_ids[0] != len(self.net_id_map):
            ids = np.fromiter((self.net_id_map.get(n, -1) for n in self._task_names), dtype=np.int32, count=k)
            self._barrel_ids = (len(self.net_id_map), torch.from_numpy(ids).to(dev))
        ids = self._barrel_ids[1]
        if self._barrel_cap == 0:
            self._barrel_cap = 1 << 16
        while True:
            cap = self._barrel_cap
            if getattr(self, "_d_barrel", None) is None or self._d_barrel[0] != cap:
                self._d_barrel = (cap, torch.empty(2 * cap, dtype=torch.int32, device=dev),
                                  torch.empty(3 * cap, dtype=torch.int32, device=dev),
                                  torch.empty(2 * cap, dtype=torch.int32, device=dev),
                                  torch.empty(2 * cap, dtype=torch.int32, device=dev),
                                  torch.zeros(5, dtype=torch.int64, device=dev))
            _, occ, cn, mem, sh, counts = self._d_barrel
            self._barrel_stamp += 1
            _lib.check(self.ops.lib.ogr_barrel_scan(
                st.length.data_ptr(), st.path.data_ptr(), ids.data_ptr(), k, st.slot_cap, self.nx, self.ny,
                s.owner_count.data_ptr(), s.owner_xor.data_ptr(), s.path_node_use.data_ptr(),
                self._d_barrel_mark.data_ptr(), self._barrel_stamp, cap, occ.data_ptr(), cn.data_ptr(),
                mem.data_ptr(), sh.data_ptr(), counts.data_ptr(), self.ops._sp()), "ogr_barrel_scan")
            self.ops.counters["launches"] += 2
            c = counts.cpu().numpy()
            self.ops.counters["d2h_bytes"] += 40
            need = int(c[1:].max())
            if need <= cap:
                break
            self._barrel_cap = 1 << int(np.ceil(np.log2(need)))
        n1, n2, n3, n4 = (int(x) for x in c[1:])
        out = (occ[:2 * n1].view(n1, 2), cn[:3 * n2].view(n2, 3), mem[:2 * n3].view(n3, 2), sh[:2 * n4].view(n4, 2))
        out = tuple(t.cpu().numpy().astype(np.int64) for t in out)
        self.ops.counters["d2h_bytes"] += 4 * (2 * n1 + 3 * n2 + 2 * n3 + 2 * n4)
        return (int(c[0]),) + out

    def _detect_barrels(self):
        """Exact barrel conflicts + shared path nodes (``_detect_barrel_conflicts`` :10778-11111).

        In persistent mode the per-hop work runs on the device over the path
        store (ogr_barrel_scan) and only the conflicting endpoints, the conflict
        nodes' barrel members and the shared path nodes come back; otherwise
        it runs on the host over the flat view of the paths.  Both give
        exact = the number of hops with a conflicting endpoint, the conflict
        nodes (their history), and per (conflicting endpoint, other member of
        its barrel) one score for both nets and one exact pair."""
        self.barrel_conflict_nets, self.barrel_owner_nets, self.barrel_victim_nets = set(), set(), set()
        self.physical_scores = defaultdict(int)
        self.exact_pairs = set()
        device = getattr(self, "store", None) is not None
        shared_list = None
        exact = 0
        if device:
            exact, occ, cn, mem, shared_list = self._barrel_scan()
            if exact:
                qn, qv = occ[:, 0], occ[:, 1]
                cnodes = _sorted_unique(cn[:, 0])
                K = max(1, len(self.net_id_map))
                one = cn[cn[:, 1] == 1]
                key = _sorted_unique(np.concatenate([one[:, 0] * K + one[:, 2], mem[:, 0] * K + mem[:, 1]]))
                vn, vid = key // K, key % K
        else:
            F = self._flat()
            if F.names:
                own = self._via_owner_of(F)
                p = np.flatnonzero(F.same)          # hop (p, p+1) of one net
                s, d = F.nodes[p], F.nodes[p + 1]
                en = F.ids[F.owner[p]]
                so, do = own[s], own[d]
                sc = (so != -1) & (so != en)
                dc = (do != -1) & (do != en)
                cm = sc | dc
                exact = int(cm.sum())
                if exact:
                    qn = np.concatenate([s[sc], d[dc]])
                    qv = np.concatenate([en[sc], en[dc]])
                    cnodes = _sorted_unique(qn)
                    vn, vid = F.via_members()
        if exact:
            names_by_id = list(self.net_id_map)
            victims = _sorted_unique(qv)
            self._accumulate_history(cnodes)
            lo = np.searchsorted(vn, cnodes, "left")
            hi = np.searchsorted(vn, cnodes, "right")
            owners = _sorted_unique(vid[_expand_ranges(lo, hi)])
            # every (conflicting endpoint, other member of its barrel) counts
            # once for both nets and names one exact pair
            lo = np.searchsorted(vn, qn, "left")
            hi = np.searchsorted(vn, qn, "right")
            j = _expand_ranges(lo, hi)
            victim = np.repeat(qv, hi - lo)
            other = vid[j]
            keep = other != victim
            victim, other = victim[keep], other[keep]
            K = len(names_by_id)
            cnt = np.bincount(victim, minlength=K) + np.bincount(other, minlength=K)
            for i in np.flatnonzero(cnt).tolist():
                self.physical_scores[names_by_id[i]] += int(cnt[i])
            for v in _sorted_unique(np.minimum(victim, other) * K + np.maximum(victim, other)).tolist():
                x, y = names_by_id[v // K], names_by_id[v % K]
                self.exact_pairs.add((x, y) if x <= y else (y, x))
            vset = {names_by_id[i] for i in victims.tolist()}
            oset = {names_by_id[i] for i in owners.tolist()}
            self.barrel_victim_nets = vset
            self.barrel_owner_nets = oset
            self.barrel_conflict_nets = vset | oset
        pairs, shared, pscores = self._path_node_conflicts(shared_list)
        self.path_node_pairs = set(pairs)
        self.path_node_scores = dict(pscores)
        if shared:
            for name, sc_ in pscores.items():
                self.physical_scores[name] += int(sc_)
            self.barrel_conflict_nets.update({n for p_ in pairs for n in p_})
            self._accumulate_history(np.fromiter(shared, dtype=np.int64, count=len(shared)))
        return exact + len(shared)

    # ------------------------------------------------------------- device steps
    def _update_pool_presence(self):
        """The via-present EMA and z prefix (:6279-6303), on the device arrays
        in persistent mode."""
        P = self.pools
        if P.device_spatial is None:
            P.update_presence()
            return
        seg = P.has_seg
        _lib.check(self.ops.lib.ogr_via_pools_presence(
            self.nx, self.ny, self.nz, self._d_col_use.data_ptr(), self._d_col_cap.data_ptr(),
            self._d_seg_use.data_ptr() if seg else None, self._d_seg_cap.data_ptr() if seg else None,
            self._d_col_pres.data_ptr(), self._d_seg_pres.data_ptr() if seg else None,
            self._d_seg_prefix.data_ptr() if seg else None, self.ops._sp()), "ogr_via_pools_presence")
        self.ops.counters["launches"] += 1

    def _upload_pools(self, pres_fac, penalty, block):
        P = self.pools
        dev = self.g.device
        on_device = P.device_spatial is not None        # use / presence already on the device
        if penalty and not on_device:
            self._d_col_pres.copy_(torch.from_numpy(np.ascontiguousarray(P.col_pres)))
            if P.has_seg:
                self._d_seg_prefix.copy_(torch.from_numpy(np.ascontiguousarray(P.seg_prefix)))
        if penalty:
            lb = self.layer_bias
            k = 0.20
            zs = np.arange(self.nz)
            sb = lb[zs]
            disc = (1.0 - k * np.maximum(sb, 0.0))[:, None] * (1.0 + 0.5 * k * np.maximum(lb[zs], 0.0))[None, :]
            self._d_disc.copy_(torch.from_numpy(np.asarray(disc, dtype=np.float64).ravel()))
        if block and not on_device:
            self._d_col_use.copy_(torch.from_numpy(np.ascontiguousarray(P.col_use)))
            if P.has_seg:
                self._d_seg_use.copy_(torch.from_numpy(np.ascontiguousarray(P.seg_use)))
        g = self.g
        seg = P.has_seg
        _lib.check(self.ops.lib.ogr_via_pools_apply(
            self.E, self.nx, self.ny, self.nz, g.edge_src.data_ptr(), g.indices.data_ptr(), g.edge_kind.data_ptr(),
            self._d_col_pres.data_ptr(), self._d_seg_prefix.data_ptr() if seg else None,
            self._d_col_use.data_ptr(), self._d_col_cap.data_ptr(),
            self._d_seg_use.data_ptr() if seg else None, self._d_seg_cap.data_ptr() if seg else None,
            self._d_disc.data_ptr(), float(np.float32(1.0)), float(np.float32(1.0)), float(np.float32(pres_fac)),
            int(bool(penalty)), int(bool(block)), self.s.total_cost.data_ptr(), self.ops._sp()),
            "ogr_via_pools_apply")
        self.ops.sync_rcost()

    def _layer_bias_for_costs(self):
        """``_compute_layer_bias`` (:8451-8534) from exact device tallies."""
        _, _, _, _, units = self.ops.tally(canonical_only=True)
        per_layer = units.astype(np.float64) / float(1 << 23)
        maxv = float(per_layer.max())
        if maxv <= 1e-9:
            raw = np.ones(self.nz, dtype=np.float32)
        else:
            raw = 1.0 + 0.75 * (per_layer / maxv)
        if self._layer_bias_ema is None:
            self._layer_bias_ema = raw.astype(np.float32)
        else:
            self._layer_bias_ema = (0.88 * self._layer_bias_ema + (1.0 - 0.88) * raw).astype(np.float32)
        self._layer_bias_ema = np.clip(self._layer_bias_ema, 1.0, 1.80)
        return self._layer_bias_ema

    # ------------------------------------------------------------- routing
    def _search(self, name, src, dst, bonus, full_graph):
        cfg = self.config
        radius = max(60, int(self._manhattan(src, dst) * 0.75 + bonus * 2.0))
        net = self.ops.net_args(
            self._net_id(name), src, dst, full_graph=full_graph,
            max_depth=min(int(radius + bonus * 2.0), 80), halo=min(16, 2 + int(max(0.0, bonus) / 0.6)),
            max_roi_nodes=MAX_ROI_NODES, pres_fac=self._pres_fac_now, owner_base=cfg.owner_penalty_base,
            path_base=cfg.path_node_penalty_base, hist_pen=cfg.node_history_penalty,
            freeze_weight=cfg.portal_cleanup_node_penalty if self.freeze else None, penalty=True)
        t = time.perf_counter()
        path = self.ops.find_path(net, engine=self.full_engine if full_graph else "cta")
        self.stats["search_s"] += time.perf_counter() - t
        self.stats["searches"] += 1
        st = self.ops.stats.cpu().numpy()
        self.stats["arcs"] += int(st[0])
        self.stats["pops"] += int(st[1])
        self.ops.stats.zero_()
        return path

    def _manhattan(self, s, d):
        sx, sy, _ = self.idx_to_coord(s)
        dx, dy, _ = self.idx_to_coord(d)
        return abs(dx - sx) + abs(dy - sy)

    def _apply(self, name, path, sign, live):
        edges = self.ops.apply_path(path, self._net_id(name), sign, self._present_pres_fac, live=live)
        self._mark_nodes(name, path, sign)
        if self.store is not None:
            self.store.set_path(self._task_index[name], path if sign > 0 else [], edges if sign > 0 else None)
        return edges

    def _order_nets(self, tasks):
        _, over_idx, over_val = self._over_map()
        names, sums, _ = self._edge_over(over_idx, over_val)
        cong_of = {n: float(sums[i]) / max(1, self.net_to_edges[n].size) for i, n in enumerate(names)}
        scores = []
        d3 = self._dist3 if getattr(self, "_dist3", None) is not None else {}
        self._dist3 = d3
        for name, (s, d) in tasks.items():
            dist = d3.get(name)
            if dist is None:
                sx, sy, sz = self.idx_to_coord(s)
                dx, dy, dz = self.idx_to_coord(d)
                dist = d3[name] = abs(dx - sx) + abs(dy - sy) + abs(dz - sz)
            cong = cong_of.get(name, 0.0)
            scores.append((dist * 3 * (cong + 1), name))
        owners, victims = self.barrel_owner_nets, self.barrel_victim_nets
        scores.sort(key=lambda it: (2 if it[1] in owners and it[1] not in victims else 1 if it[1] in owners else 0,
                                    it[0], it[1]), reverse=True)
        rotation = 0
        if not owners and not victims:
            rotation = random.Random(42 + int(self.iteration)).randint(0, min(5, len(scores) // 10))
        ordered = [n for _, n in scores]
        if rotation > 0:
            ordered = ordered[rotation:] + ordered[:rotation]
        return ordered

    def _autotune(self, tasks):
        """full_engine="auto": time the job's longest full-graph nets under
        each engine / grid, and a spread of its ROI nets under each lanes per
        node, on the current costs, and keep the fastest (the choices change
        no result)."""
        from . import autotune
        nets = autotune.sample_full_nets(tasks, self._manhattan, ROI_THRESHOLD_STEPS)
        roi_nets = autotune.sample_roi_nets(tasks, self._manhattan, ROI_THRESHOLD_STEPS)
        self.tuning = autotune.tune(self.ops, self.lattice, nets, roi_nets)
        self.full_engine = self.tuning.full_engine
        self.full_tile_delta = self.tuning.full_tile_delta
        # the timing searches added to the device counters; the job's own start at zero
        self.ops.stats.zero_()

    def _route_all(self, tasks, all_tasks):
        cfg = self.config
        self.full_graph_fallback_count = 0
        bonus = self.stagnation_counter * 0.6
        ordered = self._order_nets(tasks)
        live = bool(cfg.live_present_costs)
        if live:
            self.ops.live_begin(self._present_pres_fac)
        if self.full_engine_request == "auto" and self.tuning is None:
            self._autotune(all_tasks)
        # the engine knob is per host thread, shared by the routers of a thread:
        # every pass sets this router's choice
        from . import autotune
        autotune.full_tile(1 if self.full_tile_delta > 0 else 0, self.full_tile_delta)
        if self.mode == "persistent":
            return self._route_all_pass(tasks, all_tasks, ordered, bonus, live)
        for name in ordered:
            src, dst = tasks[name]
            if name in self.net_paths and self.net_paths[name]:
                self._apply(name, self.net_paths[name], -1, live)
                self._clear_tracking(name)
            full = self._manhattan(src, dst) >= ROI_THRESHOLD_STEPS
            path = self._search(name, src, dst, bonus, full)
            if self.search_log is not None:
                self.search_log.append((self.iteration, name, "full" if full else "roi", path))
            if (not path or len(path) <= 1) and self.full_graph_fallback_count < 5:
                path = self._search(name, src, dst, bonus * 2, False)
                if self.search_log is not None:
                    self.search_log.append((self.iteration, name, "fallback", path))
                self.full_graph_fallback_count += 1
            if path and len(path) > 1:
                edges = self._apply(name, path, +1, live)
                self.net_paths[name] = path
                self._update_tracking(name, edges)
            else:
                self.net_paths[name] = []
                self._clear_tracking(name)
        routed = sum(1 for p in self.net_paths.values() if p)
        return routed, len(all_tasks) - routed

    def _net_table(self, bonus):
        """Per-net search parameters of this pass (``extract_roi`` :2240-2255).
        Endpoints, Manhattan lengths and the full-graph flag are fixed for a
        job and uploaded once; ids once every net has one (they are assigned
        in first-use order, as before: this pass's order, then task order);
        ROI depth and halo whenever the stagnation bonus changes."""
        names = self._task_names
        n = len(names)
        dev = self.g.device
        c = self._table_cache
        if c is None or c["names"] is not names:
            ends = np.asarray([self._tasks_all[nm] for nm in names], dtype=np.int64).reshape(n, 2)
            r = ends % self.plane
            y, x = np.divmod(r, self.nx)
            dist = np.abs(x[:, 1] - x[:, 0]) + np.abs(y[:, 1] - y[:, 0])
            full = (dist >= ROI_THRESHOLD_STEPS).astype(np.int32)
            c = self._table_cache = dict(
                names=names, dist=dist, full_host=full.astype(np.uint8), bonus=None, nids=-1,
                src=torch.from_numpy(ends[:, 0].astype(np.int32)).to(dev),
                dst=torch.from_numpy(ends[:, 1].astype(np.int32)).to(dev),
                full=torch.from_numpy(full).to(dev))
        if c["nids"] != len(self.net_id_map):
            nid = np.fromiter((self._net_id(nm) for nm in names), dtype=np.int32, count=n)
            c["id"] = torch.from_numpy(nid).to(dev)
            c["nids"] = len(self.net_id_map)
        if c["bonus"] != bonus:
            depth = np.empty(2 * n, dtype=np.int32)
            halo = np.empty(2 * n, dtype=np.int32)
            for j, b in enumerate((bonus, bonus * 2)):
                radius = np.maximum(60, np.trunc(c["dist"] * 0.75 + b * 2.0).astype(np.int64))
                depth[j::2] = np.minimum(np.trunc(radius + b * 2.0).astype(np.int64), 80)
                halo[j::2] = min(16, 2 + int(max(0.0, b) / 0.6))
            c["depth"] = torch.from_numpy(depth).to(dev)
            c["halo"] = torch.from_numpy(halo).to(dev)
            c["bonus"] = bonus
        return {k: c[k] for k in ("src", "dst", "id", "full", "depth", "halo", "full_host")}

    def _route_all_pass(self, tasks, all_tasks, ordered, bonus, live):
        """The per-net loop of ``_route_all`` as one device launch."""
        cfg = self.config
        for name in ordered:
            self._net_id(name)
        table = self._net_table(bonus)
        order = np.asarray([self._task_index[n] for n in ordered], dtype=np.int32)
        w = float(cfg.owner_penalty_base) * float(self._pres_fac_now)
        if self.freeze:
            w = max(w, float(cfg.portal_cleanup_node_penalty))
        t0 = time.perf_counter()
        order_full = table["full_host"][order] if self.full_engine == "grid" else None
        status, st = route_pass(self.ops, self.store, table, order, fallback_quota=5, max_roi_nodes=MAX_ROI_NODES,
                                owner_weight=w, path_weight=float(cfg.path_node_penalty_base) * float(self._pres_fac_now),
                                history_weight=cfg.node_history_penalty, pres_fac=self._present_pres_fac, live=live,
                                order_full=order_full)
        self.stats["search_s"] += time.perf_counter() - t0
        self.stats["searches"] += len(ordered) + int(np.count_nonzero(status & 2))
        self.stats["arcs"] += int(st[0])
        self.stats["pops"] += int(st[1])
        self.full_graph_fallback_count = int(np.count_nonzero(status & 2))
        # the routed nets' paths, packed on the device to their exact lengths
        lengths = self.store.length.cpu().numpy()
        lens = np.where((status & 1) == 0, lengths[order], 0).astype(np.int64)
        offs = np.concatenate([[0], np.cumsum(lens)])
        tot = int(offs[-1])
        packed = np.zeros(0, dtype=np.int32)
        if tot:
            dev = self.g.device
            rows_d = torch.as_tensor(order.astype(np.int64), device=dev)
            lens_d = torch.as_tensor(lens, device=dev)
            rep = torch.repeat_interleave(rows_d, lens_d, output_size=tot)
            starts = torch.repeat_interleave(torch.as_tensor(offs[:-1], device=dev), lens_d, output_size=tot)
            pos = torch.arange(tot, device=dev, dtype=torch.int64) - starts
            flat = rep * self.store.slot_cap + pos
            packed = self.store.path.view(-1).index_select(0, flat).cpu().numpy()
            self.ops.counters["h2d_bytes"] += 16 * len(order)
        self.ops.counters["d2h_bytes"] += 4 * lengths.size + 4 * tot
        paths = self._net_paths
        olds, news = [], []
        for k, name in enumerate(ordered):
            old = paths.get(name)
            if old:
                olds.append(paths.array(name))
                self._clear_tracking(name)
            n = int(lens[k])
            if n >= 2:
                arr = packed[offs[k]:offs[k] + n].astype(np.int64)
                news.append(arr)
                paths.set_path(name, arr.tolist(), arr)
                self._update_tracking(name, 2 * (n - 1))
            else:
                self.net_paths[name] = []
                self._clear_tracking(name)
            if self.search_log is not None:
                self.search_log.append((self.iteration, name, "pass", self.net_paths[name] or None))
        # path-node use: every old path off, every new path on (the counts are
        # exact, so the order of the per-net updates does not matter)
        self._mark_many(olds, -1)
        self._mark_many(news, +1)
        routed = sum(1 for p in self.net_paths.values() if p)
        return routed, len(all_tasks) - routed

    # ------------------------------------------------------------- hotset
    def _via_keeper_threshold(self):
        routed = sum(bool(p) for p in self.net_paths.values())
        step = max(1, int(self.config.via_keeper_rotation_nets_per_step))
        return max(0, int(self.config.via_keeper_rotation_overuse_threshold)) * max(1, int(np.ceil(routed / step)))

    def _find_via_pool_offenders(self):
        P = self.pools
        col_over = P.col_use > P.col_cap
        col_over = col_over if np.any(col_over) else None
        seg_over = None
        if P.has_seg:
            m = P.seg_use > P.seg_cap
            seg_over = m if np.any(m) else None
        if col_over is None and seg_over is None:
            self._via_pool_keepers, self._via_pool_member_state, self._via_pool_keeper_stagnation = {}, {}, {}
            return set()
        members = self._via_pool_members(col_over, seg_over)
        rotation_allowed = P.spatial_overuse() <= self._via_keeper_threshold()
        nk, nm, ns, off = {}, {}, {}, set()
        for r, mem in sorted(members.items()):
            kind, x, y, *tail = r
            if kind == "col":
                capv, obs = int(P.col_cap[x, y]), int(P.col_use[x, y])
            else:
                capv, obs = int(P.seg_cap[x, y, tail[0]]), int(P.seg_use[x, y, tail[0]])
            capv = max(0, capv)
            state = frozenset(mem)
            nm[r] = state
            stagn = int(self._via_pool_keeper_stagnation.get(r, 0)) + 1 \
                if self._via_pool_member_state.get(r) == state else 0
            prev = [n for n in self._via_pool_keepers.get(r, ()) if n in mem][:capv]
            remaining = sorted(mem - set(prev))
            keepers = tuple(prev + remaining[:max(0, capv - len(prev))])
            if rotation_allowed and stagn >= 2 and 0 < capv < len(mem) and prev:
                ordered = sorted(mem)
                st0 = (ordered.index(prev[0]) + 1) % len(ordered)
                keepers = tuple(ordered[(st0 + o) % len(ordered)] for o in range(capv))
                stagn = 0
            ns[r] = stagn
            nk[r] = keepers
            off.update(mem - set(keepers))
            if obs > len(mem):
                off.update(mem)
        self._via_pool_keepers, self._via_pool_member_state, self._via_pool_keeper_stagnation = nk, nm, ns
        return off

    def _via_pool_members(self, col_over, seg_over):
        """Nets whose via hops use an over-full via column ("col", x, y) or a
        via segment ("seg", x, y, z-1) of z in [clamp(zlo), clamp(zhi))."""
        P = self.pools
        F = self._flat()
        members = defaultdict(set)
        h = F.hops
        if h.size == 0:
            return members
        names = F.names
        ru = F.r[h]
        net = F.owner[h]
        zu, zv = F.z[h], F.z[h + 1]
        y, x = np.divmod(ru, self.nx)
        pairs = set()
        if col_over is not None:
            m = col_over[x, y]
            for xx, yy, nn in zip(x[m].tolist(), y[m].tolist(), net[m].tolist()):
                pairs.add((("col", xx, yy), nn))
        if seg_over is not None:
            zl = np.clip(np.minimum(zu, zv), 1, self.nz - 2)
            zh = np.clip(np.maximum(zu, zv), 1, self.nz - 2)
            cnt = np.maximum(zh - zl, 0)
            if cnt.sum() > 0:
                rep = np.repeat(np.arange(cnt.size), cnt)
                zz = zl[rep] + (np.arange(int(cnt.sum())) - np.repeat(np.cumsum(cnt) - cnt, cnt)) - 1
                ok = (zz >= 0) & (zz < P.segZ)
                xs, ys, ns, zz = x[rep][ok], y[rep][ok], net[rep][ok], zz[ok]
                m = seg_over[xs, ys, zz]
                for xx, yy, z1, nn in zip(xs[m].tolist(), ys[m].tolist(), zz[m].tolist(), ns[m].tolist()):
                    pairs.add((("seg", xx, yy, z1), nn))
        for res, nn in pairs:
            members[res].add(names[nn])
        return members

    def _effective_cap(self, t):
        cfg = self.config
        base = _history_hotset_cap(t)
        if t > int(cfg.slow_progress_min_overuse) and self.iteration <= int(getattr(self, "_hotset_rate_boost_until", 0)):
            init = max(1, int(cfg.slow_progress_hotset_cap))
            mx = max(init, int(cfg.slow_progress_hotset_cap_max))
            ga = max(1, int(cfg.slow_progress_hotset_growth_after))
            ev = max(1, int(getattr(self, "_slow_progress_event_count", 1)))
            return max(base, min(mx, init * (2 ** max(0, ev - ga + 1))))
        return base

    def _bounded_cap(self, t):
        base = _history_hotset_cap(t)
        eff = self._effective_cap(t)
        conf = max(1, int(self.config.hotset_cap))
        if eff > base:
            conf = max(conf, eff)
        cap = min(conf, eff)
        floor = int(self.config.hotset_cap_floor)
        if floor > 0 and t > 2048:
            cap = max(cap, floor)
        return cap

    def _physical_hotset(self):
        off = set(self.barrel_conflict_nets)
        cfg = self.config
        mx = max(1, int(cfg.physical_hotset_cap))
        mn = min(mx, max(1, int(cfg.physical_hotset_min)))
        scale = max(1.0, float(cfg.physical_conflicts_per_hotset_net))
        cap = min(mx, max(mn, int(np.ceil(max(0, self.barrel_count) / scale))))
        if len(off) <= cap:
            return off
        return set(sorted(off, key=lambda n: (-int(self.physical_scores.get(n, 0)), str(n)))[:cap])

    def _build_hotset(self, tasks, ripped):
        over_map, over_idx_arr, over_val_arr = self._over_map()
        over_idx = set(over_idx_arr.tolist())
        via_off = self._find_via_pool_offenders()
        pscores = {n: int(s) for n, s in self.path_node_scores.items() if n in tasks and int(s) > 0}
        poff = set(pscores)
        total_neg = self._compute_overuse()[0] + self._path_node_overuse()[0]
        thr = int(self.config.portal_cleanup_edge_threshold)
        if self.config.physical_cleanup_overuse_threshold is not None:
            thr = max(thr, int(self.config.physical_cleanup_overuse_threshold))
        if not over_idx:
            unrouted = {n for n in tasks if not self.net_paths.get(n)}
            phys = self._physical_hotset() if total_neg <= thr else set()
            hot = unrouted | ripped | via_off | phys
            hot.update(_conflict_aware_hotset(sorted(poff, key=lambda n: (-pscores[n], str(n))), self.path_node_pairs,
                                              self._bounded_cap(total_neg), _exploration_fraction(total_neg),
                                              random.Random(42 + self.iteration)))
            self._last_hotset_size = len(hot)
            return hot
        enames, esums, ehit = self._edge_over(over_idx_arr, over_val_arr)
        over_sum_of = {n: float(esums[i]) for i, n in enumerate(enames) if ehit[i]}
        offenders = set(over_sum_of)
        offenders.update(poff)
        for n in tasks:
            self._net_clean_iters[n] = 0 if n in offenders else self._net_clean_iters.get(n, 0) + 1
        offenders -= {n for n in offenders if self._net_clean_iters.get(n, 0) >= 3}
        offenders |= ripped
        offenders |= via_off
        unrouted = {n for n in tasks if not self.net_paths.get(n)}
        scores = []
        for n in offenders:
            imp = float(pscores.get(n, 0))
            if n in self.net_to_edges:
                imp += over_sum_of.get(n, 0)
            scores.append((imp, n))
        for n in unrouted:
            if n not in offenders:
                scores.append((0.0, n))
        scores.sort(reverse=True)
        cap = self._bounded_cap(total_neg)
        rng = random.Random(42 + self.iteration)
        ranked = [n for _, n in scores if self.iteration - self._last_reroute_iter.get(n, -999) > 1]
        sel = _conflict_aware_hotset(ranked, self.path_node_pairs, cap, _exploration_fraction(total_neg), rng)
        for n in sel:
            self._last_reroute_iter[n] = self.iteration
        hot = set(sel)
        if len(over_idx) <= thr and total_neg <= thr:
            hot.update(self._physical_hotset())
        hot.update(unrouted)
        self._last_hotset_size = len(hot)
        return hot

    # ------------------------------------------------------------- state
    def _capture(self):
        return {n: list(p) for n, p in self.net_paths.items()}

    def _restore(self, state):
        """``_restore_routing_state`` (:7806-7838): re-commit every path."""
        self.net_paths.clear()
        self.net_paths.update({n: list(p) for n, p in state.items()})
        self.s.present.zero_()
        self.s.path_node_use.zero_()
        self.s.owner_count.zero_()
        self.s.owner_xor.zero_()
        self.node_use.fill(0)
        self.net_to_edges.clear()
        self._eidx = None
        if self.store is not None:
            self.store.length.zero_()
        # every path committed in one launch (commits add exact counts, so the
        # state equals the reference's path-by-path re-commit)
        names = [n for n, p in self.net_paths.items() if p and len(p) >= 2]
        arrs = [self._net_paths.array(n) for n in names]
        ids = [self._net_id(n) for n in names]
        slots = [self._task_index[n] for n in names] if self.store is not None else None
        for n, a, edges in zip(names, arrs, self.ops.commit_paths(arrs, ids, self.store, slots)):
            self._mark_nodes(n, None, +1, a)
            self._update_tracking(n, edges)
        self._add_trivial_use()
        self._rebuild_via_usage()

    def _add_trivial_use(self):
        """Path-node use of the trivially routed one-node nets.  The reference
        rebuilds path_node_use from every path at the start of each iteration
        (``_rebuild_via_usage_from_committed`` :4614-4615 via
        ``_rebuild_path_node_use`` :4623-4633), so those nets count from
        iteration 1 on; commits and rip-ups keep the rest up to date."""
        single = [p[0] for p in self.net_paths.values() if p and len(p) == 1]
        if not single:
            return
        idx = np.asarray(single, dtype=np.int64)
        np.add.at(self.node_use, idx, 1)
        use = self.s.path_node_use
        use.index_add_(0, torch.from_numpy(idx).to(use.device),
                       torch.ones(idx.size, dtype=use.dtype, device=use.device))

    def _rebuild_via_usage(self):
        """Column / segment use from the current paths: on the device from the
        path store in persistent mode (the host keeps only the over-full pools
        and the spatial overuse sum), else on the host from the flat view."""
        if getattr(self, "store", None) is None:
            self.pools.rebuild(self._flat())
            return
        P, st = self.pools, self.store
        seg = P.has_seg
        while True:
            cap = int(self._d_pool_over.numel()) // 5
            _lib.check(self.ops.lib.ogr_via_pools_rebuild(
                st.length.data_ptr(), st.path.data_ptr(), st.num_nets, st.slot_cap, self.nx, self.ny, self.nz,
                self._d_pool_scratch.data_ptr(), self._d_col_use.data_ptr(),
                self._d_seg_use.data_ptr() if seg else None, self._d_col_cap.data_ptr(),
                self._d_seg_cap.data_ptr() if seg else None, self._d_spatial.data_ptr(),
                self._d_pool_over.data_ptr(), cap, self._d_pool_over_n.data_ptr(), self.ops._sp()),
                "ogr_via_pools_rebuild")
            n = int(self._d_pool_over_n.item())
            if n <= cap:
                break
            self._d_pool_over = torch.zeros(5 * (2 * n), dtype=torch.int32, device=self.g.device)
        over = self._d_pool_over[:5 * n].view(n, 5).cpu().numpy() if n else np.zeros((0, 5), dtype=np.int32)
        spatial = int(self._d_spatial.item())
        self.ops.counters["launches"] += 2
        self.ops.counters["d2h_bytes"] += 12 + 20 * n
        P.set_from_device(over, spatial)

    def _rip_top_k(self, k=20):
        over_map, over_idx_arr, over_val_arr = self._over_map()
        a_src, a_dst, _, _ = self._arc_attrs(over_idx_arr)
        keep = a_src < a_dst                         # canonical arcs (src < dst) only
        enames, esums, ehit = self._edge_over(over_idx_arr[keep] if keep.size else over_idx_arr,
                                              over_val_arr[keep] if keep.size else over_val_arr,
                                              canonical_only=True)
        over_sum_of = {n: float(esums[i]) for i, n in enumerate(enames) if ehit[i]}
        _, _, mscores = self._path_node_conflicts()
        self.path_node_scores = dict(mscores)
        cands = set(mscores)
        cands.update(over_sum_of)
        scores = []
        for n in cands:
            if not self.net_paths.get(n):
                continue
            imp = float(mscores.get(n, 0))
            if n in self.net_to_edges:
                imp += over_sum_of.get(n, 0)
            if imp > 0:
                scores.append((imp, n))
        scores.sort(key=lambda it: (-it[0], str(it[1])))
        ranked = [n for _, n in scores]
        victims = set()
        if ranked and k > 0:
            if not self._stagnation_victim_history:
                self._stagnation_victim_cursor = 0
            cnt = min(int(k), len(ranked))
            start = int(self._stagnation_victim_cursor) % len(ranked)
            victims = {ranked[(start + o) % len(ranked)] for o in range(cnt)}
            self._stagnation_victim_cursor = (start + cnt) % len(ranked)
            self._stagnation_victim_history = victims
        for n in victims:
            if self.net_paths.get(n) and n in self.net_to_edges:
                self._apply(n, self.net_paths[n], -1, live=False)
                self.net_paths[n] = []
                self._clear_tracking(n)
        return victims

    def _movable_components(self, pairs):
        adj = defaultdict(set)
        for a, b in pairs:
            if a != b:
                adj[a].add(b)
                adj[b].add(a)
        movable, eligible = set(), set(adj)
        while eligible:
            n = min(eligible, key=lambda c: (self._cleanup_move_counts[c], -len(adj[c]), c))
            movable.add(n)
            eligible.discard(n)
            eligible.difference_update(adj[n])
        for n in movable:
            self._cleanup_move_counts[n] += 1
        return movable

    def _layer_congestion(self, idx, val):
        if idx.size == 0:
            return {}
        lays = self._arc_attrs(idx)[2]
        out = {}
        for z in range(1, self.nz + 1):
            m = lays == z
            if np.any(m):
                out[z] = float(np.sum(val[m]))
        return out

    # ------------------------------------------------------------- public API
    def _parse_requests(self, requests):
        """``_parse_requests`` (:4386-4467) for ``(name, src, dst)`` tuples:
        src == dst is routed trivially (``net_paths[name] = [src]``, no task);
        endpoints that are not Python ints are skipped, as the reference skips
        them.  Nets given by pads need the reference's pad portals, which this
        router does not plan, so they raise."""
        tasks = {}
        for r in requests:
            if isinstance(r, tuple) and len(r) == 3:
                name, src, dst = r
                if isinstance(src, int) and isinstance(dst, int):
                    if src != dst:
                        tasks[name] = (src, dst)
                    else:
                        self.net_paths[name] = [src]
            elif hasattr(r, "name") and hasattr(r, "pads"):
                raise TypeError("nets given by pads need pad portals; pass (name, src_node, dst_node) tuples")
        return tasks

    @staticmethod
    def _no_routable_nets(requests) -> Dict:
        """The reference's result when no request yields a task (:4355-4381)."""
        if not requests:
            return {}
        ids = [str(getattr(r, "name", r[0] if isinstance(r, tuple) and r else "unknown")) for r in requests]
        return {'success': False, 'converged': False, 'nets_routed': 0, 'total_nets': len(requests),
                'iterations': 0, 'total_time_s': 0.0, 'iteration_metrics': [], 'failed_nets': len(requests),
                'overuse_sum': 0, 'overuse_edges': 0, 'barrel_conflicts': 0, 'excluded_nets': len(requests),
                'excluded_net_ids': ids, 'error_code': 'NO-ROUTABLE-NETS',
                'message': 'No routable nets were produced from the requests'}

    def route_multiple_nets(self, requests, progress_cb=None, iteration_cb=None) -> Dict:
        if self.lattice is None:
            raise RuntimeError("initialize_graph() first")
        tasks = self._parse_requests(requests)
        if not tasks:
            return self._no_routable_nets(requests)
        self._tasks_all = tasks
        self._task_names = list(tasks)
        self._task_index = {n: i for i, n in enumerate(self._task_names)}
        self._barrel_ids = None              # the store slots' net ids, rebuilt for this job
        self._table_cache = None             # the pass's per-net parameters, rebuilt for this job
        self._dist3 = None
        if self.mode == "persistent":
            if self.store is None or self.store.num_nets != len(tasks):
                self.store = PathStore(self.g, len(tasks),
                                       window_slots=self.window_slots if self.mode == "persistent" else 0)
            self.store.length.zero_()
        self._add_trivial_use()
        return self._negotiate(tasks, progress_cb, iteration_cb)

    def _derive(self, tasks):
        """``analyze_board_characteristics`` + ``derive_routing_parameters`` +
        ``apply_derived_parameters`` (board_analyzer.py:151-305,
        parameter_derivation.py:51-278)."""
        cfg = self.config
        pitch = self.lattice.pitch
        width = self.bounds[2] - self.bounds[0]
        height = self.bounds[3] - self.bounds[1]
        nsig = max(0, self.nz - 2)
        chans = nsig * int(width / pitch) * int(height / pitch)
        hpwl = 0.0
        for _, (s, d) in tasks.items():
            sx, sy, _ = self.idx_to_coord(s)
            dx, dy, _ = self.idx_to_coord(d)
            hpwl += abs(dx - sx) * pitch + abs(dy - sy) * pitch
        rho = (hpwl * 1.3) / max(1.0, chans * pitch * 0.75)
        L, N = nsig, len(tasks)
        if rho < 0.6:
            mult, pmax = 1.15, 6.0
        elif rho < 0.9:
            mult, pmax = 1.12, 7.0
        elif rho < 1.2:
            mult, pmax = 1.10, 8.0
        else:
            mult, pmax = 1.08, 10.0
        pmax *= 0.75 if L <= 12 else 1.25 if L >= 25 else 1.0
        bonus = 6.0 if L <= 10 else 4.0 if L <= 15 else 2.0 if L <= 25 else 0.0
        pct = 0.25 if rho < 0.7 else 0.20 if rho < 1.0 else 0.15 if rho < 1.3 else 0.12
        patience = 5 if rho < 0.8 else 6 if rho < 1.1 else 8
        if L <= 12:
            patience = max(patience, 7)
        cfg.pres_fac_init, cfg.pres_fac_mult, cfg.pres_fac_max = 1.0, mult, pmax
        cfg.hist_cost_weight = 8.0 + bonus + 6.0 * max(0.0, min(1.0, rho - 0.7))
        cfg.hist_gain = 0.20 + 0.15 * max(0.0, min(1.0, rho - 0.8))
        cfg.history_decay = 1.0
        cfg.hotset_cap = max(32, min(int(N * pct), int(N * 0.30)))
        cfg.via_cost = 0.5
        cfg.stagnation_patience = patience
        if "max_iterations" not in cfg._explicit:
            cfg.max_iterations = max(cfg.max_iterations, 250)

    def _negotiate(self, tasks, progress_cb=None, iteration_cb=None):
        cfg = self.config
        self._derive(tasks)
        nsig = self.nz - 2
        pres_fac = float(cfg.pres_fac_init)
        pres_mult = float(os.getenv('ORTHO_PRES_FAC_MULT', cfg.pres_fac_mult))
        hist_gain = float(os.getenv('ORTHO_HIST_GAIN', cfg.hist_gain))
        hw_mult = 1.2 if nsig <= 12 else 1.0 if nsig <= 20 else 0.8
        floor = 32.0 if nsig <= 12 else 64.0 if nsig <= 20 else 128.0
        pres_max = float(os.getenv('ORTHO_PRES_FAC_MAX', max(float(cfg.pres_fac_max), floor)))
        hist_decay = float(os.getenv("ORTHO_HISTORY_DECAY",
                                     cfg.history_decay if cfg.history_decay is not None else 1.0))
        best_overuse, best_score, best_state, best_iter = float('inf'), None, None, 0
        stagnant = 0
        neg_hist = []
        self._slow_progress_event_count = 0
        self._hotset_rate_boost_until = 0
        last_slow = -1_000_000
        trial_ref_ceiling = trial_ref_frac = None
        trial_under = 0
        adaptive_limit = float(cfg.slow_progress_pres_fac_max)
        metrics = []
        jam = None
        failed = over_sum = over_cnt = negotiated = conflicts = 0
        t_start = time.time()
        s = self.s
        for it in range(1, cfg.max_iterations + 1):
            self.iteration = it
            t_it = time.time()
            self._pres_fac_now = pres_fac
            self._rebuild_via_usage()
            self._update_pool_presence()
            if it == 1:
                s.present_ema.copy_(s.present)
            self.ops.present_ema(0.40)
            lb = self._layer_bias_for_costs()
            vmult = 1.0
            if it >= 3 and self.pools.spatial_overuse() >= int(cfg.via_pressure_threshold):
                vmult = float(cfg.via_pressure_multiplier)
            elif pres_fac >= 64:
                _, idx, val = self._over_map()
                vo = float(val[self._arc_attrs(idx)[3]].sum()) if idx.size else 0.0
                to = float(val.sum())
                if to > 0:
                    vmult = 1.5 if vo / to > 0.7 else 0.5
            self.ops.update_costs(pres_fac, cfg.hist_cost_weight * hw_mult, vmult, cfg.base_cost_weight, lb)
            self._present_pres_fac = pres_fac
            self._upload_pools(pres_fac, penalty=True, block=it > 1)
            if cfg.reroute_only_offenders and it > 1:
                hot = self._build_hotset(tasks, self._last_ripped)
                sub = {k: v for k, v in tasks.items() if k in hot}
                self._last_ripped = set()
            else:
                sub = dict(tasks)
            work_scale = min(max(1.0, float(cfg.pressure_work_scale_max)),
                             max(1.0, len(sub) / max(1, int(cfg.pressure_reference_hotset)))) if it > 1 else 1.0
            routed, failed = self._route_all(sub, tasks)
            conflicts = self._detect_barrels()
            self.barrel_count = conflicts
            over_sum, over_cnt = self._compute_overuse()
            pno, _ = self._path_node_overuse()
            negotiated = over_sum + pno
            clean = over_sum == 0 and pno == 0
            thr = int(cfg.portal_cleanup_edge_threshold)
            if conflicts > 0 and over_cnt <= thr and negotiated <= thr:
                self._last_ripped = set(self._last_ripped) | set(self.barrel_conflict_nets)
            gate = thr if cfg.physical_cleanup_overuse_threshold is None else \
                max(thr, int(cfg.physical_cleanup_overuse_threshold))
            if conflicts > 0 and over_cnt <= gate and negotiated <= gate:
                if not self.freeze:
                    self.physical_cleanup_started = True
                self.freeze = True
                mov = self._movable_components(set(self.exact_pairs) | set(self.path_node_pairs))
                if mov:
                    self.barrel_conflict_nets = set(mov)
                    self._last_ripped = set(mov)
            elif conflicts == 0:
                self.freeze = False
                self._cleanup_move_counts.clear()
            elif self.freeze and (over_cnt > thr or negotiated > thr):
                self.freeze = False
            metrics.append({'iter': it, 'nets_routed': routed, 'overuse_sum': over_sum, 'overuse_edges': over_cnt,
                            'iter_time_s': round(time.time() - t_it, 4),
                            'total_time_s': round(time.time() - t_start, 4)})
            if self.trace is not None:
                self.trace.append(self._capture())
            score = (int(failed), int(over_sum) + int(pno), int(conflicts))
            if best_score is None or score < best_score:
                best_score, best_state, best_iter = score, self._capture(), it
                self._stagnation_victim_history = set()
                self._stagnation_victim_cursor = 0
            neg_hist.append(negotiated)
            window = max(1, int(cfg.slow_progress_window))
            slow, frac = self._rolling(neg_hist, window)
            if slow and it - last_slow >= window:
                last_slow = it
                self._slow_progress_event_count += 1
                self._hotset_rate_boost_until = it + window
                after = max(1, int(cfg.slow_progress_pressure_after))
                old_ceiling = pres_max
                rejected = None
                if (self._slow_progress_event_count >= 4 and self._last_hotset_size >= int(cfg.slow_progress_hotset_cap_max)
                        and frac is not None):
                    trial_ref_ceiling, trial_ref_frac, trial_under, rejected = self._pressure_trial(
                        old_ceiling, frac, trial_ref_ceiling, trial_ref_frac, trial_under)
                    if rejected is not None:
                        adaptive_limit = min(adaptive_limit, float(trial_ref_ceiling))
                        pres_max = min(pres_max, adaptive_limit)
                        pres_fac = min(pres_fac, pres_max)
                if self._slow_progress_event_count >= after and rejected is None:
                    mx = min(float(cfg.slow_progress_pres_fac_max), adaptive_limit)
                    pres_max = min(max(old_ceiling, mx), max(128.0, old_ceiling * 2.0))
                    pres_fac = min(pres_fac * 1.5, pres_max)
            if over_sum > 0:
                _, oidx, oval = self._over_map()
                by_layer = self._layer_congestion(oidx, oval)
                if by_layer and sum(by_layer.values()) > 0:
                    lo = np.array([by_layer.get(z, 0.0) for z in range(self.nz)])
                    mean = np.mean(lo[lo > 0]) + 1e-9
                    alpha, bmin, bmax = (0.20, 0.60, 1.80) if nsig <= 12 else \
                        (0.12, 0.75, 1.50) if nsig <= 20 else (0.08, 0.85, 1.20)
                    target = 1.0 + alpha * (lo / mean - 1.0)
                    self.layer_bias = np.clip(0.85 * self.layer_bias + 0.15 * target, bmin, bmax)
                    tot = sum(by_layer.values())
                    mz, mo = max(by_layer.items(), key=lambda x: x[1])
                    if jam is None:
                        jam = {'layer': None, 'count': 0, 'boost_until': 0}
                    if (mo / tot) * 100 >= 60.0:
                        if jam['layer'] == mz:
                            jam['count'] += 1
                        else:
                            jam = {'layer': mz, 'count': 1, 'boost_until': 0}
                        if jam['count'] >= 3 and it > jam['boost_until']:
                            self.layer_bias[mz] = min(self.layer_bias[mz] * 1.8, bmax)
                            jam['boost_until'] = it + 3
                    else:
                        jam = {'layer': None, 'count': 0, 'boost_until': 0}
            if clean:
                pres_fac = min(pres_fac, 10.0)
            hg = min(1.2, hist_gain * 1.25) if (it >= 8 and over_sum > 0) else hist_gain
            use_cap = os.getenv('ORTHO_NO_HISTORY_CAP', '0') == '0'
            self.ops.update_history(hg, cap_mult=15.0 if use_cap else 1.0, decay=hist_decay, use_cap=use_cap,
                                    use_raw_present=True)
            if progress_cb:
                try:
                    progress_cb(it, cfg.max_iterations, f"Iteration {it}")
                except Exception:
                    pass
            if iteration_cb:
                try:
                    tracks, vias = self._paths_geometry()
                    iteration_cb(it, tracks, vias, over_sum, over_cnt)
                except Exception:
                    pass
            if failed == 0 and clean:
                bc = self._detect_barrels()
                self.barrel_count = bc
                if bc == 0:
                    return {'success': True, 'converged': True, 'paths': self.net_paths, 'iterations': it,
                            'barrel_conflicts': 0, 'overuse_sum': 0, 'overuse_edges': 0, 'failed_nets': 0,
                            'iteration_metrics': metrics, 'total_time_s': round(time.time() - t_start, 4)}
            if negotiated < best_overuse:
                best_overuse, stagnant = negotiated, 0
            else:
                stagnant += 1
            if stagnant == 2:
                pres_fac = min(pres_fac * 1.5, pres_max)
            if stagnant >= cfg.stagnation_patience and it < cfg.max_iterations:
                if self.physical_cleanup_started or self.pools.spatial_overuse() > self._via_keeper_threshold():
                    stagnant = 0
                else:
                    cur = (int(failed), int(over_sum) + int(pno), int(conflicts))
                    if best_state is not None and best_score is not None and best_score < cur:
                        self._restore(best_state)
                    self.stagnation_counter += 1
                    self._last_ripped = self._rip_top_k(20)
                    self._freeze_pres_fac_until = it + 2
                    stagnant = 0
                    continue
            if it > self._freeze_pres_fac_until:
                pres_fac = min(pres_fac * (pres_mult ** work_scale), pres_max)
        cur = (int(failed), int(over_sum) + self._path_node_overuse()[0], int(self.barrel_count))
        restored = best_state is not None and best_score is not None and best_score < cur
        if restored:
            self._restore(best_state)
            failed = sum(1 for n in tasks if not self.net_paths.get(n))
            over_sum, over_cnt = self._compute_overuse()
            self.barrel_count = self._detect_barrels()
            negotiated = over_sum + self._path_node_overuse()[0]
        if 0 < negotiated <= 100:
            det = self._detail_pass(tasks, negotiated, pres_max)
            if det.get('success'):
                det['iteration_metrics'] = metrics
                det['best_iteration'] = best_iter
                return det
        final_barrels = self._detect_barrels()
        success = failed == 0 and over_sum == 0 and final_barrels == 0
        return {'success': success, 'converged': success, 'barrel_conflicts': final_barrels,
                'overuse_sum': over_sum, 'overuse_edges': over_cnt, 'failed_nets': failed,
                'path_node_overuse_sum': self._path_node_overuse()[0], 'nets_routed': len(tasks) - failed,
                'total_nets': len(tasks), 'iterations': len(metrics), 'best_iteration': best_iter,
                'restored_best_state': restored, 'iteration_metrics': metrics, 'paths': self.net_paths,
                'total_time_s': round(time.time() - t_start, 4)}

    def _rolling(self, values, window):
        cfg = self.config
        if len(values) < window + 1:
            return False, None
        start = float(values[-window - 1])
        if start <= max(0, int(cfg.slow_progress_min_overuse)):
            return False, None
        frac = max(0.0, (start - min(map(float, values[-window:]))) / max(1.0, start))
        return frac < max(0.0, float(cfg.slow_progress_min_fraction)), frac

    def _pressure_trial(self, cur_ceiling, cur_frac, ref_ceiling, ref_frac, under):
        cfg = self.config
        ceiling, frac = float(cur_ceiling), max(0.0, float(cur_frac))
        if ref_ceiling is None or ref_frac is None:
            return ceiling, frac, 0, None
        pc, pf = float(ref_ceiling), max(0.0, float(ref_frac))
        if ceiling <= pc:
            return pc, pf, 0, None
        if (pf <= 0.0 and frac > 0.0) or (pf > 0.0 and frac >= float(cfg.slow_progress_pressure_trial_min_ratio) * pf):
            return ceiling, frac, 0, None
        fails = int(under) + 1
        if fails >= max(1, int(cfg.slow_progress_pressure_trial_patience)):
            return pc, pf, 0, ceiling
        return pc, pf, fails, None

    def _detail_conflict_nets(self, edge_nets):
        return set(edge_nets) | set(self.path_node_scores) | set(self._find_via_pool_offenders()) | \
            set(self.barrel_conflict_nets)

    def _detail_pass(self, tasks, initial_overuse, pres_max_now):
        """``_detail_pass`` (:7593-7788)."""
        cfg = self.config
        best_state = self._capture()
        unrouted0 = sum(1 for n in tasks if not self.net_paths.get(n))
        best = (unrouted0, int(initial_overuse), int(self.barrel_count))
        _, over_idx_arr, over_val_arr = self._over_map()
        enames, _, ehit = self._edge_over(over_idx_arr, over_val_arr)
        hit_nets = {n for i, n in enumerate(enames) if ehit[i]}
        cn = {n for n in self.net_paths if self.net_paths[n] and n in hit_nets}
        cn = self._detail_conflict_nets(cn)
        if not cn:
            return {'success': False}
        ctasks = {n: tasks[n] for n in cn if n in tasks}
        dmax = max(float(cfg.pres_fac_max), float(pres_max_now))
        pres_fac = dmax * 0.5
        for _ in range(10):
            self.ops.update_costs(pres_fac, cfg.hist_cost_weight * 1.5, 0.3, cfg.base_cost_weight, None)
            self._present_pres_fac = pres_fac
            hot = self._build_hotset(ctasks, set())
            # the reference keeps the first 60 nets of the set (:7672); which ones
            # depends on Python's string hashing, here exactly as in the reference's
            # process (set PYTHONHASHSEED for reproducible runs)
            hot = set(list(hot)[:60])
            if not hot:
                hot = cn
            sub = {k: v for k, v in ctasks.items() if k in hot}
            old = self.stagnation_counter
            self.stagnation_counter += 3
            self._route_all(sub, tasks)
            self.stagnation_counter = old
            over_sum, _ = self._compute_overuse()
            bc = self._detect_barrels()
            self.barrel_count = bc
            pno, _ = self._path_node_overuse()
            unrouted = {n for n in tasks if not self.net_paths.get(n)}
            sc = (len(unrouted), int(over_sum) + int(pno), int(bc))
            if sc < best:
                best, best_state = sc, self._capture()
            cn = self._detail_conflict_nets(cn)
            ctasks.update({n: tasks[n] for n in cn if n in tasks})
            if over_sum + pno == 0:
                if unrouted:
                    cn = unrouted
                    ctasks.update({n: tasks[n] for n in unrouted})
                    continue
                if bc:
                    continue
                return {'success': True, 'converged': True, 'paths': self.net_paths}
            if self.trace is not None:
                self.trace.append(self._capture())
            self.ops.update_history(cfg.hist_gain * 2.0, cap_mult=15.0, decay=0.98, use_cap=True,
                                    use_raw_present=False)
            pres_fac = min(pres_fac * 1.5, dmax)
        self._restore(best_state)
        return {'success': False, 'overuse_sum': best[1]}


    # ------------------------------------------------------------- geometry (F4)
    def _paths_geometry(self):
        """``_generate_geometry_from_paths`` (:11439-11563) of the current paths;
        also what each iteration hands to ``iteration_cb`` (:7175-7227)."""
        from .geometry import GridGeometry, generate_geometry
        L = self.lattice
        axes = [L.allowed_axes(z) for z in range(L.nz)]
        return generate_geometry(self.net_paths, L.nx, L.ny, L.nz, axes, GridGeometry(self.bounds, L.pitch),
                                 self.config.layer_names, self.config.track_width, self.config.via_diameter,
                                 self.config.via_drill)

    def emit_geometry(self, board=None) -> Tuple[int, int]:
        """``emit_geometry`` (:11316-11404) for tuple requests: tracks and vias of
        every routed path; the export payload is kept only without overuse."""
        tracks, vias = self._paths_geometry()
        self._provisional_geometry = GeometryPayload(tracks, vias)
        over_sum, _ = self._compute_overuse()
        self._geometry_payload = GeometryPayload(tracks, vias) if over_sum == 0 else GeometryPayload([], [])
        return len(tracks), len(vias)

    def get_geometry_payload(self):
        """Clean geometry when there is some, else the provisional one (:11638-11650)."""
        if not self._geometry_payload.tracks and not self._geometry_payload.vias and \
                (self._provisional_geometry.tracks or self._provisional_geometry.vias):
            return self._provisional_geometry
        return self._geometry_payload

    def get_provisional_geometry(self):
        return self._provisional_geometry


class GeometryPayload:
    """Tracks and vias with attribute access (the reference's class of this name, :548)."""

    def __init__(self, tracks, vias):
        self.tracks = tracks
        self.vias = vias


# the reference exports the same class under this name (:11661)
UnifiedPathFinder = PathFinderRouter
