"""Oracle A10: the PathFinder negotiation loop (CPU restatement, tuple requests).

Restates ``PathFinderRouter._pathfinder_negotiation`` and the helpers it
drives for ``(name, src, dst)`` requests with portals disabled
(orthoroute/algorithms/manhattan/unified_pathfinder.py):

* parameter derivation          parameter_derivation.py:51-278,
                                board_analyzer.py:151-305
* iteration loop                :6163-7534
* ``_route_all``                :7903-8449 (ROI / full graph, owner
                                penalty, fallback ROI, commit / rip-up)
* ``_order_nets_by_difficulty`` :7840-7901
* ``_build_hotset`` + helpers   :8672-9391
* ``_find_via_pool_offenders``  :9393-9551
* ``_compute_layer_bias``       :8451-8534 ; layer EWMA / jam breaker
                                :7060-7129
* barrel / path-node audit      :10564-11111
* cleanup gating                :6596-6805, :10277-10360
* stagnation rip-up             :7276-7360, :9711-9810
* best-state capture / restore  :7790-7838 ; detail pass :7581-7788

Python ``random`` is used exactly where the reference uses it, so the seeded
streams coincide.  Every array operation keeps the reference's numpy dtypes.
"""
from __future__ import annotations

import heapq
import os
import random
from collections import defaultdict
from typing import Dict, List, Optional, Set, Tuple

import numpy as np

from . import accounting as acc
from .dijkstra import find_path_roi, find_path_roi_c
from .lattice import LatticeSpec, build_csr
from .roi import extract_roi_bfs, roi_radius
from .tallies import NodeState, detect_barrel_conflicts, detect_path_node_conflicts, path_to_edges


# ----------------------------------------------------------------------- config
class Config:
    """The ``PathFinderConfig`` fields the loop reads (``:570-782``)."""

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
        self.via_cost = 0.7
        self.via_pressure_threshold = 64
        self.via_pressure_multiplier = 1.5
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
        self.max_iterations_explicit = True
        for k, v in kw.items():
            setattr(self, k, v)


def derive_parameters(cfg: Config, lattice_bounds, pitch, nz, tasks, idx_to_coord):
    """``analyze_board_characteristics`` + ``derive/apply_derived_parameters``."""
    width = lattice_bounds[2] - lattice_bounds[0]
    height = lattice_bounds[3] - lattice_bounds[1]
    nsig = max(0, nz - 2)
    cx = int(width / pitch)
    cy = int(height / pitch)
    total_channels = nsig * cx * cy
    hpwl = 0.0
    for _, (s, d) in tasks.items():
        sx, sy, _ = idx_to_coord(s)
        dx, dy, _ = idx_to_coord(d)
        hpwl += abs(dx - sx) * pitch + abs(dy - sy) * pitch
    rho = (hpwl * 1.3) / max(1.0, total_channels * pitch * 0.75)
    L = nsig
    N = len(tasks)
    if rho < 0.6:
        mult, pmax = 1.15, 6.0
    elif rho < 0.9:
        mult, pmax = 1.12, 7.0
    elif rho < 1.2:
        mult, pmax = 1.10, 8.0
    else:
        mult, pmax = 1.08, 10.0
    if L <= 12:
        pmax *= 0.75
    elif L >= 25:
        pmax *= 1.25
    bonus = 6.0 if L <= 10 else 4.0 if L <= 15 else 2.0 if L <= 25 else 0.0
    hw = 8.0 + bonus + 6.0 * max(0.0, min(1.0, rho - 0.7))
    hg = 0.20 + 0.15 * max(0.0, min(1.0, rho - 0.8))
    pct = 0.25 if rho < 0.7 else 0.20 if rho < 1.0 else 0.15 if rho < 1.3 else 0.12
    hotset_cap = max(32, min(int(N * pct), int(N * 0.30)))
    if rho < 0.8:
        patience = 5
    elif rho < 1.1:
        patience = 6
    else:
        patience = 8
    if L <= 12:
        patience = max(patience, 7)
    cfg.pres_fac_init = 1.0
    cfg.pres_fac_mult = mult
    cfg.pres_fac_max = pmax
    cfg.hist_cost_weight = hw
    cfg.hist_gain = hg
    cfg.history_decay = 1.0
    cfg.hotset_cap = hotset_cap
    cfg.via_cost = 0.5
    cfg.stagnation_patience = patience
    if not cfg.max_iterations_explicit:
        cfg.max_iterations = max(cfg.max_iterations, 250)
    return rho


def resolve_pres_fac_max(cfg, nsig):
    floor = 32.0 if nsig <= 12 else 64.0 if nsig <= 20 else 128.0
    return max(float(cfg.pres_fac_max), floor)


# -------------------------------------------------------------------- helpers
def history_hotset_cap(t):
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


def exploration_fraction(t):
    if t > 16384:
        return 0.15
    if t > 2048:
        return 0.25
    return 0.40


def select_conflict_aware_hotset(ranked, conflict_pairs, cap, fraction, rng):
    """``_select_conflict_aware_hotset`` (``:8912-9037``)."""
    cap = max(0, int(cap))
    if cap == 0 or not ranked:
        return []
    cands = list(dict.fromkeys(ranked))
    cap = min(cap, len(cands))
    cset = set(cands)
    rank = {c: i for i, c in enumerate(cands)}
    adj = defaultdict(set)
    for a, b in conflict_pairs or ():
        if a == b or a not in cset or b not in cset:
            continue
        adj[a].add(b)
        adj[b].add(a)
    fraction = min(1.0, max(0.0, float(fraction)))
    primary = max(1, min(cap, int(round(cap * (1.0 - fraction)))))
    sel, sset = [], set()
    rem = {c: set(adj.get(c, ())) for c in cands}
    h = [(-len(rem[c]), rank[c], c) for c in cands if rem[c]]
    heapq.heapify(h)
    while len(sel) < primary and h:
        nd, _, c = heapq.heappop(h)
        if c in sset:
            continue
        live = len(rem[c])
        if -nd != live:
            heapq.heappush(h, (-live, rank[c], c))
            continue
        if live == 0:
            break
        sel.append(c)
        sset.add(c)
        for nb in tuple(rem[c]):
            rem[nb].discard(c)
            heapq.heappush(h, (-len(rem[nb]), rank[nb], nb))
        rem[c].clear()
    if len(sel) < primary:
        nonred = [c for c in cands if c not in sset and not (adj.get(c, set()) & sset)]
        nrs = set(nonred)
        red = [c for c in cands if c not in sset and c not in nrs]
        for c in nonred + red:
            sel.append(c)
            sset.add(c)
            if len(sel) >= primary:
                break
    if len(sel) < cap:
        expl = [c for c in cands if c not in sset]
        rng.shuffle(expl)
        sel.extend(expl[:cap - len(sel)])
    return sel


def rolling_progress_insufficient(values, window, min_fraction, min_overuse):
    window = max(1, int(window))
    if len(values) < window + 1:
        return False, None
    start = float(values[-window - 1])
    if start <= max(0, int(min_overuse)):
        return False, None
    best_later = min(map(float, values[-window:]))
    frac = max(0.0, (start - best_later) / max(1.0, start))
    return frac < max(0.0, float(min_fraction)), frac


def advance_pressure_trial(cur_ceiling, cur_frac, ref_ceiling, ref_frac, under, min_ratio=0.8, patience=2):
    ceiling = float(cur_ceiling)
    frac = max(0.0, float(cur_frac))
    if ref_ceiling is None or ref_frac is None:
        return ceiling, frac, 0, None
    pc = float(ref_ceiling)
    pf = max(0.0, float(ref_frac))
    if ceiling <= pc:
        return pc, pf, 0, None
    thr = max(0.0, float(min_ratio)) * pf
    if (pf <= 0.0 and frac > 0.0) or (pf > 0.0 and frac >= thr):
        return ceiling, frac, 0, None
    fails = int(under) + 1
    if fails >= max(1, int(patience)):
        return pc, pf, 0, ceiling
    return pc, pf, fails, None


def next_pressure_ceiling(cur, events, pressure_after=2, maximum=1024.0):
    cur = float(cur)
    if int(events) < max(1, int(pressure_after)):
        return cur
    return min(max(cur, float(maximum)), max(128.0, cur * 2.0))


# ------------------------------------------------------------------- router
class OracleRouter:
    """CPU restatement of the reference loop for (name, src, dst) tasks."""

    def __init__(self, spec: LatticeSpec, bounds, cfg: Optional[Config] = None, fast: bool = False):
        self.spec = spec
        self._find = find_path_roi_c if fast else find_path_roi
        self.cfg = cfg or Config()
        self.csr = build_csr(spec)
        c = self.csr
        self.nx, self.ny, self.nz = c.nx, c.ny, c.nz
        self.plane = c.plane
        self.N = c.num_nodes
        self.E = len(c.indices)
        self.bounds = bounds
        self.edge_src = c.edge_src()
        self.canon_mask = self.edge_src < c.indices
        self.acc = acc.Accountant(self.E)
        self.pools = acc.ViaPools(self.nx, self.ny, self.nz)
        self.via_meta = acc.via_edge_metadata(c)
        self.via_edges = c.edge_kind.astype(bool)
        self.nodes = NodeState(self.N, self.nx, self.plane)
        self.layer_bias = np.ones(self.nz, dtype=np.float32)      # router EWMA bias
        self.lb_state = acc.LayerBiasState()
        self.net_paths: Dict[str, List[int]] = {}
        self.net_to_edges: Dict[str, List[int]] = {}
        self.edge_to_nets = defaultdict(set)
        self.net_id_map: Dict[str, int] = {}
        self.iteration = 0
        self.stagnation_counter = 0
        self.full_graph_fallback_count = 0
        self._last_ripped: Set[str] = set()
        self._freeze_pres_fac_until = 0
        self._stagnation_victim_history: Set[str] = set()
        self._stagnation_victim_cursor = 0
        self._cleanup_move_counts = defaultdict(int)
        self.freeze = False
        self.physical_cleanup_started = False
        self.barrel_info = None
        self.barrel_count = 0
        self.path_node_scores: Dict[str, int] = {}
        self.path_node_pairs = set()
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
        self.stats = {"scanned": 0, "settled": 0, "searches": 0}
        self.trace = None            # optional list of per-iteration paths
        self.search_log = None       # optional list of per-search records

    # -- ids / coords -----------------------------------------------------------
    def _net_id(self, name):
        if name not in self.net_id_map:
            self.net_id_map[name] = len(self.net_id_map)
        return self.net_id_map[name]

    def idx_to_coord(self, n):
        z, r = divmod(int(n), self.plane)
        y, x = divmod(r, self.nx)
        return x, y, z

    # -- state maintenance ------------------------------------------------------
    def _path_edges(self, path):
        return path_to_edges(self.csr.indptr, self.csr.indices, path)

    def _update_tracking(self, name, edges):
        self._clear_tracking(name)
        self.net_to_edges[name] = edges
        for e in edges:
            self.edge_to_nets[e].add(name)

    def _clear_tracking(self, name):
        if name in self.net_to_edges:
            for e in self.net_to_edges[name]:
                self.edge_to_nets[e].discard(name)
            del self.net_to_edges[name]

    def _rebuild_node_owner(self):
        pairs = [(self._net_id(n), p) for n, p in self.net_paths.items() if p and len(p) >= 2]
        self.nodes.rebuild_owner(pairs)

    def _rebuild_via_usage(self):
        self.pools.rebuild(list(self.net_paths.values()))
        self._rebuild_node_owner()
        self.nodes.rebuild_use(list(self.net_paths.values()))

    def _spatial_via_overuse(self):
        return self.pools.spatial_overuse_total()

    def _compute_overuse(self):
        s, c = self.acc.compute_edge_overuse(self.canon_mask)
        return s + self._spatial_via_overuse(), c

    def _detect_barrels(self):
        count, info = detect_barrel_conflicts(self.edge_src, self.csr.indices, self.nodes, self.net_paths,
                                              self.net_to_edges, self.net_id_map, self.iteration)
        self.barrel_info = info
        self.barrel_conflict_nets = set(info['conflict_nets'])
        self.barrel_owner_nets = set(info['owner_nets'])
        self.barrel_victim_nets = set(info['victim_nets'])
        self.physical_scores = info['scores']
        self.path_node_scores = dict(info['path_node_scores'])
        self.path_node_pairs = set(info['path_node_pairs'])
        self.exact_pairs = set(info['exact_pairs'])
        return count

    def _capture(self):
        return {n: list(p) for n, p in self.net_paths.items()}

    def _restore(self, state):
        self.net_paths.clear()
        self.net_paths.update({n: list(p) for n, p in state.items()})
        self.acc.canonical.clear()
        self.acc.present.fill(0)
        self.net_to_edges.clear()
        self.edge_to_nets.clear()
        for n, p in self.net_paths.items():
            if not p or len(p) < 2:
                continue
            edges = self._path_edges(p)
            for e in edges:
                self.acc.canonical[e] = self.acc.canonical.get(e, 0) + 1
            self._update_tracking(n, edges)
        self.acc.refresh_from_canonical()
        self._rebuild_via_usage()
        self._rebuild_node_owner()
        self.nodes.rebuild_use(list(self.net_paths.values()))

    # -- hotset -----------------------------------------------------------------
    def _find_via_pool_offenders(self):
        P = self.pools
        col_over = P.col_use > P.col_cap
        col_over = col_over if np.any(col_over) else None
        seg_over = None
        if P.has_seg:
            m = P.seg_use > P.seg_cap
            seg_over = m if np.any(m) else None
        if col_over is None and seg_over is None:
            self._via_pool_keepers = {}
            self._via_pool_member_state = {}
            self._via_pool_keeper_stagnation = {}
            return set()
        members = defaultdict(set)
        for name, path in self.net_paths.items():
            if not path or len(path) < 2:
                continue
            res = set()
            for u, v in zip(path, path[1:]):
                xu, yu, zu = self.idx_to_coord(u)
                xv, yv, zv = self.idx_to_coord(v)
                if xu != xv or yu != yv or zu == zv:
                    continue
                if col_over is not None and col_over[xu, yu]:
                    res.add(("col", xu, yu))
                if seg_over is not None:
                    zl = max(1, min(min(zu, zv), self.nz - 2))
                    zh = max(1, min(max(zu, zv), self.nz - 2))
                    for z in range(zl, zh):
                        s = z - 1
                        if 0 <= s < P.segZ and seg_over[xu, yu, s]:
                            res.add(("seg", xu, yu, s))
            for r in res:
                members[r].add(name)
        rotation_allowed = self._spatial_via_overuse() <= self._via_keeper_threshold()
        nk, nm, ns = {}, {}, {}
        off = set()
        for r, mem in sorted(members.items()):
            kind, x, y, *tail = r
            if kind == "col":
                capv, obs = int(P.col_cap[x, y]), int(P.col_use[x, y])
            else:
                capv, obs = int(P.seg_cap[x, y, tail[0]]), int(P.seg_use[x, y, tail[0]])
            capv = max(0, capv)
            state = frozenset(mem)
            nm[r] = state
            unchanged = self._via_pool_member_state.get(r) == state
            stagn = int(self._via_pool_keeper_stagnation.get(r, 0)) + 1 if unchanged else 0
            prev = [n for n in self._via_pool_keepers.get(r, ()) if n in mem][:capv]
            remaining = sorted(mem - set(prev))
            keepers = tuple(prev + remaining[:max(0, capv - len(prev))])
            if rotation_allowed and stagn >= 2 and 0 < capv < len(mem) and prev:
                ordered = sorted(mem)
                start = (ordered.index(prev[0]) + 1) % len(ordered)
                keepers = tuple(ordered[(start + o) % len(ordered)] for o in range(capv))
                stagn = 0
            ns[r] = stagn
            nk[r] = keepers
            off.update(mem - set(keepers))
            if obs > len(mem):
                off.update(mem)
        self._via_pool_keepers, self._via_pool_member_state, self._via_pool_keeper_stagnation = nk, nm, ns
        return off

    def _via_keeper_threshold(self):
        routed = sum(bool(p) for p in self.net_paths.values())
        groups = max(1, int(np.ceil(max(0, routed) / max(1, self.cfg.via_keeper_rotation_nets_per_step))))
        return max(0, int(self.cfg.via_keeper_rotation_overuse_threshold)) * groups

    def _effective_cap(self, t):
        base = history_hotset_cap(t)
        cfg = self.cfg
        if t > int(cfg.slow_progress_min_overuse) and self.iteration <= int(getattr(self, "_hotset_rate_boost_until", 0)):
            init = max(1, int(cfg.slow_progress_hotset_cap))
            mx = max(init, int(cfg.slow_progress_hotset_cap_max))
            ga = max(1, int(cfg.slow_progress_hotset_growth_after))
            ev = max(1, int(getattr(self, "_slow_progress_event_count", 1)))
            steps = max(0, ev - ga + 1)
            return max(base, min(mx, init * (2 ** steps)))
        return base

    def _bounded_cap(self, t):
        base = history_hotset_cap(t)
        eff = self._effective_cap(t)
        conf = max(1, int(self.cfg.hotset_cap))
        if eff > base:
            conf = max(conf, eff)
        cap = min(conf, eff)
        floor = int(self.cfg.hotset_cap_floor)
        if floor > 0 and t > 2048:
            cap = max(cap, floor)
        return cap

    def _physical_hotset(self):
        off = set(self.barrel_conflict_nets)
        cfg = self.cfg
        mx = max(1, int(cfg.physical_hotset_cap))
        mn = min(mx, max(1, int(cfg.physical_hotset_min)))
        scale = max(1.0, float(cfg.physical_conflicts_per_hotset_net))
        cap = min(mx, max(mn, int(np.ceil(max(0, self.barrel_count) / scale))))
        if len(off) <= cap:
            return off
        ranked = sorted(off, key=lambda n: (-int(self.physical_scores.get(n, 0)), str(n)))
        return set(ranked[:cap])

    def _build_hotset(self, tasks, ripped):
        over = np.maximum(0, self.acc.present - self.acc.capacity)
        over_idx = set(map(int, np.flatnonzero(over > 0)))
        via_off = self._find_via_pool_offenders()
        pscores = {n: int(s) for n, s in self.path_node_scores.items() if n in tasks and int(s) > 0}
        poff = set(pscores)
        pno = int(np.maximum(0, np.asarray(self.nodes.path_node_use) - 1).sum())
        total_neg = self._compute_overuse()[0] + pno
        thr = int(self.cfg.portal_cleanup_edge_threshold)
        if self.cfg.physical_cleanup_overuse_threshold is not None:
            thr = max(thr, int(self.cfg.physical_cleanup_overuse_threshold))
        if len(over_idx) == 0:
            unrouted = {n for n in tasks if not self.net_paths.get(n)}
            phys = self._physical_hotset() if total_neg <= thr else set()
            hot = unrouted | ripped | via_off | phys
            cap = self._bounded_cap(total_neg)
            frac = exploration_fraction(total_neg)
            hot.update(select_conflict_aware_hotset(
                sorted(poff, key=lambda n: (-pscores[n], str(n))), self.path_node_pairs, cap, frac,
                random.Random(42 + self.iteration)))
            self._last_hotset_size = len(hot)
            return hot
        offenders = set()
        for e in over_idx:
            offenders.update(self.edge_to_nets.get(e, set()))
        offenders.update(poff)
        for n in tasks:
            if n in offenders:
                self._net_clean_iters[n] = 0
            else:
                self._net_clean_iters[n] = self._net_clean_iters.get(n, 0) + 1
        frozen = {n for n in offenders if self._net_clean_iters.get(n, 0) >= 3}
        offenders -= frozen
        offenders |= ripped
        offenders |= via_off
        unrouted = {n for n in tasks if not self.net_paths.get(n)}
        scores = []
        for n in offenders:
            imp = float(pscores.get(n, 0))
            if n in self.net_to_edges:
                imp += sum(float(over[e]) for e in self.net_to_edges[n] if e in over_idx)
            scores.append((imp, n))
        for n in unrouted:
            if n not in offenders:
                scores.append((0.0, n))
        scores.sort(reverse=True)
        cap = self._bounded_cap(total_neg)
        rng = random.Random(42 + self.iteration)
        ranked = [n for _, n in scores if self.iteration - self._last_reroute_iter.get(n, -999) > 1]
        frac = exploration_fraction(total_neg)
        sel = select_conflict_aware_hotset(ranked, self.path_node_pairs, cap, frac, rng)
        for n in sel:
            self._last_reroute_iter[n] = self.iteration
        hot = set(sel)
        raw_edges = int(np.count_nonzero(over > 0))
        if raw_edges <= thr and total_neg <= thr:
            hot.update(self._physical_hotset())
        hot.update(unrouted)
        self._last_hotset_size = len(hot)
        return hot

    # -- ordering ---------------------------------------------------------------
    def _order_nets(self, tasks):
        over = np.maximum(0, self.acc.present - self.acc.capacity)
        scores = []
        for name, (s, d) in tasks.items():
            sx, sy, sz = self.idx_to_coord(s)
            dx, dy, dz = self.idx_to_coord(d)
            dist = abs(dx - sx) + abs(dy - sy) + abs(dz - sz)
            cong = 0.0
            if name in self.net_to_edges:
                edges = self.net_to_edges[name]
                cong = sum(float(over[e]) for e in edges) / max(1, len(edges))
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

    # -- routing ----------------------------------------------------------------
    def _owner_penalty(self, roi, name):
        freeze = self.cfg.portal_cleanup_node_penalty if self.freeze else None
        return self.nodes.owner_penalty(roi, self._net_id(name), self._pres_fac_now,
                                        self.cfg.owner_penalty_base, self.cfg.path_node_penalty_base,
                                        self.cfg.node_history_penalty, freeze_weight=freeze)

    def _search(self, src, dst, roi, g2r, pen, name, kind):
        path = self._find(self.csr.indptr, self.csr.indices, src, dst, self.acc.total_cost, roi, g2r,
                          node_penalty=pen, stats=self.stats)
        self.stats["searches"] += 1
        if self.search_log is not None:
            self.search_log.append((self.iteration, name, kind, list(path) if path else None))
        return path

    def _route_all(self, tasks, all_tasks):
        cfg = self.cfg
        self.full_graph_fallback_count = 0
        bonus = self.stagnation_counter * 0.6
        ordered = self._order_nets(tasks)
        live = bool(cfg.live_present_costs)
        if live:
            self.acc.begin_live_present_costs()
        ip, ix = self.csr.indptr, self.csr.indices
        for name in ordered:
            src, dst = tasks[name]
            if name in self.net_paths and self.net_paths[name]:
                old_edges = self.net_to_edges.get(name) or self._path_edges(self.net_paths[name])
                self.nodes.clear_owner(self._net_id(name), self.net_paths[name])
                self.nodes.clear_use(self.net_paths[name])
                self.acc.clear_path(old_edges)
                if live:
                    self.acc.refresh_live_present_costs(old_edges)
                self._clear_tracking(name)
            sx, sy, _ = self.idx_to_coord(src)
            dx, dy, _ = self.idx_to_coord(dst)
            dist = abs(dx - sx) + abs(dy - sy)
            if dist < 125:
                r = roi_radius(src, dst, self.nx, self.plane, bonus)
                roi, g2r = extract_roi_bfs(ip, ix, self.N, src, dst, initial_radius=r, stagnation_bonus=bonus)
                kind = "roi"
            else:
                roi = np.arange(self.N, dtype=np.int32)
                g2r = roi
                kind = "full"
            self._net_id(name)
            pen = self._owner_penalty(roi, name)
            path = self._search(src, dst, roi, g2r, pen, name, kind)
            if (not path or len(path) <= 1) and self.full_graph_fallback_count < 5:
                r = roi_radius(src, dst, self.nx, self.plane, bonus * 2)
                roi, g2r = extract_roi_bfs(ip, ix, self.N, src, dst, initial_radius=r, stagnation_bonus=bonus * 2)
                pen = self._owner_penalty(roi, name)
                path = self._search(src, dst, roi, g2r, pen, name, "fallback")
                self.full_graph_fallback_count += 1
            if path and len(path) > 1:
                edges = self._path_edges(path)
                self.acc.commit_path(edges)
                if live:
                    self.acc.refresh_live_present_costs(edges)
                self.net_paths[name] = path
                self.nodes.mark_owner(self._net_id(name), path)
                self.nodes.mark_use(path)
                self._update_tracking(name, edges)
            else:
                self.net_paths[name] = []
                self._clear_tracking(name)
        routed = sum(1 for p in self.net_paths.values() if p)
        return routed, len(all_tasks) - routed

    def _rip_top_k(self, k=20):
        over = np.maximum(0, self.acc.present - self.acc.capacity)
        over_idx = set(map(int, np.flatnonzero((over > 0) & self.canon_mask)))
        _, _, mscores = detect_path_node_conflicts(self.nodes, self.net_paths)
        self.path_node_scores = dict(mscores)
        cands = set(mscores)
        for e in over_idx:
            cands.update(self.edge_to_nets.get(e, ()))
        scores = []
        for n in cands:
            if not self.net_paths.get(n):
                continue
            imp = float(mscores.get(n, 0))
            if n in self.net_to_edges:
                imp += sum(float(over[e]) for e in self.net_to_edges[n] if e in over_idx)
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
            sel = [ranked[(start + o) % len(ranked)] for o in range(cnt)]
            self._stagnation_victim_cursor = (start + cnt) % len(ranked)
            victims = set(sel)
            self._stagnation_victim_history = victims
        for n in victims:
            if self.net_paths.get(n) and n in self.net_to_edges:
                old = self.net_paths[n]
                self.acc.clear_path(self.net_to_edges[n])
                self.nodes.clear_owner(self._net_id(n), old)
                self.nodes.clear_use(old)
                self.net_paths[n] = []
                self._clear_tracking(n)
        return victims

    def _movable_components(self, exact_pairs):
        adj = defaultdict(set)
        for a, b in exact_pairs:
            if a == b:
                continue
            adj[a].add(b)
            adj[b].add(a)
        movable = set()
        eligible = set(adj)
        while eligible:
            n = min(eligible, key=lambda c: (self._cleanup_move_counts[c], -len(adj[c]), c))
            movable.add(n)
            eligible.discard(n)
            eligible.difference_update(adj[n])
        for n in movable:
            self._cleanup_move_counts[n] += 1
        return movable

    def _layer_congestion(self, over):
        mask = over > 0
        if not np.any(mask):
            return {}
        vals = over[mask]
        lays = self.csr.edge_layer[mask]
        out = {}
        for z in range(1, self.nz + 1):
            m = lays == z
            if np.any(m):
                out[z] = float(np.sum(vals[m]))
        return out

    # -- the loop -----------------------------------------------------------------
    def route(self, tasks: Dict[str, Tuple[int, int]]):
        cfg = self.cfg
        derive_parameters(cfg, self.bounds, self.spec.pitch, self.nz, tasks, self.idx_to_coord)
        nsig = self.nz - 2
        pres_fac = float(cfg.pres_fac_init)
        pres_mult = float(cfg.pres_fac_mult)
        hist_gain = float(cfg.hist_gain)
        hw_mult = 1.2 if nsig <= 12 else 1.0 if nsig <= 20 else 0.8
        pres_max = resolve_pres_fac_max(cfg, nsig)
        pres_mult = float(os.getenv('ORTHO_PRES_FAC_MULT', pres_mult))
        pres_max = float(os.getenv('ORTHO_PRES_FAC_MAX', pres_max))
        hist_gain = float(os.getenv('ORTHO_HIST_GAIN', hist_gain))
        hist_decay = float(os.getenv("ORTHO_HISTORY_DECAY", cfg.history_decay if cfg.history_decay is not None else 1.0))
        best_overuse = float('inf')
        best_score = None
        best_state = None
        best_iter = 0
        stagnant = 0
        neg_hist = []
        self._slow_progress_event_count = 0
        self._hotset_rate_boost_until = 0
        last_slow_trigger = -1_000_000
        trial_ref_ceiling = trial_ref_frac = None
        trial_under = 0
        adaptive_limit = float(cfg.slow_progress_pres_fac_max)
        metrics = []
        jam = None
        failed = 0
        over_sum = over_cnt = 0
        negotiated = 0
        for it in range(1, cfg.max_iterations + 1):
            self.iteration = it
            self._pres_fac_now = pres_fac
            self.acc.refresh_from_canonical()
            self._rebuild_via_usage()
            self.pools.update_presence()
            if it == 1:
                self.acc.present_ema = self.acc.present.copy()
            self.acc.update_present_ema(0.40)
            lb = self.lb_state.compute(self.acc.present_ema, self.acc.capacity, self.csr.edge_layer, self.nz,
                                       self.nodes.path_node_use)
            vmult = 1.0
            if it >= 3 and self._spatial_via_overuse() >= int(cfg.via_pressure_threshold):
                vmult = float(cfg.via_pressure_multiplier)
            elif pres_fac >= 64:
                over = np.maximum(0, self.acc.present - self.acc.capacity)
                vo = float(over[self.via_edges].sum())
                to = float(over.sum())
                if to > 0:
                    vmult = 1.5 if vo / to > 0.7 else 0.5
            self.acc.update_costs(self.csr.base_costs, pres_fac, cfg.hist_cost_weight * hw_mult,
                                  via_cost_multiplier=vmult, base_cost_weight=cfg.base_cost_weight,
                                  edge_layer=self.csr.edge_layer, layer_bias_per_layer=lb,
                                  edge_kind=self.csr.edge_kind)
            acc.apply_via_pooling_penalties(self.acc.total_cost, self.via_meta, self.pools, self.layer_bias, pres_fac)
            if it > 1:
                acc.block_via_edges(self.acc.total_cost, self.via_meta, self.pools)
            if cfg.reroute_only_offenders and it > 1:
                hot = self._build_hotset(tasks, self._last_ripped)
                sub = {k: v for k, v in tasks.items() if k in hot}
                self._last_ripped = set()
            else:
                sub = dict(tasks)
            work_scale = min(max(1.0, float(cfg.pressure_work_scale_max)),
                             max(1.0, max(0, len(sub)) / max(1, int(cfg.pressure_reference_hotset)))) \
                if it > 1 else 1.0
            routed, failed = self._route_all(sub, tasks)
            self.acc.refresh_from_canonical()
            conflicts = self._detect_barrels()
            self.barrel_count = conflicts
            over_sum, over_cnt = self._compute_overuse()
            pno, _ = self.nodes.path_node_overuse()
            negotiated = over_sum + pno
            clean = over_sum == 0 and pno == 0
            thr = int(cfg.portal_cleanup_edge_threshold)
            ready = over_cnt <= thr and negotiated <= thr
            if conflicts > 0 and ready:
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
            metrics.append({'iter': it, 'nets_routed': routed, 'overuse_sum': over_sum, 'overuse_edges': over_cnt})
            if self.trace is not None:
                self.trace.append({n: list(p) for n, p in self.net_paths.items()})
            score = (int(failed), int(over_sum) + int(pno), int(conflicts))
            if best_score is None or score < best_score:
                best_score, best_state, best_iter = score, self._capture(), it
                self._stagnation_victim_history = set()
                self._stagnation_victim_cursor = 0
            neg_hist.append(negotiated)
            window = max(1, int(cfg.slow_progress_window))
            slow, frac = rolling_progress_insufficient(neg_hist, window, cfg.slow_progress_min_fraction,
                                                       cfg.slow_progress_min_overuse)
            if slow and it - last_slow_trigger >= window:
                last_slow_trigger = it
                self._slow_progress_event_count += 1
                self._hotset_rate_boost_until = it + window
                after = max(1, int(cfg.slow_progress_pressure_after))
                old_ceiling = pres_max
                rejected = None
                if (self._slow_progress_event_count >= 4 and self._last_hotset_size >= int(cfg.slow_progress_hotset_cap_max)
                        and frac is not None):
                    trial_ref_ceiling, trial_ref_frac, trial_under, rejected = advance_pressure_trial(
                        old_ceiling, frac, trial_ref_ceiling, trial_ref_frac, trial_under,
                        cfg.slow_progress_pressure_trial_min_ratio, cfg.slow_progress_pressure_trial_patience)
                    if rejected is not None:
                        adaptive_limit = min(adaptive_limit, float(trial_ref_ceiling))
                        pres_max = min(pres_max, adaptive_limit)
                        pres_fac = min(pres_fac, pres_max)
                if self._slow_progress_event_count >= after and rejected is None:
                    pres_max = next_pressure_ceiling(old_ceiling, self._slow_progress_event_count, after,
                                                     min(float(cfg.slow_progress_pres_fac_max), adaptive_limit))
                    pres_fac = min(pres_fac * 1.5, pres_max)
            over = np.maximum(0, self.acc.present - self.acc.capacity)
            by_layer = self._layer_congestion(over) if over_sum > 0 else None
            if by_layer is None and over_sum > 0:
                by_layer = self._layer_congestion(over)
            if by_layer and sum(by_layer.values()) > 0:
                lo = np.array([by_layer.get(z, 0.0) for z in range(self.nz)])
                mean = np.mean(lo[lo > 0]) + 1e-9
                pressure = lo / mean
                if nsig <= 12:
                    alpha, bmin, bmax = 0.20, 0.60, 1.80
                elif nsig <= 20:
                    alpha, bmin, bmax = 0.12, 0.75, 1.50
                else:
                    alpha, bmin, bmax = 0.08, 0.85, 1.20
                target = 1.0 + alpha * (pressure - 1.0)
                self.layer_bias = 0.85 * self.layer_bias + 0.15 * target
                self.layer_bias = np.clip(self.layer_bias, bmin, bmax)
                tot = sum(by_layer.values())
                if tot > 0:
                    mz, mo = max(by_layer.items(), key=lambda x: x[1])
                    pct = (mo / tot) * 100
                    if jam is None:
                        jam = {'layer': None, 'count': 0, 'boost_until': 0}
                    if pct >= 60.0:
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
            cap_env = os.getenv('ORTHO_NO_HISTORY_CAP', '0') == '0'
            self.acc.update_history(hg, base_costs=self.csr.base_costs if cap_env else None,
                                    history_cap_multiplier=15.0 if cap_env else 1.0, decay_factor=hist_decay,
                                    use_raw_present=True)
            if failed == 0 and clean:
                self._rebuild_node_owner()
                bc = self._detect_barrels()
                self.barrel_count = bc
                if bc == 0:
                    return {'success': True, 'converged': True, 'paths': self.net_paths, 'iterations': it,
                            'iteration_metrics': metrics}
            if negotiated < best_overuse:
                best_overuse = negotiated
                stagnant = 0
            else:
                stagnant += 1
            if stagnant == 2:
                pres_fac = min(pres_fac * 1.5, pres_max)
            if stagnant >= cfg.stagnation_patience and it < cfg.max_iterations:
                if not ((not self.physical_cleanup_started) and self._spatial_via_overuse() <= max(0, self._via_keeper_threshold())):
                    stagnant = 0
                else:
                    cur = (int(failed), int(over_sum) + int(pno), int(conflicts))
                    if best_state is not None and best_score is not None and best_score < cur:
                        self._restore(best_state)
                    self.stagnation_counter += 1
                    victims = self._rip_top_k(20)
                    self._last_ripped = victims
                    self._freeze_pres_fac_until = it + 2
                    stagnant = 0
                    continue
            if it > self._freeze_pres_fac_until:
                pres_fac = min(pres_fac * (pres_mult ** work_scale), pres_max)
        cur = (int(failed), int(over_sum) + int(self.nodes.path_node_overuse()[0]), int(self.barrel_count))
        restored = best_state is not None and best_score is not None and best_score < cur
        if restored:
            self._restore(best_state)
            failed = sum(1 for n in tasks if not self.net_paths.get(n))
            over_sum, over_cnt = self._compute_overuse()
            self.barrel_count = self._detect_barrels()
            pno, _ = self.nodes.path_node_overuse()
            negotiated = over_sum + pno
        if 0 < negotiated <= 100:
            det = self._detail_pass(tasks, negotiated, pres_max)
            if det.get('success'):
                det['iteration_metrics'] = metrics
                return det
        self._rebuild_node_owner()
        final_barrels = self._detect_barrels()
        success = failed == 0 and over_sum == 0 and final_barrels == 0
        return {'success': success, 'converged': success, 'barrel_conflicts': final_barrels,
                'overuse_sum': over_sum, 'overuse_edges': over_cnt, 'failed_nets': failed,
                'path_node_overuse_sum': self.nodes.path_node_overuse()[0],
                'iterations': len(metrics), 'best_iteration': best_iter, 'iteration_metrics': metrics,
                'paths': self.net_paths}

    def _detail_conflict_nets(self, edge_nets):
        return set(edge_nets) | set(self.path_node_scores) | set(self._find_via_pool_offenders()) | \
            set(self.barrel_conflict_nets)

    def _detail_pass(self, tasks, initial_overuse, pres_max_now):
        cfg = self.cfg
        original = self._capture()
        best_state = original
        unrouted0 = sum(1 for n in tasks if not self.net_paths.get(n))
        best = (unrouted0, int(initial_overuse), 0, int(self.barrel_count))
        best = (best[0], best[1] + best[2], best[3])
        over = np.maximum(0, self.acc.present - self.acc.capacity)
        conflict_edges = set(int(e) for e in np.flatnonzero(over > 0))
        cn = set()
        for n, p in self.net_paths.items():
            if p and any(e in conflict_edges for e in self._path_edges(p)):
                cn.add(n)
        cn = self._detail_conflict_nets(cn)
        if not cn:
            return {'success': False}
        ctasks = {n: tasks[n] for n in cn if n in tasks}
        dmax = max(float(cfg.pres_fac_max), float(pres_max_now))
        pres_fac = dmax * 0.5
        for _ in range(1, 11):
            self.acc.refresh_from_canonical()
            self.acc.update_costs(self.csr.base_costs, pres_fac, cfg.hist_cost_weight * 1.5,
                                  via_cost_multiplier=0.3, base_cost_weight=cfg.base_cost_weight)
            hot = self._build_hotset(ctasks, set())
            # unified_pathfinder.py:7672 keeps the first 60 nets of the set: the
            # choice follows Python's string hashing (fix PYTHONHASHSEED to reproduce)
            hot = set(list(hot)[:60])
            if not hot:
                hot = cn
            sub = {k: v for k, v in ctasks.items() if k in hot}
            old = self.stagnation_counter
            self.stagnation_counter += 3
            self._pres_fac_now_detail = pres_fac
            self._route_all(sub, tasks)
            self.stagnation_counter = old
            self.acc.refresh_from_canonical()
            over_sum, over_cnt = self._compute_overuse()
            self._rebuild_node_owner()
            bc = self._detect_barrels()
            self.barrel_count = bc
            pno, _ = self.nodes.path_node_overuse()
            neg = over_sum + pno
            unrouted = {n for n in tasks if not self.net_paths.get(n)}
            sc = (len(unrouted), int(over_sum) + int(pno), int(bc))
            if sc < best:
                best = sc
                best_state = self._capture()
            cn = self._detail_conflict_nets(cn)
            ctasks.update({n: tasks[n] for n in cn if n in tasks})
            if neg == 0:
                if unrouted:
                    cn = unrouted
                    ctasks.update({n: tasks[n] for n in unrouted})
                    continue
                if bc:
                    continue
                return {'success': True, 'paths': self.net_paths}
            if self.trace is not None:
                self.trace.append({n: list(p) for n, p in self.net_paths.items()})
            self.acc.update_history(cfg.hist_gain * 2.0, base_costs=self.csr.base_costs,
                                    history_cap_multiplier=15.0, decay_factor=0.98)
            pres_fac = min(pres_fac * 1.5, dmax)
        self._restore(best_state)
        return {'success': False, 'overuse_sum': best[1]}
