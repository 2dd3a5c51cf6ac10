"""Oracle A8–A9: path → arcs, node use / ownership, overuse and barrel tallies.

Reference: ``orthoroute/algorithms/manhattan/unified_pathfinder.py``

* ``_path_to_directed_edges`` / ``_path_to_edges`` (forward arcs then the
  arcs of the reversed path)                                 ``:9981-10046``
* ``_canonical_edge_resource_mask`` (one arc per segment,
  ``src < dst``)                                             ``:4919-4932``
* ``_unique_path_nodes`` / ``_rebuild_path_node_use`` / mark / clear
                                                             ``:4617-4659``
* via barrel ownership: ``_via_nodes_for_hop``,
  ``_mark_via_barrel_ownership_for_path``,
  ``_clear_via_barrel_ownership_for_path``,
  ``_rebuild_node_owner``                                    ``:4744-5034``,
                                                             ``:5222-5246``
* ``_compute_path_node_overuse``                             ``:10718-10726``
* ``_detect_path_node_conflicts``                            ``:10564-10606``
* ``_detect_barrel_conflicts`` (exact + shared path nodes;
  escape and portal-grid terms are empty without portals)    ``:10778-11111``
* ``_accumulate_node_conflict_history``                      ``:10048-10081``
"""
from __future__ import annotations

from collections import defaultdict
from itertools import combinations
from typing import Dict, List, Set

import numpy as np


def path_to_directed_edges(indptr, indices, path) -> List[int]:
    if len(path) < 2:
        return []
    out = []
    for u, v in zip(path, path[1:]):
        s, e = int(indptr[u]), int(indptr[u + 1])
        row = indices[s:e]
        hit = np.flatnonzero(row == v)
        if hit.size == 0:
            raise ValueError(f"Path hop is not a graph edge: {u}->{v}")
        out.append(s + int(hit[0]))
    return out


def path_to_edges(indptr, indices, path) -> List[int]:
    fwd = path_to_directed_edges(indptr, indices, path)
    rev = path_to_directed_edges(indptr, indices, list(reversed(path)))
    return fwd + rev


def canonical_mask(edge_src, indices) -> np.ndarray:
    return edge_src < indices


def unique_nodes(path) -> np.ndarray:
    if not path:
        return np.empty(0, dtype=np.int32)
    return np.unique(np.asarray(path, dtype=np.int32))


def via_nodes_for_path(path, nx, plane) -> List[int]:
    nodes = set()
    for u, v in zip(path, path[1:]):
        zu, ru = divmod(int(u), plane)
        zv, rv = divmod(int(v), plane)
        if ru != rv or zu == zv:
            continue
        for z in range(min(zu, zv), max(zu, zv) + 1):
            nodes.add(z * plane + ru)
    return sorted(nodes)


class NodeState:
    """node_owner / members, path_node_use, node_conflict_history."""

    def __init__(self, N, nx, plane):
        self.N, self.nx, self.plane = N, nx, plane
        self.owner = np.full(N, -1, dtype=np.int32)
        self.members: Dict[int, Set[int]] = {}
        self.path_node_use = np.zeros(N, dtype=np.int16)
        self.node_history = np.zeros(N, dtype=np.float32)
        self._hist_iter = None
        self._hist_nodes: Set[int] = set()

    # ownership ---------------------------------------------------------------
    def rebuild_owner(self, paths_by_id):
        self.owner.fill(-1)
        self.members = {}
        for nid, path in paths_by_id:
            if not path or len(path) < 2:
                continue
            for n in via_nodes_for_path(path, self.nx, self.plane):
                self.members.setdefault(n, set()).add(nid)
        for n, m in self.members.items():
            self.owner[n] = next(iter(m)) if len(m) == 1 else -2

    def mark_owner(self, nid, path):
        if not path or len(path) < 2:
            return
        for n in via_nodes_for_path(path, self.nx, self.plane):
            m = self.members.setdefault(n, set())
            m.add(nid)
            self.owner[n] = nid if len(m) == 1 else -2

    def clear_owner(self, nid, path):
        if not path or len(path) < 2:
            return
        for n in via_nodes_for_path(path, self.nx, self.plane):
            m = self.members.get(n)
            if not m:
                self.owner[n] = -1
                continue
            m.discard(nid)
            if not m:
                self.members.pop(n, None)
                self.owner[n] = -1
            elif len(m) == 1:
                self.owner[n] = next(iter(m))
            else:
                self.owner[n] = -2

    # path node use -------------------------------------------------------------
    def rebuild_use(self, paths):
        self.path_node_use.fill(0)
        for p in paths:
            nodes = unique_nodes(p)
            if nodes.size:
                self.path_node_use[nodes] += 1

    def mark_use(self, path):
        nodes = unique_nodes(path)
        if nodes.size:
            self.path_node_use[nodes] += 1

    def clear_use(self, path):
        nodes = unique_nodes(path)
        if nodes.size:
            self.path_node_use[nodes] = np.maximum(self.path_node_use[nodes] - 1, 0)

    def path_node_overuse(self):
        over = np.maximum(np.asarray(self.path_node_use, dtype=np.int64) - 1, 0)
        return int(over.sum()), int(np.count_nonzero(over))

    # node conflict history -----------------------------------------------------
    def accumulate_history(self, nodes, iteration, increment=1.0):
        nodes = np.unique(np.asarray(list(nodes), dtype=np.int64))
        if nodes.size == 0:
            return
        if self._hist_iter != iteration:
            self._hist_iter = iteration
            self._hist_nodes = set()
        nodes = np.asarray([n for n in nodes if int(n) not in self._hist_nodes], dtype=np.int64)
        if nodes.size == 0:
            return
        self.node_history[nodes] += np.float32(increment)
        self._hist_nodes.update(map(int, nodes))

    # owner penalty (A6 companion) ----------------------------------------------
    def owner_penalty(self, roi_nodes, current_id, pres_fac, owner_base=25.0,
                      path_base=25.0, hist_pen=5.0, freeze_weight=None):
        """``_build_owner_penalty`` (``unified_pathfinder.py:5308-5384``)."""
        owners = self.owner[roi_nodes]
        foreign = (owners != -1) & (owners != current_id)
        occupied = self.path_node_use[roi_nodes] > 0
        hist = self.node_history[roi_nodes]
        if not foreign.any() and not occupied.any() and not hist.any():
            return None
        weight = float(owner_base) * float(pres_fac)
        if freeze_weight is not None:
            weight = max(weight, float(freeze_weight))
        path_weight = float(path_base) * float(pres_fac)
        return (foreign.astype(np.float32) * weight
                + occupied.astype(np.float32) * path_weight
                + hist * float(hist_pen))


def detect_path_node_conflicts(node_state: NodeState, paths: Dict[str, List[int]]):
    shared_mask = node_state.path_node_use > 1
    if not shared_mask.any():
        return set(), set(), {}
    members = defaultdict(set)
    scores = defaultdict(int)
    for name, path in paths.items():
        if not path:
            continue
        nodes = unique_nodes(path)
        if not nodes.size:
            continue
        for n in nodes[shared_mask[nodes]]:
            members[int(n)].add(name)
            scores[name] += 1
    pairs = set()
    for m in members.values():
        pairs.update(combinations(sorted(m), 2))
    return pairs, set(members), dict(scores)


def detect_barrel_conflicts(edge_src, indices, node_state: NodeState, paths: Dict[str, List[int]],
                            net_to_edges: Dict[str, List[int]], net_id_map: Dict[str, int], iteration):
    """Exact barrel conflicts + shared path nodes.  Returns (count, info dict)."""
    info = dict(conflict_nets=set(), owner_nets=set(), victim_nets=set(), exact=0, path_node=0,
                exact_pairs=set(), path_node_pairs=set(), scores=defaultdict(int), path_node_scores={})
    chunks, ids = [], []
    for name, path in paths.items():
        if not path or len(path) < 2:
            continue
        nid = net_id_map[name]
        res = net_to_edges.get(name)
        if res is None:
            raise RuntimeError(f"edge tracking missing for committed net {name}")
        chunk = np.asarray(res, dtype=np.int32)[:len(res) // 2]
        if chunk.size == 0:
            continue
        chunks.append(chunk)
        ids.append(np.full(chunk.size, nid, dtype=np.int32))
    count_exact = 0
    if chunks:
        e = np.concatenate(chunks)
        en = np.concatenate(ids)
        s = edge_src[e]
        d = indices[e]
        so = node_state.owner[s]
        do = node_state.owner[d]
        sc = (so != -1) & (so != en)
        dc = (do != -1) & (do != en)
        cm = sc | dc
        count_exact = int(cm.sum())
        if count_exact:
            pos = np.flatnonzero(cm)
            victims = set(map(int, en[pos]))
            parts = []
            if sc.any():
                parts.append(s[np.flatnonzero(sc)])
            if dc.any():
                parts.append(d[np.flatnonzero(dc)])
            cnodes = np.unique(np.concatenate(parts))
            node_state.accumulate_history(cnodes, iteration)
            owners = set()
            for n in cnodes:
                owners.update(node_state.members.get(int(n), ()))
            id_to_name = {v: k for k, v in net_id_map.items()}
            for p in pos:
                vid = int(en[p])
                cn = []
                if sc[p]:
                    cn.append(int(s[p]))
                if dc[p]:
                    cn.append(int(d[p]))
                for n in cn:
                    for oid in node_state.members.get(n, ()):
                        if oid == vid:
                            continue
                        vn, on = id_to_name.get(vid), id_to_name.get(oid)
                        if vn is not None and on is not None:
                            info['scores'][vn] += 1
                            info['scores'][on] += 1
                            info['exact_pairs'].add(tuple(sorted((vn, on))))
            info['victim_nets'] = {id_to_name[i] for i in victims if i in id_to_name}
            info['owner_nets'] = {id_to_name[i] for i in owners if i in id_to_name}
            info['conflict_nets'] = {id_to_name[i] for i in (victims | owners) if i in id_to_name}
    info['exact'] = count_exact
    pairs, shared, pscores = detect_path_node_conflicts(node_state, paths)
    info['path_node_pairs'] = set(pairs)
    info['path_node_scores'] = dict(pscores)
    info['path_node'] = len(shared)
    if shared:
        for name, sc_ in pscores.items():
            info['scores'][name] += int(sc_)
        info['conflict_nets'].update({n for p in pairs for n in p})
        node_state.accumulate_history(shared, iteration)
    return count_exact + len(shared), info
