"""Oracle A7–A8: ROI heap Dijkstra and backtrace (CPU restatement).

Reference: ``SimpleDijkstra.find_path_roi``
(``orthoroute/algorithms/manhattan/unified_pathfinder.py:2451-2548``).

Semantics kept exactly:

* heap entries are ``(python float label, roi index)``; ties pop the lower
  ROI index first;
* ``dist`` is a float32 array: a relaxation ``alt = (du + float(cost)) +
  float(pen[v])`` (FP64) is accepted iff ``alt < float(dist[v])``, then
  ``dist[v] = float32(alt)``, ``parent[v] = u`` and ``alt`` is pushed;
* each node is settled once; the search stops when dst is popped;
* backtrace walks ``parent`` from dst and reverses; a single-node path is
  ``None``.

``find_path_multisource`` restates the multi-source multi-sink twin
(``:2550-2659``) the same way.
"""
from __future__ import annotations

import heapq
from typing import List, Optional

import numpy as np


def find_path_roi(indptr, indices, src, dst, costs, roi_nodes, global_to_roi,
                  node_penalty=None, stats=None) -> Optional[List[int]]:
    roi_src = int(global_to_roi[src])
    roi_dst = int(global_to_roi[dst])
    if roi_src < 0 or roi_dst < 0:
        return None
    R = len(roi_nodes)
    dist = np.full(R, np.inf, dtype=np.float32)
    parent = np.full(R, -1, dtype=np.int32)
    visited = np.zeros(R, dtype=bool)
    dist[roi_src] = 0.0
    heap = [(0.0, roi_src)]
    # Python-level views for speed (same values as the numpy arrays).
    ip = indptr.tolist() if hasattr(indptr, "tolist") else indptr
    ix = indices
    cst = costs
    pen = node_penalty
    scanned = 0
    settled = 0
    while heap:
        du, u = heapq.heappop(heap)
        if visited[u]:
            continue
        visited[u] = True
        settled += 1
        if u == roi_dst:
            break
        ug = int(roi_nodes[u])
        s, e = ip[ug], ip[ug + 1]
        for ei in range(s, e):
            scanned += 1
            vg = int(ix[ei])
            v = int(global_to_roi[vg])
            if v < 0 or visited[v]:
                continue
            alt = du + float(cst[ei])
            if pen is not None:
                alt += float(pen[v])
            if alt < dist[v]:
                dist[v] = alt
                parent[v] = u
                heapq.heappush(heap, (alt, v))
    if stats is not None:
        stats["scanned"] = stats.get("scanned", 0) + scanned
        stats["settled"] = stats.get("settled", 0) + settled
    if not np.isfinite(dist[roi_dst]):
        return None
    path, cur = [], roi_dst
    while cur != -1:
        path.append(int(roi_nodes[cur]))
        cur = int(parent[cur])
    path.reverse()
    return path if len(path) > 1 else None


def find_path_multisource(indptr, indices, src_seeds, dst_targets, costs, roi_nodes, global_to_roi,
                          node_penalty=None, plane=None, stats=None):
    """``SimpleDijkstra.find_path_multisource_multisink``
    (``unified_pathfinder.py:2550-2659``): seeds ``(global node, cost)``
    start with label ``float(cost) + float(pen)`` (dist32 = float32 of it, no
    parent); a target is popped but not expanded and keeps the first target
    whose ``label + target cost`` is strictly below the best so far; the heap
    runs until empty.  Returns ``(path, entry_layer, exit_layer)`` or None
    (a one-node path is None)."""
    R = len(roi_nodes)
    dist = np.full(R, np.inf, dtype=np.float32)
    parent = np.full(R, -1, dtype=np.int32)
    visited = np.zeros(R, dtype=bool)
    heap = []
    for g, c in src_seeds:
        r = int(global_to_roi[g])
        if r >= 0:
            sc = float(c)
            if node_penalty is not None:
                sc += float(node_penalty[r])
            dist[r] = sc
            heapq.heappush(heap, (sc, r))
    targets = {}
    for g, c in dst_targets:
        r = int(global_to_roi[g])
        if r >= 0:
            targets[r] = (g, c)
    if not heap or not targets:
        return None
    ip = indptr.tolist() if hasattr(indptr, "tolist") else indptr
    best, best_total = None, np.inf
    scanned = settled = 0
    while heap:
        du, u = heapq.heappop(heap)
        if visited[u]:
            continue
        visited[u] = True
        settled += 1
        if u in targets:
            total = du + targets[u][1]
            if total < best_total:
                best_total, best = total, u
            continue
        ug = int(roi_nodes[u])
        for ei in range(ip[ug], ip[ug + 1]):
            scanned += 1
            v = int(global_to_roi[int(indices[ei])])
            if v < 0 or visited[v]:
                continue
            alt = du + float(costs[ei])
            if node_penalty is not None:
                alt += float(node_penalty[v])
            if alt < dist[v]:
                dist[v] = alt
                parent[v] = u
                heapq.heappush(heap, (alt, v))
    if stats is not None:
        stats["scanned"] = stats.get("scanned", 0) + scanned
        stats["settled"] = stats.get("settled", 0) + settled
    if best is None:
        return None
    path, cur = [], best
    while cur != -1:
        path.append(int(roi_nodes[cur]))
        cur = int(parent[cur])
    path.reverse()
    if len(path) <= 1:
        return None
    if plane:
        return path, path[0] // plane, path[-1] // plane
    return path, 0, 0


# --- C restatement (same semantics, ~100x faster) ------------------------------
_CLIB = None


def _clib():
    global _CLIB
    if _CLIB is None:
        import ctypes
        from . import build as _b
        lib = ctypes.CDLL(_b.build())
        P = ctypes.c_void_p
        lib.oracle_heap_dijkstra.argtypes = [ctypes.c_int32, ctypes.c_int32, P, P, P, P, ctypes.c_int32, P, P, P,
                                             ctypes.POINTER(ctypes.c_int32), P, ctypes.c_int32]
        lib.oracle_heap_dijkstra.restype = ctypes.c_int
        _CLIB = lib
    return _CLIB


def find_path_roi_c(indptr, indices, src, dst, costs, roi_nodes, global_to_roi, node_penalty=None,
                    stats=None) -> Optional[List[int]]:
    """``find_path_roi`` through ``oracle/csrc/heap_dijkstra.c``."""
    import ctypes
    lib = _clib()
    ip = np.ascontiguousarray(indptr, dtype=np.int32)
    ix = np.ascontiguousarray(indices, dtype=np.int32)
    c = np.ascontiguousarray(costs, dtype=np.float32)
    roi = np.ascontiguousarray(roi_nodes, dtype=np.int32)
    g2r = np.ascontiguousarray(global_to_roi, dtype=np.int32)
    pen = None if node_penalty is None else np.ascontiguousarray(node_penalty, dtype=np.float32)
    out = np.empty(max(len(roi), 2), dtype=np.int32)
    n = ctypes.c_int32(0)
    st = np.zeros(2, dtype=np.int64)
    rc = lib.oracle_heap_dijkstra(int(src), int(dst), ip.ctypes.data, ix.ctypes.data, c.ctypes.data,
                                  roi.ctypes.data, len(roi), g2r.ctypes.data,
                                  None if pen is None else pen.ctypes.data, out.ctypes.data, ctypes.byref(n),
                                  st.ctypes.data, len(ip) - 1)
    if rc < 0:
        raise MemoryError("oracle heap Dijkstra allocation failed")
    if stats is not None:
        stats["scanned"] = stats.get("scanned", 0) + int(st[0])
        stats["settled"] = stats.get("settled", 0) + int(st[1])
    if rc != 0:
        return None
    return out[: n.value].tolist()
