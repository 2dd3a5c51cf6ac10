"""Oracle A6: bidirectional cost-blind BFS region of interest (CPU restatement).

Reference: ``ROIExtractor.extract_roi`` / ``extract_roi_bfs``
(``orthoroute/algorithms/manhattan/unified_pathfinder.py:2240-2384``).

The reference walks Python lists node by node.  Within one wave step the
marks it writes are a pure set function of the frontier (a node unseen at
the start of the step gets the wave's mark, a node seen by the other wave
becomes 3 and flags the meeting), so this restatement expands each frontier
with numpy and produces the same ``seen`` array, meeting depth and early
stop.  ROI order = ascending global id (``np.where(seen > 0)``), truncated
to 50,000 nodes with src/dst swapped to the front when they fall past the
cut (``:2359-2379``).
"""
from __future__ import annotations

import numpy as np

MAX_ROI_NODES = 50_000


def roi_radius(src, dst, nx, plane, stagnation_bonus=0.0):
    """``extract_roi`` radius (``:2240-2255``)."""
    sz, sr = divmod(int(src), plane)
    sy, sx = divmod(sr, nx)
    dz, dr = divmod(int(dst), plane)
    dy, dx = divmod(dr, nx)
    dist = abs(dx - sx) + abs(dy - sy)
    return max(60, int(dist * 0.75 + stagnation_bonus * 2.0))


def _expand(indptr, indices, blocked, frontier):
    if frontier.size == 0:
        return np.empty(0, dtype=np.int64)
    starts = indptr[frontier].astype(np.int64)
    ends = indptr[frontier + 1].astype(np.int64)
    lens = ends - starts
    tot = int(lens.sum())
    if tot == 0:
        return np.empty(0, dtype=np.int64)
    off = np.repeat(starts - np.concatenate(([0], np.cumsum(lens)[:-1])), lens)
    eids = np.arange(tot, dtype=np.int64) + off
    if blocked is not None:
        eids = eids[~blocked[eids]]
    return indices[eids].astype(np.int64)


def extract_roi_bfs(indptr, indices, N, src, dst, initial_radius=40, stagnation_bonus=0.0,
                    blocked=None, max_nodes=MAX_ROI_NODES, return_meta=False):
    seen = np.zeros(N, dtype=np.uint8)
    seen[src] = 1
    seen[dst] = 2
    q_src = np.array([src], dtype=np.int64)
    q_dst = np.array([dst], dtype=np.int64)
    depth = 0
    max_depth = min(int(initial_radius + stagnation_bonus * 2.0), 80)
    met = False
    meeting_depth = None
    halo = min(16, 2 + int(max(0.0, stagnation_bonus) / 0.6))

    def step(q, mark):
        nb = _expand(indptr, indices, blocked, q)
        if nb.size == 0:
            return np.empty(0, dtype=np.int64), False
        s = seen[nb]
        met_flag = bool(np.any((s != 0) & (s != mark)))
        fresh = np.unique(nb[s == 0])
        other = nb[(s != 0) & (s != mark)]
        seen[other] = 3
        seen[fresh] = mark
        return fresh, met_flag

    while depth < max_depth and (q_src.size or q_dst.size):
        q_src, m1 = step(q_src, 1)
        met = met or m1
        q_dst, m2 = step(q_dst, 2)
        met = met or m2
        depth += 1
        if met and meeting_depth is None:
            meeting_depth = depth
        if meeting_depth is not None and depth >= meeting_depth + halo:
            break
        if int((seen > 0).sum()) > max_nodes * 1.5:
            break

    roi = np.where(seen > 0)[0]
    must = [src, dst]
    missing = [n for n in must if n not in roi]
    if missing:
        roi = np.append(roi, missing)
    if roi.size > max_nodes:
        kept = [i for i, node in enumerate(roi) if node in must]
        for pos, k in enumerate(kept):
            if k >= max_nodes:
                roi[k], roi[pos] = roi[pos], roi[k]
        roi = roi[:max_nodes]
    g2r = np.full(N, -1, dtype=np.int32)
    g2r[roi] = np.arange(len(roi), dtype=np.int32)
    if return_meta:
        return roi, g2r, {"depth": depth, "meeting_depth": meeting_depth, "seen": seen}
    return roi, g2r


def extract_roi(indptr, indices, N, nx, plane, src, dst, stagnation_bonus=0.0, blocked=None):
    r = roi_radius(src, dst, nx, plane, stagnation_bonus)
    return extract_roi_bfs(indptr, indices, N, src, dst, initial_radius=r,
                           stagnation_bonus=stagnation_bonus, blocked=blocked)
