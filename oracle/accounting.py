"""Oracle A2–A5: edge accounting and via pools (CPU restatement, numpy float32).

Every expression keeps the reference's numpy dtypes and operation order so the
float32 results are bit-identical (numpy 2 treats Python scalars as weak, so
``f32_array * python_float`` stays float32).

Reference: ``orthoroute/algorithms/manhattan/unified_pathfinder.py``

* ``EdgeAccountant.commit_path / clear_path``           ``:1096-1135``
* ``EdgeAccountant.update_history``                     ``:1226-1289``
* ``EdgeAccountant.update_present_ema``                 ``:1291-1299``
* ``EdgeAccountant.update_costs``                       ``:1301-1384``
* ``begin_live_present_costs / refresh_live_present``   ``:1386-1422``
* via pools: ``_accumulate_via_usage_for_path``         ``:4470-4546``
  via-present EMA + z prefix                            ``:6279-6303``
  ``_apply_via_pooling_penalties`` (CPU branch)         ``:5884-5980``
  ``_block_via_edges_with_collisions`` (CPU branch)     ``:6094-6161``
  ``_build_via_edge_metadata`` (CPU branch)             ``:9930-9979``
* ``_compute_layer_bias``                               ``:8451-8534``
"""
from __future__ import annotations

from typing import Dict, List, Optional

import numpy as np

JITTER_MOD = 9973
JITTER_SCALE = 1e-6


def jitter(E: int) -> np.ndarray:
    """``arange(E, float32) % 9973 * 1e-6`` (``:1378-1384``)."""
    j = np.arange(E, dtype=np.float32) % JITTER_MOD
    return j * JITTER_SCALE


class Accountant:
    """State of ``EdgeAccountant`` for one lattice."""

    def __init__(self, E: int):
        self.E = E
        self.canonical: Dict[int, int] = {}
        self.present = np.zeros(E, dtype=np.float32)
        self.present_ema = np.zeros(E, dtype=np.float32)
        self.history = np.zeros(E, dtype=np.float32)
        self.capacity = np.ones(E, dtype=np.float32)
        self.total_cost: Optional[np.ndarray] = None
        self.blocked_edges: Optional[np.ndarray] = None
        self._present_cost_scale = 1.0
        self._live_static_cost = None

    # -- canonical / present -------------------------------------------------
    def refresh_from_canonical(self):
        self.present.fill(0)
        if not self.canonical:
            return
        idx = np.fromiter(self.canonical.keys(), dtype=np.int64, count=len(self.canonical))
        cnt = np.fromiter(self.canonical.values(), dtype=np.float32, count=len(self.canonical))
        self.present[idx] = cnt

    def commit_path(self, edge_indices: List[int]):
        if not edge_indices:
            return
        for i in edge_indices:
            self.canonical[i] = self.canonical.get(i, 0) + 1
        np.add.at(self.present, np.asarray(edge_indices, dtype=np.int64), 1.0)

    def clear_path(self, edge_indices: List[int]):
        if not edge_indices:
            return
        for i in edge_indices:
            if i in self.canonical:
                self.canonical[i] -= 1
                if self.canonical[i] <= 0:
                    del self.canonical[i]
        np.add.at(self.present, np.asarray(edge_indices, dtype=np.int64), -1.0)
        np.maximum(self.present, 0, out=self.present)

    # -- costs ---------------------------------------------------------------
    def update_present_ema(self, beta: float = 0.40):
        self.present_ema = beta * self.present + (1.0 - beta) * self.present_ema

    def update_costs(self, base_costs, pres_fac, hist_weight=1.0, add_jitter=True,
                     via_cost_multiplier=1.0, base_cost_weight=0.01, *,
                     edge_layer=None, layer_bias_per_layer=None, edge_kind=None):
        over = np.maximum(0, self.present_ema - self.capacity)
        have_bias = (edge_layer is not None) and (layer_bias_per_layer is not None) and (edge_kind is not None)
        per_edge_bias = 1.0
        if have_bias:
            per_edge_bias = np.where(edge_kind == 0, layer_bias_per_layer[edge_layer], 1.0)
        adjusted = base_costs * via_cost_multiplier * base_cost_weight * per_edge_bias
        if have_bias:
            present_term = (pres_fac * per_edge_bias) * over
            self._present_cost_scale = pres_fac * per_edge_bias
        else:
            present_term = pres_fac * over
            self._present_cost_scale = float(pres_fac)
        self.total_cost = adjusted + present_term + hist_weight * self.history
        if self.blocked_edges is not None:
            self.total_cost[self.blocked_edges] = np.float32("inf")
        if add_jitter:
            self.total_cost += jitter(len(self.total_cost))

    def begin_live_present_costs(self):
        scale = self._present_cost_scale
        iteration_over = np.maximum(0, self.present_ema - self.capacity)
        self._live_static_cost = self.total_cost - scale * iteration_over
        prospective = np.maximum(0, self.present + 1.0 - self.capacity)
        self.total_cost[:] = self._live_static_cost + scale * prospective

    def refresh_live_present_costs(self, edge_indices: List[int]):
        if not edge_indices or self._live_static_cost is None:
            return
        ea = np.asarray(edge_indices, dtype=np.int64)
        scale = self._present_cost_scale
        prospective = np.maximum(0, self.present[ea] + 1.0 - self.capacity[ea])
        edge_scale = scale if np.isscalar(scale) else scale[ea]
        self.total_cost[ea] = self._live_static_cost[ea] + edge_scale * prospective

    def update_history(self, gain, base_costs=None, history_cap_multiplier=10.0,
                       decay_factor=0.98, use_raw_present=False):
        self.history *= decay_factor
        src = self.present if use_raw_present else self.present_ema
        over = np.maximum(0, src - self.capacity)
        inc = gain * over
        if base_costs is not None:
            inc = np.minimum(inc, history_cap_multiplier * base_costs)
        self.history += inc

    def compute_edge_overuse(self, canonical_mask: Optional[np.ndarray]):
        """Edge part of ``compute_overuse`` (``:1137-1166``)."""
        eo = np.maximum(0, self.present - self.capacity)
        if canonical_mask is not None:
            eo = eo[canonical_mask]
        return int(eo.sum()), int(np.count_nonzero(eo))


# -- layer bias ----------------------------------------------------------------
class LayerBiasState:
    """``_compute_layer_bias`` EMA (``:8451-8534``), alpha 0.88, max_boost 1.8."""

    def __init__(self):
        self.ema = None

    def compute(self, present_ema, capacity, edge_layer, num_layers, path_node_use,
                alpha=0.88, max_boost=1.80, depth_alpha=0.0):
        over = np.maximum(0, present_ema - capacity)
        per_layer = np.bincount(edge_layer, weights=over, minlength=num_layers)
        if path_node_use is not None and num_layers > 0 and path_node_use.size % num_layers == 0:
            pno = np.maximum(0, path_node_use - 1)
            per_layer = per_layer + pno.reshape(num_layers, -1).sum(axis=1)
        maxv = float(per_layer.max())
        if maxv <= 1e-9:
            raw = np.ones(num_layers, dtype=np.float32)
        else:
            raw = 1.0 + 0.75 * (per_layer / maxv)
        if depth_alpha:
            raw = raw + depth_alpha * np.arange(num_layers, dtype=np.float32)
        if self.ema is None:
            self.ema = raw.astype(np.float32)
        else:
            self.ema = (alpha * self.ema + (1.0 - alpha) * raw).astype(np.float32)
        ceiling = max_boost + depth_alpha * max(0, num_layers - 1)
        self.ema = np.clip(self.ema, 1.0, ceiling)
        return self.ema


# -- via pools -------------------------------------------------------------------
class ViaPools:
    """Via column / segment pools of one lattice (``:3019-3048``)."""

    def __init__(self, nx, ny, nz, col_cap=4, seg_cap=2):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.col_cap = np.full((nx, ny), col_cap, dtype=np.int16)
        self.col_use = np.zeros((nx, ny), dtype=np.int16)
        self.col_pres = np.zeros((nx, ny), dtype=np.float32)
        self.segZ = nz - 2 if nz > 2 else 0
        self.has_seg = nz > 2
        if self.has_seg:
            self.seg_cap = np.full((nx, ny, self.segZ), seg_cap, dtype=np.int8)
            self.seg_use = np.zeros((nx, ny, self.segZ), dtype=np.int16)
            self.seg_pres = np.zeros((nx, ny, self.segZ), dtype=np.float32)
            self.seg_prefix = np.zeros((nx, ny, self.segZ), dtype=np.float32)
            self.seg_pres_via = None

    def accumulate_path(self, path, col_use, seg_use):
        """``_accumulate_via_usage_for_path`` (``:4470-4546``) without keepouts."""
        plane = self.nx * self.ny
        prev_xy = None
        run_lo = run_hi = None
        for u, v in zip(path, path[1:]):
            zu, ru = divmod(int(u), plane)
            yu, xu = divmod(ru, self.nx)
            zv, rv = divmod(int(v), plane)
            yv, xv = divmod(rv, self.nx)
            if xu == xv and yu == yv and zu != zv:
                if (xu, yu) != prev_xy:
                    col_use[xu, yu] += 1
                    run_lo = run_hi = None
                prev_xy = (xu, yu)
                if seg_use is not None:
                    z_lo, z_hi = min(zu, zv), max(zu, zv)
                    z_lo = max(1, min(z_lo, self.nz - 2))
                    z_hi = max(1, min(z_hi, self.nz - 2))
                    for z in range(z_lo, z_hi):
                        if run_lo is not None and run_lo <= z < run_hi:
                            continue
                        s = z - 1
                        if 0 <= s < self.segZ:
                            seg_use[xu, yu, s] += 1
                    if z_hi > z_lo:
                        run_lo = z_lo if run_lo is None else min(run_lo, z_lo)
                        run_hi = z_hi if run_hi is None else max(run_hi, z_hi)
            else:
                prev_xy = None
                run_lo = run_hi = None

    def rebuild(self, paths):
        col = np.zeros((self.nx, self.ny), dtype=np.int16)
        seg = np.zeros((self.nx, self.ny, self.segZ), dtype=np.int16) if self.has_seg else None
        for p in paths:
            if p and len(p) > 1:
                self.accumulate_path(p, col, seg)
        self.col_use[:] = col
        if self.has_seg:
            self.seg_use[:] = seg

    def update_presence(self, alpha=0.6, beta=0.4):
        """Via-present EMA and z prefix (``:6279-6303``)."""
        over = np.maximum(0, self.col_use - self.col_cap).astype(np.float32)
        self.col_pres = alpha * over + beta * self.col_pres
        if self.has_seg:
            over = np.maximum(0, self.seg_use - self.seg_cap).astype(np.float32)
            prev = self.seg_pres_via if self.seg_pres_via is not None else self.seg_pres
            self.seg_pres_via = alpha * over + beta * prev
            self.seg_pres = self.seg_pres_via.copy()
            np.cumsum(self.seg_pres, axis=2, out=self.seg_prefix)

    def spatial_overuse_total(self) -> int:
        t = int(np.maximum(0, self.col_use - self.col_cap).sum())
        if self.has_seg:
            t += int(np.maximum(0, self.seg_use - self.seg_cap).sum())
        return t


def via_edge_metadata(csr):
    """``_build_via_edge_metadata`` CPU branch (``:9930-9979``)."""
    idx = np.where(csr.edge_kind.astype(bool))[0]
    if idx.size == 0:
        return None
    u = np.searchsorted(csr.indptr, idx, side='right') - 1
    v = csr.indices[idx]
    plane = csr.nx * csr.ny
    xu = (u % plane) % csr.nx
    yu = (u % plane) // csr.nx
    zu = u // plane
    zv = v // plane
    z_lo = np.clip(np.minimum(zu, zv), 1, csr.nz - 2)
    z_hi = np.clip(np.maximum(zu, zv), 1, csr.nz - 2)
    return {'indices': idx.astype(np.int32),
            'xy': np.stack([xu, yu], axis=1).astype(np.int32),
            'z_lo': z_lo.astype(np.int32), 'z_hi': z_hi.astype(np.int32)}


def apply_via_pooling_penalties(total_cost, meta, pools: ViaPools, layer_bias, pres_fac,
                                col_weight=1.0, seg_weight=1.0, k=0.20):
    """CPU branch of ``_apply_via_pooling_penalties`` (``:5884-5980``)."""
    if meta is None:
        return
    n = len(meta['indices'])
    xy, z_lo, z_hi = meta['xy'], meta['z_lo'], meta['z_hi']
    pen = np.zeros(n, dtype=np.float32)
    pen += col_weight * pools.col_pres[xy[:, 0], xy[:, 1]]
    if pools.has_seg:
        hi = z_hi - 2
        lo = z_lo - 2
        valid = z_hi > z_lo
        hv = (hi >= 0) & (hi < pools.segZ)
        lv = (lo >= 0) & (lo < pools.segZ)
        ph = np.zeros(n, dtype=np.float32)
        pl = np.zeros(n, dtype=np.float32)
        if np.any(hv):
            ph[hv] = pools.seg_prefix[xy[hv, 0], xy[hv, 1], hi[hv]]
        if np.any(lv):
            pl[lv] = pools.seg_prefix[xy[lv, 0], xy[lv, 1], lo[lv]]
        pen += seg_weight * ((ph - pl) * valid)
    if layer_bias is not None:
        sb = layer_bias[z_lo]
        db = layer_bias[z_hi]
        disc = (1.0 - k * np.maximum(sb, 0.0)) * (1.0 + 0.5 * k * np.maximum(db, 0.0))
        pen *= disc
    mask = pen > 0
    total_cost[meta['indices'][mask]] += pres_fac * pen[mask]


def block_via_edges(total_cost, meta, pools: ViaPools):
    """CPU branch of ``_block_via_edges_with_collisions`` (``:6094-6161``)."""
    if meta is None:
        return 0
    xy, z_lo, z_hi = meta['xy'], meta['z_lo'], meta['z_hi']
    blocked = pools.col_use[xy[:, 0], xy[:, 1]] >= pools.col_cap[xy[:, 0], xy[:, 1]]
    if pools.has_seg:
        for z in range(1, pools.nz - 1):
            s = z - 1
            if not (0 <= s < pools.segZ):
                continue
            spans = (z_lo <= z) & (z < z_hi)
            full = pools.seg_use[xy[:, 0], xy[:, 1], s] >= pools.seg_cap[xy[:, 0], xy[:, 1], s]
            blocked |= spans & full
    total_cost[meta['indices'][blocked]] = np.float32('inf')
    return int(blocked.sum())
