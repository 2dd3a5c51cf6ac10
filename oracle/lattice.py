"""Oracle A1: 3-D Manhattan lattice → CSR graph (CPU restatement).

Follows ``orthoroute/algorithms/manhattan/unified_pathfinder.py``:

* node numbering ``z*Nx*Ny + y*Nx + x`` (``pathfinder/kicad_geometry.py:59-71``);
* layer axes: explicit per-layer list, else F.Cu 'v' then alternating
  h/v (``unified_pathfinder.py:1473-1499``);
* legal via pairs, built as a Python ``set`` in the same insertion order so
  its iteration order matches (``unified_pathfinder.py:1534-1586``,
  explicit spans ``:1734-1743``);
* lateral edges on inner layers only, preferred axis, then optional
  wrong-way axis, then via edges for every (x, y, pair) in set order
  (``unified_pathfinder.py:1811-1886``);
* via site policy per pair (``:1604-1654``, ``:1760-1789``);
* CSR = ``edge_array.sort(order='src', kind='mergesort')`` on the structured
  (src, dst, cost) array (``CSRGraph.finalize`` ``:935``).  numpy breaks ties
  on the fields not named in ``order``, so each row ends up sorted by
  destination id (then cost), not in insertion order;
  ``edge_layer = src // plane``, ``edge_kind = src_layer != dst_layer``.

The edges are produced vectorised and sorted lexicographically by
(src, dst, cost), which gives the reference's arrays byte for byte.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np


def default_layer_dirs(nz: int) -> List[str]:
    """F.Cu vertical, then In1=H, In2=V, ... (``unified_pathfinder.py:1491-1499``)."""
    return ['v'] + ['h' if z % 2 == 1 else 'v' for z in range(1, nz)]


def legal_via_pairs(nz: int, allow_any_layer_via: bool):
    """Same set, same insertion order as ``Lattice3D.get_legal_via_pairs``."""
    if nz <= 2:
        return {(0, 1)}
    routing = list(range(1, nz - 1))
    if allow_any_layer_via:
        pairs = set()
        for z1 in routing:
            for z2 in routing:
                if z1 < z2:
                    pairs.add((z1, z2))
        for z in routing:
            pairs.add((0, z))
        return pairs
    return {(z, z + 1) for z in range(0, nz - 2)}


def via_site_policy(required_spacing: float, pitch: float) -> Tuple[str, int]:
    """``Lattice3D._via_site_policy`` (``unified_pathfinder.py:1604-1614``)."""
    required_spacing = max(0.0, float(required_spacing))
    if required_spacing <= pitch + 1e-9:
        return "all", 1
    if required_spacing <= pitch * math.sqrt(2.0) + 1e-9:
        return "checkerboard", 1
    return "stride", max(2, int(math.ceil(required_spacing / pitch)))


def site_mask(nx: int, ny: int, mode: str, stride: int) -> np.ndarray:
    """Boolean [Nx, Ny] of legal via sites (``_matches_via_site_policy``)."""
    xs = np.arange(nx)[:, None]
    ys = np.arange(ny)[None, :]
    if mode == "all":
        return np.ones((nx, ny), dtype=bool)
    if mode == "checkerboard":
        return ((xs + ys) % 2) == 0
    return ((xs % stride) == 0) & ((ys % stride) == 0)


@dataclass
class LatticeSpec:
    nx: int
    ny: int
    nz: int
    pitch: float = 0.4
    layer_dirs: Optional[List[str]] = None
    via_cost: float = 0.7
    allow_any_layer_via: Optional[bool] = None
    allowed_via_spans: Optional[Sequence[Tuple[int, int]]] = None
    adjacent_via_step_scale: float = 4.0
    min_via_center_spacing: float = 0.4
    wrong_way_cost_multiplier: float = float("inf")
    lateral_all: bool = False

    def dirs(self) -> List[str]:
        return list(self.layer_dirs) if self.layer_dirs is not None else default_layer_dirs(self.nz)

    def lateral_layers(self) -> List[int]:
        if self.lateral_all:
            return list(range(self.nz))
        if self.nz > 2:
            return list(range(1, self.nz - 1))
        return list(range(self.nz))

    def via_pairs_ordered(self) -> List[Tuple[int, int]]:
        """Legal pairs in the iteration order of the reference's set."""
        if self.allowed_via_spans is not None:
            s = {(min(int(a), int(b)), max(int(a), int(b)))
                 for a, b in self.allowed_via_spans
                 if a != b and 0 <= a < self.nz and 0 <= b < self.nz}
        else:
            any_via = self.allow_any_layer_via
            if any_via is None:
                any_via = self.nz <= 18
            s = legal_via_pairs(self.nz, any_via)
        return list(s)

    def via_pair_costs(self, pairs) -> List[float]:
        """Per-pair via cost in float64, as ``build_graph`` computes it (``:1870-1880``)."""
        adjacent_only = self.nz > 2 and len(pairs) > 0 and all(abs(b - a) == 1 for a, b in pairs)
        out = []
        for a, b in pairs:
            span = abs(b - a)
            if adjacent_only:
                out.append(self.via_cost * self.adjacent_via_step_scale)
            else:
                out.append(self.via_cost * (1.0 + 0.15 * (span - 1)))
        return out


@dataclass
class CSR:
    nx: int
    ny: int
    nz: int
    indptr: np.ndarray
    indices: np.ndarray
    base_costs: np.ndarray
    edge_layer: np.ndarray
    edge_kind: np.ndarray
    layer_dirs: List[str] = field(default_factory=list)
    via_pairs: List[Tuple[int, int]] = field(default_factory=list)

    @property
    def num_nodes(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def plane(self) -> int:
        return self.nx * self.ny

    def edge_src(self) -> np.ndarray:
        n = self.num_nodes
        return np.repeat(np.arange(n, dtype=np.int32), np.diff(self.indptr)).astype(np.int32)


def _interleave(u: np.ndarray, v: np.ndarray):
    src = np.empty(2 * u.size, dtype=np.int64)
    dst = np.empty(2 * u.size, dtype=np.int64)
    src[0::2] = u
    dst[0::2] = v
    src[1::2] = v
    dst[1::2] = u
    return src, dst


def build_csr(spec: LatticeSpec) -> CSR:
    """Build the CSR exactly as ``Lattice3D.build_graph`` + ``CSRGraph.finalize``."""
    nx, ny, nz = spec.nx, spec.ny, spec.nz
    plane = nx * ny
    n = plane * nz
    dirs = spec.dirs()
    pitch32 = np.float32(spec.pitch)
    srcs, dsts, costs = [], [], []

    def add_block(u, v, cost):
        s, d = _interleave(u, v)
        srcs.append(s)
        dsts.append(d)
        costs.append(np.full(s.size, np.float32(cost), dtype=np.float32))

    lat = spec.lateral_layers()
    for z in lat:
        if dirs[z] == 'h':
            y, x = np.meshgrid(np.arange(ny), np.arange(nx - 1), indexing='ij')
            u = z * plane + y.ravel() * nx + x.ravel()
            add_block(u, u + 1, pitch32)
        else:
            x, y = np.meshgrid(np.arange(nx), np.arange(ny - 1), indexing='ij')
            u = z * plane + y.ravel() * nx + x.ravel()
            add_block(u, u + nx, pitch32)
    if math.isfinite(spec.wrong_way_cost_multiplier):
        ww = spec.pitch * spec.wrong_way_cost_multiplier
        for z in lat:
            if dirs[z] == 'h':
                x, y = np.meshgrid(np.arange(nx), np.arange(ny - 1), indexing='ij')
                u = z * plane + y.ravel() * nx + x.ravel()
                add_block(u, u + nx, ww)
            else:
                y, x = np.meshgrid(np.arange(ny), np.arange(nx - 1), indexing='ij')
                u = z * plane + y.ravel() * nx + x.ravel()
                add_block(u, u + 1, ww)

    pairs = spec.via_pairs_ordered()
    pcost = spec.via_pair_costs(pairs)
    if pairs:
        pol = {p: via_site_policy(spec.min_via_center_spacing, spec.pitch) for p in pairs}
        masks = [site_mask(nx, ny, *pol[p]).ravel() for p in pairs]   # index = x*ny + y
        # insertion order: for x, for y, for pair
        xy = np.arange(nx * ny)
        xs, ys = xy // ny, xy % ny
        P = len(pairs)
        za = np.array([p[0] for p in pairs], dtype=np.int64)
        zb = np.array([p[1] for p in pairs], dtype=np.int64)
        keep = np.stack(masks, axis=1)                               # [nx*ny, P]
        base = (ys * nx + xs)[:, None]
        u = (za[None, :] * plane + base)[keep]
        v = (zb[None, :] * plane + base)[keep]
        c = np.broadcast_to(np.array(pcost, dtype=np.float64)[None, :], keep.shape)[keep]
        s, d = _interleave(u, v)
        srcs.append(s)
        dsts.append(d)
        cc = np.empty(s.size, dtype=np.float32)
        cc[0::2] = c.astype(np.float32)
        cc[1::2] = c.astype(np.float32)
        costs.append(cc)

    src = np.concatenate(srcs)
    dst = np.concatenate(dsts)
    cost = np.concatenate(costs)
    if src.size == 0:
        raise ValueError("Routing graph has no edges")
    order = np.lexsort((cost, dst, src))
    src = src[order]
    indices = dst[order].astype(np.int32)
    base_costs = cost[order].astype(np.float32)
    counts = np.bincount(src, minlength=n)
    indptr = np.zeros(n + 1, dtype=np.int32)
    indptr[1:] = np.cumsum(counts)
    edge_layer = (src // plane).astype(np.uint8)
    edge_kind = ((src // plane) != (indices // plane)).astype(np.uint8)
    return CSR(nx, ny, nz, indptr, indices, base_costs, edge_layer, edge_kind,
               layer_dirs=dirs, via_pairs=pairs)


def reverse_edge_index(csr: CSR) -> np.ndarray:
    """rev[e] = index of the arc v→u for arc e = u→v (lattice arcs come in pairs)."""
    src = csr.edge_src().astype(np.int64)
    dst = csr.indices.astype(np.int64)
    n = csr.num_nodes
    key_fwd = src * n + dst
    key_rev = dst * n + src
    order = np.argsort(key_fwd)
    pos = np.searchsorted(key_fwd[order], key_rev)
    return order[pos].astype(np.int32)
