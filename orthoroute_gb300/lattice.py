"""Host-side description of the 3-D Manhattan routing lattice.

Mirrors ``Lattice3D`` (orthoroute/algorithms/manhattan/unified_pathfinder.py
:1429-1955) and ``KiCadGeometry`` (pathfinder/kicad_geometry.py:14-75):
node ``z*Nx*Ny + y*Nx + x``; F.Cu vertical then alternating H/V unless the
layer axes are given; lateral arcs on inner layers only (all layers on
2-layer boards); via pairs full blind/buried up to 18 layers, adjacent-only
beyond; via cost ``via_cost*(1+0.15*(span-1))`` or ``via_cost*4`` for
adjacent-only stacks; via sites filtered by the centre-spacing policy.

The device builds the CSR from the per-layer partner table produced here.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np


def default_layer_dirs(nz: int) -> List[str]:
    return ['v'] + ['h' if z % 2 == 1 else 'v' for z in range(1, nz)]


def _via_site_mode(spacing: float, pitch: float) -> int:
    """0 all sites, 1 checkerboard, k>=2 stride k (``_via_site_policy`` :1604-1614)."""
    spacing = max(0.0, float(spacing))
    if spacing <= pitch + 1e-9:
        return 0
    if spacing <= pitch * math.sqrt(2.0) + 1e-9:
        return 1
    return max(2, int(math.ceil(spacing / pitch)))


@dataclass
class Lattice:
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

    def __post_init__(self):
        if self.layer_dirs is None:
            self.layer_dirs = default_layer_dirs(self.nz)
        self.layer_dirs = [str(a).strip().lower() for a in self.layer_dirs]
        if len(self.layer_dirs) != self.nz or any(a not in ("h", "v") for a in self.layer_dirs):
            raise ValueError("layer_dirs must give one 'h'/'v' entry per layer")

    # -- geometry -----------------------------------------------------------
    @property
    def plane(self) -> int:
        return self.nx * self.ny

    @property
    def num_nodes(self) -> int:
        return self.nx * self.ny * self.nz

    def node_idx(self, x: int, y: int, z: int) -> int:
        return z * self.plane + y * self.nx + x

    def idx_to_coord(self, n: int) -> Tuple[int, int, int]:
        z, r = divmod(int(n), self.plane)
        y, x = divmod(r, self.nx)
        return x, y, z

    def allowed_axes(self, z: int) -> List[str]:
        """Axes a planar move on layer z may take (``get_allowed_axes``)."""
        axis = self.layer_dirs[z]
        other = "v" if axis == "h" else "h"
        return [axis] + ([other] if math.isfinite(self.wrong_way_cost_multiplier) else [])

    def lateral_layers(self) -> List[int]:
        return list(range(1, self.nz - 1)) if self.nz > 2 else list(range(self.nz))

    def via_pairs(self) -> List[Tuple[int, int]]:
        if self.allowed_via_spans is not None:
            pairs = {(min(int(a), int(b)), max(int(a), int(b))) for a, b in self.allowed_via_spans
                     if a != b and 0 <= a < self.nz and 0 <= b < self.nz}
            return sorted(pairs)
        if self.nz <= 2:
            return [(0, 1)]
        any_via = self.allow_any_layer_via if self.allow_any_layer_via is not None else self.nz <= 18
        inner = range(1, self.nz - 1)
        if any_via:
            pairs = {(a, b) for a in inner for b in inner if a < b} | {(0, z) for z in inner}
        else:
            pairs = {(z, z + 1) for z in range(0, self.nz - 2)}
        return sorted(pairs)

    def via_pair_cost(self, a: int, b: int, adjacent_only: bool) -> float:
        if adjacent_only:
            return self.via_cost * self.adjacent_via_step_scale
        return self.via_cost * (1.0 + 0.15 * (abs(b - a) - 1))

    # -- device descriptor ----------------------------------------------------
    def descriptor(self):
        """Return (ogr_lattice_desc, keep-alive arrays)."""
        from ._lib import LatticeDesc
        pairs = self.via_pairs()
        adjacent_only = self.nz > 2 and bool(pairs) and all(abs(b - a) == 1 for a, b in pairs)
        site = _via_site_mode(self.min_via_center_spacing, self.pitch)
        partners = [[] for _ in range(self.nz)]
        for a, b in pairs:
            c = np.float32(self.via_pair_cost(a, b, adjacent_only))
            partners[a].append((b, c))
            partners[b].append((a, c))
        ptr = np.zeros(self.nz + 1, dtype=np.int32)
        zs, cs, ss = [], [], []
        for z in range(self.nz):
            for zz, c in sorted(partners[z]):
                zs.append(zz)
                cs.append(c)
                ss.append(site)
            ptr[z + 1] = len(zs)
        axis = np.zeros(self.nz, dtype=np.uint8)
        for z in self.lateral_layers():
            axis[z] = 1 if self.layer_dirs[z] == 'h' else 2
        arrs = dict(axis=axis, ptr=ptr, z=np.asarray(zs, dtype=np.int32),
                    cost=np.asarray(cs, dtype=np.float32), site=np.asarray(ss, dtype=np.int32))
        ww = self.pitch * self.wrong_way_cost_multiplier if math.isfinite(self.wrong_way_cost_multiplier) else -1.0
        d = LatticeDesc(self.nx, self.ny, self.nz, float(np.float32(self.pitch)), float(np.float32(ww)),
                        arrs["axis"].ctypes.data, arrs["ptr"].ctypes.data, arrs["z"].ctypes.data,
                        arrs["cost"].ctypes.data, arrs["site"].ctypes.data)
        return d, arrs
