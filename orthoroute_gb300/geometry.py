"""F4: geometry emission — routed node paths to track segments and vias.

Restates the reference's ``_generate_geometry_from_paths``
(``unified_pathfinder.py:11439-11563``) for tuple requests (no pad-escape
portals, no HDI stack), with ``_coalesce_vertical_runs`` (:11565-11596),
``_segment_world`` (:11138-11160) and ``_via_world`` (:11199-11230), and the
lattice-to-world mapping of ``KiCadGeometry`` (``pathfinder/kicad_geometry.py``:
24-50).  The output dicts have the reference's keys and float values (the
same Python float operations in the same order), so a router's geometry can
be compared with the reference's byte for byte.
"""
from __future__ import annotations

import os
from typing import Dict, List, Sequence, Tuple


class GridGeometry:
    """Pitch-aligned board grid from the board bounds (min_x, min_y, max_x, max_y)."""

    def __init__(self, bounds: Sequence[float], pitch: float):
        self.min_x, self.min_y, self.max_x, self.max_y = (float(v) for v in bounds)
        self.pitch = float(pitch)
        self.grid_min_x = round(self.min_x / self.pitch) * self.pitch
        self.grid_min_y = round(self.min_y / self.pitch) * self.pitch

    def lattice_to_world(self, x: int, y: int) -> Tuple[float, float]:
        return (self.grid_min_x + (x * self.pitch), self.grid_min_y + (y * self.pitch))

    def quantise(self, v: float, origin: float) -> float:
        return origin + round((v - origin) / self.pitch) * self.pitch


def _sign(v: int) -> int:
    return (v > 0) - (v < 0)


def coalesce_vertical_runs(path: Sequence[int], coord) -> List[int]:
    """Adjacent z hops at one (x, y) in one direction become one via span."""
    if len(path) < 3:
        return list(path)
    out = [path[0]]
    via_xy, via_dir = None, 0
    for prev, node in zip(path, path[1:]):
        x0, y0, z0 = coord(prev)
        x1, y1, z1 = coord(node)
        dz = z1 - z0
        vertical = x0 == x1 and y0 == y1 and dz != 0
        direction = _sign(dz) if vertical else 0
        if vertical and via_xy == (x0, y0) and direction == via_dir:
            out[-1] = node
        else:
            out.append(node)
        if vertical:
            via_xy, via_dir = (x0, y0), direction
        else:
            via_xy, via_dir = None, 0
    return out


def generate_geometry(net_paths: Dict[str, Sequence[int]], nx: int, ny: int, nz: int,
                      allowed_axes: Sequence[Sequence[str]], geom: GridGeometry, layer_names: Sequence[str],
                      track_width: float, via_diameter: float, via_drill: float) -> Tuple[List[dict], List[dict]]:
    """(tracks, vias) of every routed path, in net_paths order."""
    plane = nx * ny

    def coord(n):
        z, r = divmod(int(n), plane)
        y, x = divmod(r, nx)
        return x, y, z

    def lname(z):
        return layer_names[z] if z < len(layer_names) else f"L{z}"

    def segment(a, b, z, net):
        ax, ay, _ = coord(a)
        bx, by, _ = coord(b)
        ax_mm, ay_mm = geom.lattice_to_world(ax, ay)
        bx_mm, by_mm = geom.lattice_to_world(bx, by)
        return {"net": net, "layer": lname(z),
                "x1": geom.quantise(ax_mm, geom.grid_min_x), "y1": geom.quantise(ay_mm, geom.grid_min_y),
                "x2": geom.quantise(bx_mm, geom.grid_min_x), "y2": geom.quantise(by_mm, geom.grid_min_y),
                "width": track_width}

    def via(at, net, z0, z1):
        x, y, _ = coord(at)
        x_mm, y_mm = geom.lattice_to_world(x, y)
        if z0 > z1:
            z0, z1 = z1, z0
        return {"net": net, "x": geom.quantise(x_mm, geom.grid_min_x), "y": geom.quantise(y_mm, geom.grid_min_y),
                "from_layer": lname(z0), "to_layer": lname(z1), "diameter": via_diameter, "drill": via_drill}

    lateral_all = os.environ.get("ORTHO_LATERAL_ALL", "0") == "1"
    tracks, vias = [], []
    for net, path in net_paths.items():
        if not path:
            continue
        path = coalesce_vertical_runs(path, coord)
        run_start = prev = path[0]
        prev_dir = None
        prev_layer = coord(prev)[2]
        for node in path[1:]:
            x0, y0, z0 = coord(prev)
            x1, y1, z1 = coord(node)
            if z0 == z1 and (z0 == 0 or z0 == nz - 1) and not lateral_all:
                # the reference drops planar moves on the outer layers (none are in the graph)
                prev, prev_layer, run_start = node, z1, node
                continue
            dx, dy, dz = abs(x1 - x0), abs(y1 - y0), abs(z1 - z0)
            if dz == 0:
                if dx + dy != 1:
                    continue
                axis = "h" if dy == 0 else "v"
                if axis not in allowed_axes[z0]:
                    continue
            if z1 != z0:
                if prev != run_start:
                    tracks.append(segment(run_start, prev, prev_layer, net))
                vias.append(via(prev, net, z0, z1))
                run_start = node
                prev_dir = None
            else:
                d = (_sign(x1 - x0), _sign(y1 - y0))
                if prev_dir is not None and d != prev_dir:
                    tracks.append(segment(run_start, prev, prev_layer, net))
                    run_start = prev
                prev_dir = d
            prev, prev_layer = node, z1
        if prev != run_start:
            tracks.append(segment(run_start, prev, prev_layer, net))
    return tracks, vias
