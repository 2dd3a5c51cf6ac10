"""F4 geometry emission against the reference's own output on the final
paths of the two pinned routing runs (tests/golden/geometry.json)."""
import json
import os

import pytest

from orthoroute_gb300.geometry import GridGeometry, coalesce_vertical_runs, generate_geometry

G = os.path.join(os.path.dirname(__file__), "golden", "geometry.json")
GOLD = json.load(open(G))


@pytest.mark.parametrize("tag", sorted(GOLD))
def test_geometry_matches_reference(tag):
    d = GOLD[tag]
    geom = GridGeometry(d["bounds"], d["pitch"])
    assert [geom.grid_min_x, geom.grid_min_y] == d["grid_min"]
    tracks, vias = generate_geometry(dict((k, v) for k, v in d["paths"]), d["nx"], d["ny"], d["nz"], d["axes"], geom, d["layer_names"],
                                     d["track_width"], d["via_diameter"], d["via_drill"])
    assert tracks == d["tracks"]
    assert vias == d["vias"]


def test_coalesce_vertical_runs():
    nx, plane = 4, 16

    def coord(n):
        z, r = divmod(n, plane)
        y, x = divmod(r, nx)
        return x, y, z
    p = [5, 5 + plane, 5 + 2 * plane, 6 + 2 * plane, 6 + plane, 6]
    assert coalesce_vertical_runs(p, coord) == [5, 5 + 2 * plane, 6 + 2 * plane, 6]
