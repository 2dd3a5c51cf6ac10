"""Generate the geometry fixture (F4): the reference's own
``PathFinderRouter._generate_geometry_from_paths`` (unified_pathfinder.py:
11439-11563) on the final paths of the two pinned routing runs.

    python tests/golden/make_geometry_golden.py /path/to/OrthoRoute

Writes tests/golden/geometry.json: per run the lattice, board bounds, final
paths and the reference's tracks and vias.  The tests only read the file.
"""
from __future__ import annotations

import json
import logging
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as mg  # noqa: E402


def main(ref_root):
    sys.path.insert(0, ref_root)
    logging.disable(logging.CRITICAL)
    from orthoroute.algorithms.manhattan import unified_pathfinder as up
    from orthoroute.domain.models.board import Board, Component, Coordinate, Net, Pad
    out = {}
    for tag, (nx, ny, nz, n_nets, iters, seed) in {
        "r0": (24, 24, 6, 24, 6, 101),
        "r1": (28, 24, 8, 36, 8, 202),
    }.items():
        cfg = up.PathFinderConfig()
        cfg.use_gpu = False
        cfg.portal_enabled = False
        cfg.max_iterations = iters
        cfg.preferred_layer_directions = mg.default_dirs(nz)
        router = up.PathFinderRouter(config=cfg, use_gpu=False)
        router.initialize_graph(mg.make_board(Board, Component, Coordinate, Net, Pad, nx, ny, nz))
        reqs = mg.seeded_two_pin_nets(nx, ny, nz, n_nets, seed, dmin=4, dmax=40)
        router.route_multiple_nets(reqs)
        tracks, vias = router._generate_geometry_from_paths()
        geom = router.lattice.geom
        out[tag] = dict(
            nx=nx, ny=ny, nz=nz,
            bounds=[geom.min_x, geom.min_y, geom.max_x, geom.max_y],
            pitch=geom.pitch, grid_min=[geom.grid_min_x, geom.grid_min_y],
            layer_names=list(cfg.layer_names), track_width=cfg.track_width,
            via_diameter=cfg.via_diameter, via_drill=cfg.via_drill,
            axes=[router.lattice.get_allowed_axes(z) for z in range(nz)],
            paths=[[k, [int(x) for x in v]] for k, v in router.net_paths.items()],
            tracks=tracks, vias=vias)
    with open(os.path.join(HERE, "geometry.json"), "w") as f:
        json.dump(out, f, sort_keys=True)
    print("wrote", os.path.join(HERE, "geometry.json"))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
