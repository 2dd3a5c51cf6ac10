"""Golden vectors for the multi-source multi-sink search, made by the reference itself.

Run in a container that holds the reference checkout (read only):

    python tests/golden/make_multisource_golden.py /path/to/OrthoRoute

It builds a 40x36x6 lattice with the reference's ``Lattice3D``, extracts ROIs
with its ``ROIExtractor`` and calls ``SimpleDijkstra.find_path_multisource_multisink``
(``unified_pathfinder.py:2550-2659``) on seeded portal-like seed and target
sets (a column of entry layers over a pad, with per-layer costs), with and
without node penalties, tied costs, blocked arcs, a seed that is also a
target, and targets outside the ROI.  Inputs that are not regenerated from the
seed (ROI, seeds, targets, penalties) and the outputs go to
``tests/golden/multisource.npz``; the arc costs are regenerated from the seed
by ``multisource_costs`` below, which the tests share.
"""
from __future__ import annotations

import logging
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NX, NY, NZ = 40, 36, 6
CASES = 10


def multisource_costs(E, i):
    rng = np.random.default_rng(4100 + i)
    costs = (0.12 + rng.random(E) * 0.05).astype(np.float32)
    if i % 3 == 1:
        costs = (0.12 + rng.integers(0, 4, size=E) * 0.01).astype(np.float32)   # many ties
    if i % 4 == 3:
        costs[rng.choice(E, size=E // 20, replace=False)] = np.float32("inf")
    return costs


def portal_column(rng, x, y, plane, nx, nz, base):
    """Entry nodes over one pad: layers 1..nz-2 with rising layer costs."""
    return [(int(z * plane + y * nx + x), float(base + 0.05 * z + round(float(rng.random()) * 0.1, 3)))
            for z in range(1, nz - 1)]


def main(ref_root):
    sys.path.insert(0, ref_root)
    logging.disable(logging.WARNING)
    from orthoroute.algorithms.manhattan import unified_pathfinder as up

    L = up.Lattice3D((0, 0, (NX - 1) * 0.4 + 1e-6, (NY - 1) * 0.4 + 1e-6), 0.4, NZ,
                     preferred_layer_directions=["h" if z % 2 else "v" for z in range(NZ)])
    g = L.build_graph(0.7, allow_any_layer_via=True, min_via_center_spacing=0.4)
    E = len(g.indices)
    plane = NX * NY
    ex = up.ROIExtractor(g, lattice=L)
    S = up.SimpleDijkstra(g, L)
    out = {}
    for i in range(CASES):
        rng = np.random.default_rng(4200 + i)
        costs = multisource_costs(E, i)
        sx, sy = int(rng.integers(0, NX)), int(rng.integers(0, NY))
        dx, dy = int(rng.integers(0, NX)), int(rng.integers(0, NY))
        seeds = portal_column(rng, sx, sy, plane, NX, NZ, 0.0)
        targets = portal_column(rng, dx, dy, plane, NX, NZ, 0.02)
        if i % 2 == 1:       # a second candidate pad position on each side
            seeds += portal_column(rng, min(sx + 1, NX - 1), sy, plane, NX, NZ, 0.3)
            targets += portal_column(rng, dx, max(dy - 1, 0), plane, NX, NZ, 0.3)
        if i == 5:           # a seed that is also a target, too dear to win
            targets.append((seeds[0][0], 50.0))
        if i == 7:           # a seed that is also a target and wins: one-node path, None
            targets.append((seeds[1][0], 0.0))
        seeds = sorted(dict(seeds).items())
        targets = sorted(dict(targets).items())
        s0, d0 = seeds[0][0] % plane, targets[0][0] % plane
        roi, g2r = ex.extract_roi(s0 + plane, d0 + plane, stagnation_bonus=0.0)
        if i == 9:           # targets outside the ROI
            keep = np.asarray([n for n in roi if n not in dict(targets)], dtype=np.int32)
            g2r = np.full(len(g2r), -1, dtype=np.int32)
            g2r[keep] = np.arange(len(keep), dtype=np.int32)
            roi = keep
        pen = None
        if i % 2 == 0:
            pen = (rng.integers(0, 3, size=len(roi)) * 0.25 * (i + 1)).astype(np.float32)
        res = S.find_path_multisource_multisink(seeds, targets, costs, roi, g2r, node_penalty=pen)
        path, ent, exl = res if res else ([], -1, -1)
        out[f"m{i}_roi"] = np.asarray(roi, dtype=np.int32)
        out[f"m{i}_seeds"] = np.asarray([n for n, _ in seeds], dtype=np.int32)
        out[f"m{i}_seed_cost"] = np.asarray([c for _, c in seeds], dtype=np.float64)
        out[f"m{i}_targets"] = np.asarray([n for n, _ in targets], dtype=np.int32)
        out[f"m{i}_target_cost"] = np.asarray([c for _, c in targets], dtype=np.float64)
        if pen is not None:
            out[f"m{i}_pen"] = pen
        out[f"m{i}_path"] = np.asarray(path, dtype=np.int32)
        out[f"m{i}_layers"] = np.asarray([ent, exl], dtype=np.int32)
        print(i, len(roi), len(path), ent, exl)
    np.savez_compressed(os.path.join(HERE, "multisource.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
