"""Host-side policy helpers of the router (no GPU): the vectorised via-pool
membership, barrel node expansion and per-net overuse sums agree with the
per-hop loops they replace (the reference's own formulation)."""
from collections import defaultdict

import numpy as np
import pytest

from orthoroute_gb300 import router as R


class _Host:
    """Just the attributes the helpers read."""


def _host(nx=9, ny=7, nz=8, seg_z=6):
    h = _Host()
    h.nx, h.ny, h.nz, h.plane = nx, ny, nz, nx * ny
    h.pools = type("Pools", (), {"segZ": seg_z})()
    return h


def _rand_path(rng, h, n):
    p = [int(rng.integers(0, h.plane * h.nz))]
    for _ in range(n):
        z, r = divmod(p[-1], h.plane)
        if rng.random() < 0.4:
            z2 = int(rng.integers(0, h.nz))
            p.append((z2 if z2 != z else (z + 1) % h.nz) * h.plane + r)
        else:
            p.append(z * h.plane + (r + 1) % h.plane)
    return p


def _coord(h, n):
    z, r = divmod(int(n), h.plane)
    y, x = divmod(r, h.nx)
    return x, y, z


@pytest.mark.parametrize("seed", range(4))
def test_via_pool_members_match_hop_loop(seed):
    rng = np.random.default_rng(seed)
    h = _host()
    h.net_paths = {f"N{i}": _rand_path(rng, h, int(rng.integers(1, 30))) for i in range(40)}
    h.net_paths["N5"] = []
    col_over = rng.random((h.nx, h.ny)) < 0.3
    seg_over = rng.random((h.nx, h.ny, h.pools.segZ)) < 0.3
    got = R.PathFinderRouter._via_pool_members(h, col_over, seg_over)
    want = defaultdict(set)
    for name, path in h.net_paths.items():
        if not path or len(path) < 2:
            continue
        res = set()
        for u, v in zip(path, path[1:]):
            xu, yu, zu = _coord(h, u)
            xv, yv, zv = _coord(h, v)
            if xu != xv or yu != yv or zu == zv:
                continue
            if col_over[xu, yu]:
                res.add(("col", xu, yu))
            zl = max(1, min(min(zu, zv), h.nz - 2))
            zh = max(1, min(max(zu, zv), h.nz - 2))
            for z in range(zl, zh):
                if 0 <= z - 1 < h.pools.segZ and seg_over[xu, yu, z - 1]:
                    res.add(("seg", xu, yu, z - 1))
        for r in res:
            want[r].add(name)
    assert dict(got) == dict(want)


def test_via_nodes_match_hop_loop():
    rng = np.random.default_rng(7)
    h = _host()
    for _ in range(50):
        path = _rand_path(rng, h, int(rng.integers(0, 25)))
        nodes = set()
        for u, v in zip(path, path[1:]):
            zu, ru = divmod(u, h.plane)
            zv, rv = divmod(v, h.plane)
            if ru != rv or zu == zv:
                continue
            for z in range(min(zu, zv), max(zu, zv) + 1):
                nodes.add(z * h.plane + ru)
        assert R.PathFinderRouter._via_nodes(h, path) == sorted(nodes)


def test_edge_over_sums_match_generator_sums():
    rng = np.random.default_rng(3)
    h = _host()
    h._eidx = None
    h.net_to_edges = {f"N{i}": rng.integers(0, 500, size=int(rng.integers(0, 40))).astype(np.int64)
                      for i in range(30)}
    h._edge_index = lambda: R.PathFinderRouter._edge_index(h)
    over_idx = np.unique(rng.integers(0, 500, size=60)).astype(np.int64)
    over_val = (rng.random(over_idx.size).astype(np.float32) * 3).astype(np.float64)
    over_map = dict(zip(over_idx.tolist(), over_val.tolist()))
    names, sums, hit = R.PathFinderRouter._edge_over(h, over_idx, over_val)
    for i, n in enumerate(names):
        edges = h.net_to_edges[n].tolist()
        assert sums[i] == sum(float(over_map[e]) for e in edges if e in over_map)
        assert sums[i] == sum(float(over_map.get(e, 0.0)) for e in edges)
        assert bool(hit[i]) == any(e in over_map for e in edges)
