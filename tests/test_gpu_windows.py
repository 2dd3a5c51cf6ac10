"""Batched disjoint-ROI windows give exactly the sequential pass's results:
paths, per-net status (failures, fallbacks) and every state array, over
several passes (so rip-ups of earlier paths, window breaks on failed searches
and the undo of later rip-ups all occur)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _table(lat, nets, dev, bonus=0.0):
    n = len(nets)
    src = np.array([s for s, _ in nets], dtype=np.int32)
    dst = np.array([d for _, d in nets], dtype=np.int32)
    depth = np.empty(2 * n, dtype=np.int32)
    halo = np.empty(2 * n, dtype=np.int32)
    for i, (s, d) in enumerate(nets):
        sx, sy = s % lat.nx, (s // lat.nx) % lat.ny
        dx, dy = d % lat.nx, (d // lat.nx) % lat.ny
        dist = abs(sx - dx) + abs(sy - dy)
        for j, b in enumerate((bonus, bonus * 2)):
            radius = max(60, int(dist * 0.75 + b * 2.0))
            depth[2 * i + j] = min(int(radius + b * 2.0), 80)
            halo[2 * i + j] = min(16, 2 + int(max(0.0, b) / 0.6))
    arr = dict(src=src, dst=dst, id=np.arange(n, dtype=np.int32), full=np.zeros(n, dtype=np.int32), depth=depth,
               halo=halo)
    return {k: torch.from_numpy(v).to(dev) for k, v in arr.items()}


def _run(window_slots, seed, quota=5):
    from orthoroute_gb300 import Lattice
    from orthoroute_gb300.device import DeviceGraph, DeviceState, Ops, PathStore, route_pass
    lat = Lattice(60, 50, 6)
    g = DeviceGraph(lat)
    s = DeviceState(g)
    ops = Ops(g, s)
    rng = np.random.default_rng(seed)
    costs = (0.4 + rng.random(g.E) * 0.05).astype(np.float32)
    costs[rng.random(g.E) < 0.35] = np.float32("inf")       # blocked arcs: some ROI searches fail
    s.total_cost.copy_(torch.from_numpy(costs))
    s.live_static.copy_(torch.from_numpy(costs))
    nets = []
    while len(nets) < 90:
        a, b = (int(v) for v in rng.integers(0, lat.nx * lat.ny, size=2))
        d = abs(a % lat.nx - b % lat.nx) + abs(a // lat.nx - b // lat.nx)
        if 4 <= d <= 30:
            nets.append((a, b))
    store = PathStore(g, len(nets), window_slots=window_slots)
    table = _table(lat, nets, g.device)
    out = []
    for it in range(3):
        order = np.roll(np.arange(len(nets), dtype=np.int32), 7 * it)
        status, st = route_pass(ops, store, table, order, fallback_quota=quota, max_roi_nodes=50_000,
                                owner_weight=25.0 * (it + 1), path_weight=25.0 * (it + 1), history_weight=5.0,
                                pres_fac=float(it + 1), live=True, windows=window_slots > 0)
        out.append((status.copy(), st.copy(), store.length.cpu().numpy().copy(), store.path.cpu().numpy().copy(),
                    store.arcs.cpu().numpy().copy()))
    state = {k: getattr(s, k).cpu().numpy().copy() for k in
             ("present", "total_cost", "path_node_use", "owner_count", "owner_xor")}
    return out, state


@pytest.mark.parametrize("seed,lanes,look,quota", [(3, 4, 8, 5), (11, 4, 8, 5), (3, 2, 16, 5), (11, 4, 0, 5),
                                                   (3, 4, 8, 1), (11, 4, 8, 0)])
def test_windows_match_sequential_pass(seed, lanes, look, quota):
    """look > 0: windows skip clashing nets and take later disjoint ones (failed
    out-of-order members are undone and retried in turn); 0: consecutive only.
    quota 0 / 1: the pass's fallbacks run out, after which a window's failed
    members are final and its later members commit instead of being undone."""
    from orthoroute_gb300.autotune import search_lanes, window_lookahead
    before, look0 = search_lanes(0), window_lookahead()
    try:
        search_lanes(lanes)
        window_lookahead(look)
        seq, seq_state = _run(0, seed, quota)
        win, win_state = _run(16, seed, quota)
    finally:
        search_lanes(before)
        window_lookahead(look0)
    failed = 0
    spent = False      # a pass whose fallbacks ran out while searches still failed
    for (s0, st0, l0, p0, a0), (s1, st1, l1, p1, a1) in zip(seq, win):
        spent |= np.count_nonzero(s0 & 2) >= quota and np.count_nonzero((s0 & 3) == 1) > 0
        np.testing.assert_array_equal(s0, s1)
        np.testing.assert_array_equal(st0, st1)
        np.testing.assert_array_equal(l0, l1)
        for n in range(len(l0)):
            np.testing.assert_array_equal(p0[n, :l0[n]], p1[n, :l1[n]])
            if l0[n] >= 2:
                np.testing.assert_array_equal(a0[n, :2 * (l0[n] - 1)], a1[n, :2 * (l1[n] - 1)])
        failed += int(np.count_nonzero(s0 & 3))
    for k in seq_state:
        np.testing.assert_array_equal(seq_state[k], win_state[k], err_msg=k)
    assert failed > 0, "the case should exercise failed searches and fallbacks"
    if quota < 5:
        assert spent, "the case should exhaust the pass's fallbacks"
