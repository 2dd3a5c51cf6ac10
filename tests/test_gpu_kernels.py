"""GPU parity of every hot-path kernel against the CPU oracle (bit-exact).

All calls go through the C ABI (``orthoroute_gb300._lib``) on ``cuda:0``.
"""
import json
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from oracle import accounting as oacc
from oracle.dijkstra import find_path_roi, find_path_roi_c
from oracle.lattice import LatticeSpec, build_csr
from oracle.roi import extract_roi_bfs, roi_radius
from oracle.tallies import NodeState, path_to_edges

G = os.path.join(os.path.dirname(__file__), "golden")


def _dev():
    from orthoroute_gb300 import Lattice
    from orthoroute_gb300.device import DeviceGraph, DeviceState, Ops
    return Lattice, DeviceGraph, DeviceState, Ops


def make(nx, ny, nz, **kw):
    Lattice, DeviceGraph, DeviceState, Ops = _dev()
    L = Lattice(nx, ny, nz, **kw)
    g = DeviceGraph(L)
    s = DeviceState(g)
    ops = Ops(g, s)
    spec_kw = {k: v for k, v in kw.items() if k in ("allow_any_layer_via", "wrong_way_cost_multiplier",
                                                    "min_via_center_spacing", "via_cost")}
    ref = build_csr(LatticeSpec(nx, ny, nz, **spec_kw))
    return g, s, ops, ref


@pytest.mark.parametrize("dims,kw", [
    ((7, 5, 6), {}), ((30, 20, 8), {}), ((9, 8, 12), {"allow_any_layer_via": False}),
    ((12, 10, 20), {}), ((6, 5, 2), {}), ((11, 9, 6), {"wrong_way_cost_multiplier": 3.0}),
    ((10, 10, 6), {"min_via_center_spacing": 0.5}), ((10, 10, 6), {"min_via_center_spacing": 0.9}),
])
def test_csr_matches_oracle(dims, kw):
    g, s, ops, ref = make(*dims, **kw)
    np.testing.assert_array_equal(g.indptr.cpu().numpy(), ref.indptr)
    np.testing.assert_array_equal(g.indices.cpu().numpy(), ref.indices)
    np.testing.assert_array_equal(g.base_costs.cpu().numpy(), ref.base_costs)
    np.testing.assert_array_equal(g.edge_layer.cpu().numpy(), ref.edge_layer)
    np.testing.assert_array_equal(g.edge_kind.cpu().numpy(), ref.edge_kind)
    np.testing.assert_array_equal(g.edge_src.cpu().numpy(), ref.edge_src())
    rev = g.rev.cpu().numpy()
    np.testing.assert_array_equal(ref.indices[rev], ref.edge_src())
    np.testing.assert_array_equal(rev[rev], np.arange(len(rev)))


def test_csr_large_hash():
    """600x400x12 (config-1 lattice, 31.19M arcs): compare against the oracle."""
    g, s, ops, ref = make(600, 400, 12)
    assert g.E == len(ref.indices)
    for a, b in [(g.indptr, ref.indptr), (g.indices, ref.indices), (g.base_costs, ref.base_costs)]:
        np.testing.assert_array_equal(a.cpu().numpy(), b)


def _rand_state(s, E, nz, rng):
    present = rng.integers(0, 4, size=E).astype(np.float32)
    ema = (rng.random(E) * 3).astype(np.float32)
    hist = (rng.random(E) * 0.5).astype(np.float32)
    bias = (1.0 + rng.random(nz) * 0.6).astype(np.float32)
    s.present.copy_(torch.from_numpy(present))
    s.present_ema.copy_(torch.from_numpy(ema))
    s.history.copy_(torch.from_numpy(hist))
    return present, ema, hist, bias


@pytest.mark.parametrize("params", [(1.0, 12.0, 1.0, 0.3, True), (3.7, 9.6, 1.5, 0.3, True),
                                    (57.3, 14.4, 0.5, 0.01, False), (1234.5, 8.0, 1.0, 0.3, True)])
def test_costs_live_history_match_oracle(params):
    pres_fac, hw, vmult, bw, use_bias = params
    g, s, ops, ref = make(40, 30, 8)
    rng = np.random.default_rng(int(pres_fac * 10))
    E = g.E
    present, ema, hist, bias = _rand_state(s, E, 8, rng)
    A = oacc.Accountant(E)
    A.present[:] = present
    A.present_ema[:] = ema
    A.history[:] = hist
    kw = dict(edge_layer=ref.edge_layer, layer_bias_per_layer=bias, edge_kind=ref.edge_kind) if use_bias else {}
    A.update_costs(ref.base_costs, pres_fac, hw, via_cost_multiplier=vmult, base_cost_weight=bw, **kw)
    ops.update_costs(pres_fac, hw, vmult, bw, bias if use_bias else None)
    np.testing.assert_array_equal(s.total_cost.cpu().numpy(), A.total_cost)
    A.begin_live_present_costs()
    ops.live_begin(pres_fac)
    np.testing.assert_array_equal(s.total_cost.cpu().numpy(), A.total_cost)
    np.testing.assert_array_equal(s.live_static.cpu().numpy(), A._live_static_cost)
    # a committed path refreshes its arcs exactly like commit_path + refresh_live_present_costs
    path = [ref.plane + 3 * 40 + 5, ref.plane + 3 * 40 + 6, ref.plane + 3 * 40 + 7,
            2 * ref.plane + 3 * 40 + 7, 2 * ref.plane + 4 * 40 + 7]   # H layer 1, via, V layer 2
    arcs = ops.apply_path(path, net_id=3, sign=1, pres_fac=pres_fac)
    want = path_to_edges(ref.indptr, ref.indices, path)
    assert arcs == want
    A.commit_path(want)
    A.refresh_live_present_costs(want)
    np.testing.assert_array_equal(s.present.cpu().numpy(), A.present)
    np.testing.assert_array_equal(s.total_cost.cpu().numpy(), A.total_cost)
    ops.apply_path(path, net_id=3, sign=-1, pres_fac=pres_fac)
    A.clear_path(want)
    A.refresh_live_present_costs(want)
    np.testing.assert_array_equal(s.present.cpu().numpy(), A.present)
    np.testing.assert_array_equal(s.total_cost.cpu().numpy(), A.total_cost)
    for gain, decay in [(0.2, 1.0), (1.2, 0.98)]:
        A.update_history(gain, base_costs=ref.base_costs, history_cap_multiplier=15.0, decay_factor=decay,
                         use_raw_present=True)
        ops.update_history(gain, cap_mult=15.0, decay=decay)
        np.testing.assert_array_equal(s.history.cpu().numpy(), A.history)
    A.update_present_ema(0.40)
    ops.present_ema(0.40)
    np.testing.assert_array_equal(s.present_ema.cpu().numpy(), A.present_ema)


def test_tally_matches_oracle():
    g, s, ops, ref = make(50, 40, 8)
    rng = np.random.default_rng(3)
    present, ema, hist, bias = _rand_state(s, g.E, 8, rng)
    # EMA values as the loop produces them: 0.4*present + 0.6*ema chains of integers
    e = np.zeros(g.E, dtype=np.float32)
    for _ in range(4):
        p = rng.integers(0, 3, size=g.E).astype(np.float32)
        e = np.float32(0.4) * p + np.float32(0.6) * e
    s.present_ema.copy_(torch.from_numpy(e))
    use = rng.integers(0, 3, size=g.N).astype(np.int32)
    s.path_node_use.copy_(torch.from_numpy(use))
    mask = ref.edge_src() < ref.indices
    A = oacc.Accountant(g.E)
    A.present[:] = present
    over_sum, over_cnt, nsum, ncnt, units = ops.tally()
    assert (over_sum, over_cnt) == A.compute_edge_overuse(mask)
    ov = np.maximum(np.asarray(use, dtype=np.int64) - 1, 0)
    assert (nsum, ncnt) == (int(ov.sum()), int(np.count_nonzero(ov)))
    per_layer = np.bincount(ref.edge_layer, weights=np.maximum(0, e - np.float32(1.0)), minlength=8)
    per_layer = per_layer + ov.reshape(8, -1).sum(axis=1)
    np.testing.assert_array_equal(units.astype(np.float64) / 2.0 ** 23, per_layer)


@pytest.fixture(scope="module")
def roi_graph():
    meta = json.load(open(os.path.join(G, "golden.json")))
    nx, ny, nz = meta["roi_lattice"]
    return make(nx, ny, nz), meta


def test_roi_matches_reference_fixture(roi_graph):
    (g, s, ops, ref), meta = roi_graph
    z = np.load(os.path.join(G, "roi.npz"))
    for i, (src, dst, bonus, maxn) in enumerate(meta["roi_cases"]):
        r = roi_radius(src, dst, ref.nx, ref.plane, bonus)
        depth = min(int(r + bonus * 2.0), 80)
        halo = min(16, 2 + int(max(0.0, bonus) / 0.6))
        net = ops.net_args(0, src, dst, max_depth=depth, halo=halo, max_roi_nodes=maxn)
        np.testing.assert_array_equal(ops.extract_roi(net), z[f"roi{i}"], err_msg=f"case {i}")


@pytest.mark.parametrize("seed", range(6))
def test_roi_matches_oracle_random(seed):
    g, s, ops, ref = make(70, 60, 8)
    rng = np.random.default_rng(100 + seed)
    for _ in range(6):
        src, dst = (int(v) for v in rng.integers(0, ref.num_nodes, size=2))
        bonus = float(rng.choice([0.0, 0.6, 1.8, 6.0]))
        maxn = int(rng.choice([50_000, 5_000, 800]))
        r = roi_radius(src, dst, ref.nx, ref.plane, bonus)
        roi, _ = extract_roi_bfs(ref.indptr, ref.indices, ref.num_nodes, src, dst, initial_radius=r,
                                 stagnation_bonus=bonus, max_nodes=maxn)
        net = ops.net_args(0, src, dst, max_depth=min(int(r + bonus * 2.0), 80),
                           halo=min(16, 2 + int(max(0.0, bonus) / 0.6)), max_roi_nodes=maxn)
        np.testing.assert_array_equal(ops.extract_roi(net), roi)


def _penalty_state(s, N, rng, net_id):
    cnt = rng.choice([0, 0, 0, 1, 2], size=N).astype(np.int32)
    xr = np.where(cnt == 1, rng.choice([net_id, net_id + 1, net_id + 7], size=N), 0).astype(np.int32)
    use = rng.choice([0, 0, 1, 2], size=N).astype(np.int32)
    hist = (rng.integers(0, 3, size=N) * rng.random(N)).astype(np.float32)
    s.owner_count.copy_(torch.from_numpy(cnt))
    s.owner_xor.copy_(torch.from_numpy(xr))
    s.path_node_use.copy_(torch.from_numpy(use))
    s.node_history.copy_(torch.from_numpy(hist))
    ns = NodeState(N, 1, 1)
    ns.owner[:] = np.where(cnt == 0, -1, np.where(cnt == 1, xr, -2))
    ns.path_node_use[:] = use
    ns.node_history[:] = hist
    return ns


@pytest.mark.parametrize("seed", range(8))
def test_find_path_matches_oracle(seed):
    g, s, ops, ref = make(48, 40, 6)
    rng = np.random.default_rng(seed)
    E, N = g.E, g.N
    kind = seed % 4
    if kind == 0:
        costs = (0.12 + rng.random(E) * 0.05).astype(np.float32)
    elif kind == 1:   # heavy ties
        costs = (0.12 + rng.integers(0, 3, size=E) * 0.01).astype(np.float32)
    elif kind == 2:   # blocked arcs
        costs = (0.12 + rng.random(E) * 0.02).astype(np.float32)
        costs[rng.choice(E, size=E // 10, replace=False)] = np.float32("inf")
    else:             # realistic: base*bw + jitter
        costs = (np.float32(0.12) + oacc.jitter(E)).astype(np.float32)
    s.total_cost.copy_(torch.from_numpy(costs))
    net_id = 5
    ns = _penalty_state(s, N, rng, net_id) if seed % 2 == 0 else None
    pres_fac = float(rng.choice([1.0, 2.3, 40.0]))
    for _ in range(5):
        src, dst = (int(v) for v in rng.integers(0, ref.plane, size=2))
        r = roi_radius(src, dst, ref.nx, ref.plane)
        roi, g2r = extract_roi_bfs(ref.indptr, ref.indices, N, src, dst, initial_radius=r)
        pen = ns.owner_penalty(roi, net_id, pres_fac) if ns is not None else None
        st = {}
        want = find_path_roi(ref.indptr, ref.indices, src, dst, costs, roi, g2r, node_penalty=pen, stats=st)
        net = ops.net_args(net_id, src, dst, max_depth=min(r, 80), halo=2, pres_fac=pres_fac,
                           penalty=ns is not None)
        ops.stats.zero_()
        got = ops.find_path(net)
        assert got == want, (seed, src, dst)
        if want is not None:
            arcs, pops, roi_n, _ = ops.stats.cpu().tolist()
            assert (arcs, pops, roi_n) == (st["scanned"], st["settled"], len(roi)), (seed, src, dst)


@pytest.mark.parametrize("engine", ["grid", "cta"])
def test_find_path_full_graph_matches_oracle(engine):
    g, s, ops, ref = make(60, 30, 6)
    rng = np.random.default_rng(9)
    costs = (np.float32(0.12) + oacc.jitter(g.E)).astype(np.float32)
    s.total_cost.copy_(torch.from_numpy(costs))
    N = g.N
    ident = np.arange(N, dtype=np.int32)
    for _ in range(3):
        src, dst = (int(v) for v in rng.integers(0, ref.plane, size=2))
        want = find_path_roi(ref.indptr, ref.indices, src, dst, costs, ident, ident)
        got = ops.find_path(ops.net_args(0, src, dst, full_graph=True, penalty=False), engine=engine)
        assert got == want


def _costs(kind, E, rng):
    if kind == 0:
        return (0.12 + rng.random(E) * 0.05).astype(np.float32)
    if kind == 1:   # heavy ties
        return (0.12 + rng.integers(0, 3, size=E) * 0.01).astype(np.float32)
    if kind == 2:   # blocked arcs
        c = (0.12 + rng.random(E) * 0.02).astype(np.float32)
        c[rng.choice(E, size=E // 10, replace=False)] = np.float32("inf")
        return c
    return (np.float32(0.12) + oacc.jitter(E)).astype(np.float32)   # base + jitter


@pytest.mark.parametrize("seed", range(8))
def test_full_grid_search_matches_oracle(seed):
    """Whole-lattice search on all SMs: paths and heap statistics vs the oracle."""
    dims = [(80, 60, 8), (120, 40, 6), (64, 64, 12), (200, 150, 4)][seed % 4]
    g, s, ops, ref = make(*dims)
    rng = np.random.default_rng(100 + seed)
    costs = _costs(seed % 4, g.E, rng)
    s.total_cost.copy_(torch.from_numpy(costs))
    N = g.N
    ident = np.arange(N, dtype=np.int32)
    net_id = 3
    ns = _penalty_state(s, N, rng, net_id) if seed % 2 == 0 else None
    pres_fac = float(rng.choice([1.0, 2.3, 40.0]))
    pen = ns.owner_penalty(ident, net_id, pres_fac) if ns is not None else None
    for _ in range(3):
        src, dst = (int(v) for v in rng.integers(0, ref.plane, size=2))
        st = {}
        want = find_path_roi_c(ref.indptr, ref.indices, src, dst, costs, ident, ident, node_penalty=pen, stats=st)
        ops.stats.zero_()
        got = ops.find_path(ops.net_args(net_id, src, dst, full_graph=True, pres_fac=pres_fac,
                                         penalty=ns is not None), engine="grid")
        assert got == want, (seed, src, dst)
        if want is not None:
            arcs, pops, roi_n, phases = ops.stats.cpu().tolist()
            assert (arcs, pops, roi_n) == (st["scanned"], st["settled"], N)
            assert phases >= 1


def test_full_grid_search_large_lattice():
    """A 300x200x8 lattice (480k nodes): frontiers spread over every CTA."""
    g, s, ops, ref = make(300, 200, 8)
    rng = np.random.default_rng(77)
    costs = _costs(3, g.E, rng)
    s.total_cost.copy_(torch.from_numpy(costs))
    ident = np.arange(g.N, dtype=np.int32)
    for src, dst in [(5, ref.plane - 7), (int(rng.integers(0, ref.plane)), int(rng.integers(0, ref.plane)))]:
        st = {}
        want = find_path_roi_c(ref.indptr, ref.indices, src, dst, costs, ident, ident, stats=st)
        ops.stats.zero_()
        got = ops.find_path(ops.net_args(0, src, dst, full_graph=True, penalty=False), engine="grid")
        assert got == want
        assert ops.stats.cpu().tolist()[:2] == [st["scanned"], st["settled"]]


def test_full_grid_search_unreachable_and_trivial():
    g, s, ops, ref = make(40, 30, 4)
    costs = np.full(g.E, np.float32("inf"), dtype=np.float32)
    s.total_cost.copy_(torch.from_numpy(costs))
    assert ops.find_path(ops.net_args(0, 3, 100, full_graph=True, penalty=False), engine="grid") is None
    s.total_cost.fill_(0.4)
    assert ops.find_path(ops.net_args(0, 3, 3, full_graph=True, penalty=False), engine="grid") is None


def _walled_searches(g, s, ops, ref, engine, rng, n=3):
    """Searches whose dst has every in-arc blocked: the heap pops every node
    it reaches and scans each one's row before it runs empty, and the GPU's
    counts must be those."""
    N = g.N
    base = _costs(3, g.E, rng)
    for _ in range(n):
        src, dst = (int(v) for v in rng.integers(0, ref.plane, size=2))
        if src == dst:
            continue
        costs = base.copy()
        costs[ref.indices == dst] = np.float32("inf")
        s.total_cost.copy_(torch.from_numpy(costs))
        ops.stats.zero_()
        if engine == "roi":
            r = roi_radius(src, dst, ref.nx, ref.plane)
            roi, g2r = extract_roi_bfs(ref.indptr, ref.indices, N, src, dst, initial_radius=r)
            got = ops.find_path(ops.net_args(0, src, dst, max_depth=min(r, 80), halo=2, penalty=False))
        else:
            roi = g2r = np.arange(N, dtype=np.int32)
            got = ops.find_path(ops.net_args(0, src, dst, full_graph=True, penalty=False), engine=engine)
        st = {}
        want = find_path_roi_c(ref.indptr, ref.indices, src, dst, costs, roi, g2r, stats=st)
        assert want is None and got is None, (src, dst)
        arcs, pops = ops.stats.cpu().tolist()[:2]
        assert st["settled"] > 100
        assert (arcs, pops) == (st["scanned"], st["settled"]), (engine, src, dst)


@pytest.mark.parametrize("engine", ["roi", "grid", "cta"])
def test_failed_search_statistics_match_oracle(engine):
    g, s, ops, ref = make(60, 40, 6)
    _walled_searches(g, s, ops, ref, engine, np.random.default_rng(31))


def test_find_path_replays_reference_net_trace():
    """Every recorded find_path_roi call of a real reference routing run."""
    meta = json.load(open(os.path.join(G, "golden.json")))["r0"]
    g, s, ops, ref = make(meta["nx"], meta["ny"], meta["nz"])
    z = np.load(os.path.join(G, "runs.npz"))
    for j in range(meta["n_trace"]):
        src, dst = z[f"r0_t{j}_sd"].tolist()
        roi = z[f"r0_t{j}_roi"]
        s.total_cost.copy_(torch.from_numpy(z[f"r0_t{j}_costs"]))
        hist = np.zeros(g.N, dtype=np.float32)
        pen = z[f"r0_t{j}_pen"] if f"r0_t{j}_pen" in z else None
        if pen is not None:
            hist[roi] = pen   # inject the ROI-local penalty as node history x 1.0
        s.node_history.copy_(torch.from_numpy(hist))
        s.owner_count.zero_()
        s.path_node_use.zero_()
        r = roi_radius(src, dst, ref.nx, ref.plane)
        net = ops.net_args(0, src, dst, max_depth=min(r, 80), halo=2, pres_fac=0.0, hist_pen=1.0,
                           penalty=pen is not None)
        np.testing.assert_array_equal(ops.extract_roi(net), roi)
        got = ops.find_path(net)
        np.testing.assert_array_equal(np.asarray(got or [], dtype=np.int32), z[f"r0_t{j}_path"])


def test_solver_seam_replays_reference_net_trace():
    """ogr_find_path_roi with the reference's own ROI, costs and penalty arrays."""
    meta = json.load(open(os.path.join(G, "golden.json")))["r0"]
    g, s, ops, ref = make(meta["nx"], meta["ny"], meta["nz"])
    z = np.load(os.path.join(G, "runs.npz"))
    for j in range(meta["n_trace"]):
        src, dst = z[f"r0_t{j}_sd"].tolist()
        costs = torch.from_numpy(z[f"r0_t{j}_costs"]).to(g.device)
        pen = z[f"r0_t{j}_pen"] if f"r0_t{j}_pen" in z else None
        ops.stats.zero_()
        got = ops.find_path_given_roi(src, dst, costs, z[f"r0_t{j}_roi"], pen)
        np.testing.assert_array_equal(np.asarray(got or [], dtype=np.int32), z[f"r0_t{j}_path"])


@pytest.mark.parametrize("seed", range(3))
def test_solver_seam_matches_oracle(seed):
    g, s, ops, ref = make(48, 40, 6)
    rng = np.random.default_rng(50 + seed)
    costs = _costs(seed % 4, g.E, rng)
    d_costs = torch.from_numpy(costs).to(g.device)
    for _ in range(4):
        src, dst = (int(v) for v in rng.integers(0, ref.plane, size=2))
        r = roi_radius(src, dst, ref.nx, ref.plane)
        roi, g2r = extract_roi_bfs(ref.indptr, ref.indices, g.N, src, dst, initial_radius=r)
        pen = (rng.integers(0, 3, size=len(roi)) * rng.random(len(roi))).astype(np.float32)
        st = {}
        want = find_path_roi(ref.indptr, ref.indices, src, dst, costs, roi, g2r, node_penalty=pen, stats=st)
        ops.stats.zero_()
        got = ops.find_path_given_roi(src, dst, d_costs, roi, pen)
        assert got == want
        if want is not None:
            assert ops.stats.cpu().tolist()[:3] == [st["scanned"], st["settled"], len(roi)]


def test_apply_path_node_state_matches_oracle():
    g, s, ops, ref = make(20, 16, 8)
    ns = NodeState(g.N, ref.nx, ref.plane)
    paths = {
        1: [ref.plane + 5, 3 * ref.plane + 5, 5 * ref.plane + 5, 5 * ref.plane + 6],
        2: [2 * ref.plane + 5, 3 * ref.plane + 5, 4 * ref.plane + 5],
        3: [ref.plane + 40, 6 * ref.plane + 40, 2 * ref.plane + 40, 2 * ref.plane + 60],
    }
    # path 3 revisits column 40 on overlapping z ranges; ownership dedups nodes
    for nid, p in paths.items():
        ops.apply_path(p, nid, +1, 1.0, live=False)
        ns.mark_owner(nid, p)
        ns.mark_use(p)
    owner = lambda: np.where(s.owner_count.cpu().numpy() == 0, -1,
                             np.where(s.owner_count.cpu().numpy() == 1, s.owner_xor.cpu().numpy(), -2))
    np.testing.assert_array_equal(owner(), ns.owner)
    np.testing.assert_array_equal(s.path_node_use.cpu().numpy(), ns.path_node_use.astype(np.int32))
    ops.apply_path(paths[2], 2, -1, 1.0, live=False)
    ns.clear_owner(2, paths[2])
    ns.clear_use(paths[2])
    np.testing.assert_array_equal(owner(), ns.owner)
    np.testing.assert_array_equal(s.path_node_use.cpu().numpy(), ns.path_node_use.astype(np.int32))


@pytest.mark.parametrize("quarter", [1, 2, 3])
def test_full_grid_search_any_grid_size(quarter):
    """The autotuner's grid sizes: the same paths and statistics on 1/4 .. 3/4 of the CTAs."""
    from orthoroute_gb300.autotune import full_grid
    g, s, ops, ref = make(120, 90, 8)
    rng = np.random.default_rng(500 + quarter)
    costs = _costs(quarter, g.E, rng)
    s.total_cost.copy_(torch.from_numpy(costs))
    ident = np.arange(g.N, dtype=np.int32)
    cur, lim = full_grid(0)
    try:
        full_grid(max(1, lim * quarter // 4))
        for _ in range(3):
            src, dst = (int(v) for v in rng.integers(0, ref.plane, size=2))
            st = {}
            want = find_path_roi_c(ref.indptr, ref.indices, src, dst, costs, ident, ident, stats=st)
            ops.stats.zero_()
            got = ops.find_path(ops.net_args(0, src, dst, full_graph=True, penalty=False), engine="grid")
            assert got == want
            if want is not None:
                assert ops.stats.cpu().tolist()[:2] == [st["scanned"], st["settled"]]
    finally:
        full_grid(cur)


def test_autotune_times_every_candidate(tmp_path, monkeypatch):
    from orthoroute_gb300 import Lattice, autotune
    monkeypatch.setenv("ORTHOROUTE_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    g, s, ops, ref = make(200, 60, 6)
    s.total_cost.copy_(torch.from_numpy(_costs(3, g.E, np.random.default_rng(1))))
    cur, lim = autotune.full_grid(0)
    lat = Lattice(200, 60, 6)
    nets = [(2, 60 * 200 - 3), (200 * 30 + 1, 200 * 31 - 2)]
    try:
        t = autotune.tune(ops, lat, nets)
        assert not t.cached and t.samples == 2
        # the tile engine's window widths are timed when the grid engine wins
        tile = {f"tile_delta{h}" for h in autotune.TILE_DELTA_HOPS} if t.full_engine == "grid" else set()
        assert set(t.ms_per_search) == ({f"grid{c}" for _, c in autotune.candidates(lim)[:-1]} | {"cta"} |
                                        {f"full_lanes{k}_reuse{r}" for k in autotune.FULL_LANES for r in (0, 1)} |
                                        tile)
        assert autotune.full_lanes(0) == t.full_lanes and autotune.full_reuse() == t.full_reuse
        assert t.full_engine in ("grid", "cta")
        if t.full_engine == "grid":
            assert autotune.full_grid(0)[0] == t.full_ctas
        assert autotune.full_tile(-1) == ((1, t.full_tile_delta) if t.full_tile_delta > 0 else (0, autotune.full_tile(-1)[1]))
        t2 = autotune.tune(ops, lat, nets)
        assert t2.cached and (t2.full_engine, t2.full_ctas, t2.full_tile_delta) == \
            (t.full_engine, t.full_ctas, t.full_tile_delta)
    finally:
        autotune.full_tile(0)
        autotune.full_grid(cur)
        autotune.full_lanes(16)
        autotune.full_reuse(0)


@pytest.mark.parametrize("lanes", [2, 8, 16])
def test_find_path_any_lanes_per_node(lanes):
    """The autotuner's lane widths of the ROI search: the same paths and heap
    statistics as the oracle at 2, 8 and 16 lanes per node (4 is the default)."""
    from orthoroute_gb300.autotune import search_lanes
    g, s, ops, ref = make(48, 40, 6)
    rng = np.random.default_rng(70 + lanes)
    E, N = g.E, g.N
    costs = (0.12 + rng.integers(0, 3, size=E) * 0.01).astype(np.float32)   # ties
    costs[rng.choice(E, size=E // 20, replace=False)] = np.float32("inf")
    s.total_cost.copy_(torch.from_numpy(costs))
    net_id = 5
    ns = _penalty_state(s, N, rng, net_id)
    before = search_lanes(0)
    try:
        search_lanes(lanes)
        for _ in range(5):
            src, dst = (int(v) for v in rng.integers(0, ref.plane, size=2))
            r = roi_radius(src, dst, ref.nx, ref.plane)
            roi, g2r = extract_roi_bfs(ref.indptr, ref.indices, N, src, dst, initial_radius=r)
            pen = ns.owner_penalty(roi, net_id, 2.3)
            st = {}
            want = find_path_roi(ref.indptr, ref.indices, src, dst, costs, roi, g2r, node_penalty=pen, stats=st)
            ops.stats.zero_()
            got = ops.find_path(ops.net_args(net_id, src, dst, max_depth=min(r, 80), halo=2, pres_fac=2.3))
            assert got == want, (lanes, src, dst)
            if want is not None:
                assert ops.stats.cpu().tolist()[:2] == [st["scanned"], st["settled"]]
    finally:
        search_lanes(before)


def test_autotune_picks_roi_lanes(tmp_path, monkeypatch):
    from orthoroute_gb300 import Lattice, autotune
    monkeypatch.setenv("ORTHOROUTE_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    g, s, ops, ref = make(60, 50, 6)
    s.total_cost.copy_(torch.from_numpy(_costs(3, g.E, np.random.default_rng(2))))
    before = autotune.search_lanes(0)
    try:
        roi_nets = [(3 + 61 * k, 3 + 61 * k + 20) for k in range(6)]
        t = autotune.tune(ops, Lattice(60, 50, 6), [], roi_nets)
        assert {f"roi_lanes{k}" for k in autotune.LANES} <= set(t.ms_per_search)
        assert t.roi_lanes in autotune.LANES and autotune.search_lanes(0) == t.roi_lanes
    finally:
        autotune.search_lanes(before)


def test_commit_paths_equals_one_by_one():
    """The batched restore commit: the same present, path-node use, barrel
    ownership, arcs and path-store slots as committing the paths one at a time."""
    from orthoroute_gb300.device import PathStore
    rng = np.random.default_rng(12)
    nx, ny, nz = 30, 24, 8
    paths = []                   # simple random walks over the lattice's arcs
    g, s, ops, ref = make(nx, ny, nz)
    indptr, indices = ref.indptr, ref.indices
    for k in range(60):
        node = int(rng.integers(0, ref.num_nodes))
        p, seen = [node], {node}
        for _ in range(int(rng.integers(1, 40))):
            nb = [int(v) for v in indices[indptr[p[-1]]:indptr[p[-1] + 1]] if int(v) not in seen]
            if not nb:
                break
            p.append(nb[int(rng.integers(0, len(nb)))])
            seen.add(p[-1])
        if len(p) >= 2:
            paths.append(p)
    ids = [3 + k for k in range(len(paths))]
    # one by one
    one = [ops.apply_path(p, i, +1, 1.0, live=False) for p, i in zip(paths, ids)]
    want = {k: getattr(s, k).cpu().numpy().copy() for k in ("present", "path_node_use", "owner_count", "owner_xor")}
    for k in want:
        getattr(s, k).zero_()
    store = PathStore(g, len(paths) + 5)
    slots = [len(paths) + 4 - k for k in range(len(paths))]
    got_arcs = ops.commit_paths([np.asarray(p) for p in paths], ids, store, slots)
    for k, v in want.items():
        np.testing.assert_array_equal(getattr(s, k).cpu().numpy(), v, err_msg=k)
    for a, b in zip(got_arcs, one):
        assert a.tolist() == list(b)
    L = store.length.cpu().numpy()
    P = store.path.cpu().numpy()
    A = store.arcs.cpu().numpy()
    for p, sl, b in zip(paths, slots, one):
        assert L[sl] == len(p) and P[sl, :len(p)].tolist() == p
        # the slot's arcs too: the per-net overuse sums of a restored state read them
        assert A[sl, :2 * (len(p) - 1)].tolist() == list(b)


@pytest.mark.parametrize("lanes,reuse", [(4, 0), (8, 0), (4, 1), (16, 1)])
def test_full_grid_search_any_lanes(lanes, reuse):
    """The whole-lattice search with 4, 8 or 16 lanes per frontier node, with
    and without the reuse of clean pulls: the same paths and heap statistics
    as the oracle (16 lanes without reuse is the default)."""
    from orthoroute_gb300.autotune import full_lanes, full_reuse
    g, s, ops, ref = make(120, 90, 8)
    rng = np.random.default_rng(600 + lanes)
    costs = _costs(lanes % 4, g.E, rng)
    s.total_cost.copy_(torch.from_numpy(costs))
    ident = np.arange(g.N, dtype=np.int32)
    net_id = 2
    ns = _penalty_state(s, g.N, rng, net_id)
    pen = ns.owner_penalty(ident, net_id, 2.3)
    before = full_lanes(0)
    try:
        full_lanes(lanes)
        full_reuse(reuse)
        for _ in range(3):
            src, dst = (int(v) for v in rng.integers(0, ref.plane, size=2))
            st = {}
            want = find_path_roi_c(ref.indptr, ref.indices, src, dst, costs, ident, ident, node_penalty=pen, stats=st)
            ops.stats.zero_()
            got = ops.find_path(ops.net_args(net_id, src, dst, full_graph=True, pres_fac=2.3), engine="grid")
            assert got == want
            if want is not None:
                assert ops.stats.cpu().tolist()[:2] == [st["scanned"], st["settled"]]
    finally:
        full_lanes(before)
        full_reuse(0)
