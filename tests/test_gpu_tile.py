"""The tile-window engine of the whole-lattice search (tilesearch.cu): the
same paths and heap statistics as the oracle's heap search for every window
width and tile size, with penalties, ties and blocked arcs; nets it cannot
take exactly are handed to the phase engine and stay exact."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from oracle.dijkstra import find_path_roi_c

from test_gpu_kernels import _costs, _penalty_state, _walled_searches, make


def pstate(s, N, rng, net_id):
    """A penalty state whose node history (x5) stays on the engine's exact
    grid (0 or >= 2^-7), like the router's whole-unit history increments."""
    ns = _penalty_state(s, N, rng, net_id)
    hist = np.where(ns.node_history > 0, 0.5 + ns.node_history, 0).astype(np.float32)
    ns.node_history[:] = hist
    s.node_history.copy_(torch.from_numpy(hist))
    return ns


def tile_profile(reset=0):
    import ctypes as C
    from orthoroute_gb300 import _lib
    out = (C.c_int64 * 24)()
    _lib.check(_lib.load().ogr_tile_profile(out, int(reset)), "ogr_tile_profile")
    return list(out)


@pytest.fixture
def tile_engine():
    from orthoroute_gb300 import autotune

    def use(delta, tx=0, ty=0):
        autotune.full_tile(1, delta, tx, ty)
    yield use
    autotune.full_tile(0)


def run_cases(ops, ref, costs, rng, n, pen=None, ns=None, net_id=0, pres_fac=1.0):
    ident = np.arange(ref.num_nodes, dtype=np.int32)
    for _ in range(n):
        src, dst = (int(v) for v in rng.integers(0, ref.plane, size=2))
        st = {}
        want = find_path_roi_c(ref.indptr, ref.indices, src, dst, costs, ident, ident, node_penalty=pen, stats=st)
        ops.stats.zero_()
        got = ops.find_path(ops.net_args(net_id, src, dst, full_graph=True, pres_fac=pres_fac,
                                         penalty=ns is not None), engine="grid")
        assert got == want, (src, dst)
        if want is not None:
            arcs, pops, roi_n, rounds = ops.stats.cpu().tolist()
            assert (arcs, pops, roi_n) == (st["scanned"], st["settled"], ref.num_nodes)


@pytest.mark.parametrize("seed", range(8))
def test_tile_search_matches_oracle(seed, tile_engine):
    dims = [(80, 60, 8), (120, 40, 6), (64, 64, 12), (200, 150, 4)][seed % 4]
    g, s, ops, ref = make(*dims)
    rng = np.random.default_rng(900 + seed)
    costs = _costs(seed % 4, g.E, rng)
    s.total_cost.copy_(torch.from_numpy(costs))
    net_id = 3
    ns = pstate(s, g.N, rng, net_id) if seed % 2 == 0 else None
    pres_fac = float(rng.choice([1.0, 2.3, 40.0]))
    ident = np.arange(g.N, dtype=np.int32)
    pen = ns.owner_penalty(ident, net_id, pres_fac) if ns is not None else None
    tile_engine([1.0, 2.5, 8.0, 30.0][seed % 4])
    before = tile_profile()
    run_cases(ops, ref, costs, rng, 3, pen, ns, net_id, pres_fac)
    after = tile_profile()
    assert after[0] - before[0] >= 1                       # the tile engine ran
    assert after[4] - before[4] == 0                       # and kept every net


@pytest.mark.parametrize("tx,ty,delta", [(4, 4, 0.5), (7, 5, 1.5), (16, 3, 4.0), (1, 1, 0.8)])
def test_tile_search_any_tile_size(tx, ty, delta, tile_engine):
    g, s, ops, ref = make(90, 70, 6)
    rng = np.random.default_rng(tx * 100 + ty)
    costs = _costs(tx % 4, g.E, rng)
    s.total_cost.copy_(torch.from_numpy(costs))
    net_id = 5
    ns = pstate(s, g.N, rng, net_id)
    pen = ns.owner_penalty(np.arange(g.N, dtype=np.int32), net_id, 2.3)
    tile_engine(delta, tx, ty)
    run_cases(ops, ref, costs, rng, 3, pen, ns, net_id, 2.3)


def test_tile_search_large_lattice(tile_engine):
    """300x200x8 (480k nodes): corner to corner and random."""
    g, s, ops, ref = make(300, 200, 8)
    rng = np.random.default_rng(77)
    costs = _costs(3, g.E, rng)
    s.total_cost.copy_(torch.from_numpy(costs))
    ident = np.arange(g.N, dtype=np.int32)
    tile_engine(1.0)
    for src, dst in [(5, ref.plane - 7), (int(rng.integers(0, ref.plane)), int(rng.integers(0, ref.plane)))]:
        st = {}
        want = find_path_roi_c(ref.indptr, ref.indices, src, dst, costs, ident, ident, stats=st)
        ops.stats.zero_()
        got = ops.find_path(ops.net_args(0, src, dst, full_graph=True, penalty=False), engine="grid")
        assert got == want
        assert ops.stats.cpu().tolist()[:2] == [st["scanned"], st["settled"]]


@pytest.mark.parametrize("kw", [dict(wrong_way_cost_multiplier=3.0), dict(min_via_center_spacing=0.5),
                                dict(allow_any_layer_via=True)])
def test_tile_search_lattice_variants(kw, tile_engine):
    g, s, ops, ref = make(70, 50, 6, **kw)
    rng = np.random.default_rng(31)
    costs = _costs(0, g.E, rng)
    s.total_cost.copy_(torch.from_numpy(costs))
    tile_engine(1.2, 9, 9)
    run_cases(ops, ref, costs, rng, 3)


def test_tile_search_hands_over_small_costs(tile_engine):
    """Costs below 2^-7 are off the engine's exact int64 grid: the net goes to
    the phase engine, and the result is still the heap's."""
    g, s, ops, ref = make(60, 40, 6)
    rng = np.random.default_rng(4)
    costs = (0.002 + rng.random(g.E) * 0.004).astype(np.float32)
    s.total_cost.copy_(torch.from_numpy(costs))
    tile_engine(0.05)
    before = tile_profile()
    run_cases(ops, ref, costs, rng, 2)
    after = tile_profile()
    assert after[4] - before[4] == after[0] - before[0] >= 1


def test_tile_search_hands_over_tiny_penalties(tile_engine):
    """Node penalties of a few thousandths (history x5 below 2^-7) are handed
    over too, where a tile holds one; the results stay the heap's."""
    g, s, ops, ref = make(80, 60, 8)
    rng = np.random.default_rng(21)
    costs = _costs(0, g.E, rng)
    s.total_cost.copy_(torch.from_numpy(costs))
    ns = _penalty_state(s, g.N, rng, 2)
    pen = ns.owner_penalty(np.arange(g.N, dtype=np.int32), 2, 1.0)
    tile_engine(1.0)
    run_cases(ops, ref, costs, rng, 3, pen, ns, 2, 1.0)


def test_tile_search_unreachable_and_trivial(tile_engine):
    g, s, ops, ref = make(40, 30, 6)
    costs = np.full(g.E, np.float32("inf"), dtype=np.float32)
    s.total_cost.copy_(torch.from_numpy(costs))
    tile_engine(1.0)
    assert ops.find_path(ops.net_args(0, 3, 100, full_graph=True, penalty=False), engine="grid") is None
    assert ops.find_path(ops.net_args(0, 3, 3, full_graph=True, penalty=False), engine="grid") is None
    costs = np.full(g.E, np.float32(0.12), dtype=np.float32)
    s.total_cost.copy_(torch.from_numpy(costs))
    rng = np.random.default_rng(8)
    run_cases(ops, ref, costs, rng, 2)


def test_tile_search_failed_search_statistics(tile_engine):
    """A search that cannot reach dst counts every node it reaches, as the heap."""
    g, s, ops, ref = make(60, 40, 6)
    tile_engine(1.0)
    _walled_searches(g, s, ops, ref, "grid", np.random.default_rng(32))


def test_tile_search_many_in_a_row(tile_engine):
    """Consecutive searches reuse the node words through the search stamp
    (no clearing between searches); 40 searches in a row stay exact."""
    g, s, ops, ref = make(50, 40, 6)
    rng = np.random.default_rng(12)
    tile_engine(0.7)
    for k in range(8):
        costs = _costs(k % 4, g.E, rng)
        s.total_cost.copy_(torch.from_numpy(costs))
        run_cases(ops, ref, costs, rng, 5)
