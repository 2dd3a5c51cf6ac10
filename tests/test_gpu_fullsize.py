"""Invariants of a routing job on the full 600x400x12 lattice (2.88 M nodes,
21.1 M arcs) that do not depend on size: every path runs from its net's
source to its sink over lattice arcs; the device congestion state (present
per arc, path-node use, barrel ownership) equals the one recomputed from the
final paths; and the batched disjoint-ROI windows give the sequential pass's
paths and tallies."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _job(window_slots, n_nets=300, iters=2):
    import bench
    from orthoroute_gb300.router import PathFinderConfig, PathFinderRouter
    cfg = bench.CONFIGS["c1"]
    reqs = bench.make_requests(cfg)[:n_nets]
    R = PathFinderRouter(PathFinderConfig(max_iterations=iters), window_slots=window_slots)
    R.initialize_lattice(bench.make_lattice(cfg), bench.board_bounds(cfg["nx"], cfg["ny"]))
    res = R.route_multiple_nets(reqs)
    return R, reqs, res


def test_full_size_job_invariants():
    R, reqs, res = _job(32)
    N, E = R.N, R.E
    assert (N, E) == (2_880_000, 21_110_000)
    # paths: source to sink over lattice arcs
    src = R.g.edge_src.cpu().numpy().astype(np.int64)
    dst = R.g.indices.cpu().numpy().astype(np.int64)
    keys = np.sort(src * N + dst)
    routed = 0
    for name, s, d in reqs:
        p = R.net_paths.get(name)
        if not p:
            continue
        routed += 1
        assert p[0] == s and p[-1] == d, name
        a = np.asarray(p, dtype=np.int64)
        hop = a[:-1] * N + a[1:]
        pos = np.minimum(np.searchsorted(keys, hop), keys.size - 1)
        assert np.array_equal(keys[pos], hop), name
    assert routed >= len(reqs) // 2
    # present = arcs of every path, both directions
    arcs = np.concatenate([e for e in R.net_to_edges.values() if len(e)])
    want_present = np.bincount(arcs, minlength=E).astype(np.float32)
    np.testing.assert_array_equal(R.s.present.cpu().numpy(), want_present)
    # path-node use = distinct nets per node (host mirror and device)
    nodes = np.concatenate([np.unique(np.asarray(p, dtype=np.int64)) for p in R.net_paths.values() if len(p) >= 2])
    want_use = np.bincount(nodes, minlength=N)
    np.testing.assert_array_equal(R.s.path_node_use.cpu().numpy(), want_use.astype(np.int32))
    np.testing.assert_array_equal(R.node_use.astype(np.int64), want_use)
    # barrel ownership: -1 / net id / -2 from the device count + xor, against the paths' via nodes
    cnt = R.s.owner_count.cpu().numpy()
    xr = R.s.owner_xor.cpu().numpy()
    dev_owner = np.where(cnt == 0, -1, np.where(cnt == 1, xr, -2))
    np.testing.assert_array_equal(dev_owner, R._via_owner_of(R._flat()).astype(dev_owner.dtype))


def test_full_size_windows_match_sequential_pass():
    Rw, reqs, rw = _job(32)
    Rs, _, rs = _job(0)
    assert {k: list(v) for k, v in Rw.net_paths.items()} == {k: list(v) for k, v in Rs.net_paths.items()}
    for k in ("overuse_sum", "overuse_edges", "barrel_conflicts", "failed_nets"):
        assert rw.get(k) == rs.get(k), k
