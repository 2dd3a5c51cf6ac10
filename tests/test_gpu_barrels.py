"""Exact barrel conflicts and shared path nodes on the device
(ogr_barrel_scan) against the host formulation over the flat view of the
paths and against the oracle's detect_barrel_conflicts
(oracle/tallies.py, the restatement of _detect_barrel_conflicts
unified_pathfinder.py:10778-11111): the conflict count, the victim / owner /
conflict net sets, the exact and shared-node pairs, the scores and the nodes
whose conflict history grows."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def congested_router(nx, ny, nz, n_nets, iters, seed, trivial=0):
    from orthoroute_gb300 import Lattice
    from orthoroute_gb300.router import PathFinderConfig, PathFinderRouter
    rng = np.random.default_rng(seed)
    reqs = []
    while len(reqs) < n_nets:
        x0, x1 = rng.integers(2, nx - 2, size=2)
        y0, y1 = rng.integers(2, ny - 2, size=2)
        if abs(int(x1) - int(x0)) + abs(int(y1) - int(y0)) >= 4:
            reqs.append((f"N{len(reqs)}", int(y0) * nx + int(x0), int(y1) * nx + int(x1)))
    for j in range(trivial):          # one-node nets: they count in path-node use
        reqs.append((f"T{j}", reqs[j][1], reqs[j][1]))
    R = PathFinderRouter(PathFinderConfig(max_iterations=iters), mode="persistent", full_engine="grid")
    R.initialize_lattice(Lattice(nx, ny, nz))
    R.route_multiple_nets(reqs)
    return R


def snapshot(R, hist):
    return dict(conflicts=set(R.barrel_conflict_nets), owners=set(R.barrel_owner_nets),
                victims=set(R.barrel_victim_nets), scores={k: v for k, v in R.physical_scores.items() if v},
                exact_pairs=set(R.exact_pairs), pn_pairs=set(R.path_node_pairs),
                pn_scores=dict(R.path_node_scores), hist=[sorted(h) for h in hist])


@pytest.mark.parametrize("dims,n_nets,iters,seed,trivial",
                         [((40, 30, 6), 160, 1, 1, 0), ((36, 28, 4), 140, 2, 2, 6), ((50, 40, 8), 220, 1, 3, 3)])
def test_device_barrel_scan_matches_host_and_oracle(dims, n_nets, iters, seed, trivial):
    from oracle.tallies import NodeState, detect_barrel_conflicts, path_to_edges
    R = congested_router(*dims, n_nets, iters, seed, trivial)
    hist = []
    R._accumulate_history = lambda nodes: hist.append(np.asarray(nodes, dtype=np.int64).tolist())
    n_dev = R._detect_barrels()
    dev = snapshot(R, hist)
    assert n_dev > 0 and dev["exact_pairs"], "the job must have barrel conflicts for the check to bite"
    # the host formulation over the flat view of all paths
    store, R.store = R.store, None
    hist.clear()
    try:
        n_host = R._detect_barrels()
    finally:
        R.store = store
    assert n_host == n_dev
    assert snapshot(R, hist) == dev
    # the oracle's loop formulation
    nx, ny, nz = dims
    plane = nx * ny
    ip = R.g.indptr.cpu().numpy()
    ix = R.g.indices.cpu().numpy()
    src = R.g.edge_src.cpu().numpy()
    paths = {n: list(p) for n, p in R.net_paths.items() if p}
    ns = NodeState(R.N, nx, plane)
    ns.rebuild_owner([(R.net_id_map[n], p) for n, p in paths.items() if n in R.net_id_map])
    ns.rebuild_use(list(paths.values()))
    n2e = {n: path_to_edges(ip, ix, p) for n, p in paths.items() if len(p) >= 2}
    count, info = detect_barrel_conflicts(src, ix, ns, paths, n2e, dict(R.net_id_map), 1)
    assert count == n_dev
    assert info["conflict_nets"] == dev["conflicts"]
    assert info["owner_nets"] == dev["owners"] and info["victim_nets"] == dev["victims"]
    assert info["exact_pairs"] == dev["exact_pairs"] and info["path_node_pairs"] == dev["pn_pairs"]
    assert {k: v for k, v in info["scores"].items() if v} == dev["scores"]
    assert info["path_node_scores"] == dev["pn_scores"]
