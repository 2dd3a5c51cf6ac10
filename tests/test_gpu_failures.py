"""Failure handling without a GPU fault.

The whole-lattice search's waits are bounded: its grid barrier gives up after
a spin bound and its phase loop after a phase cap, each returning a status
word the host reads (the reference's counterpart is the persistent kernel's
queue-overflow flag, pathfinder/persistent_kernel.py:699-700, raised as a
RuntimeError).  These tests shrink the bounds with ogr_debug_limits so they
run out, and check that

* the failure surfaces as a Python exception naming the status;
* the routing pass stopped before committing the failed net, so the device
  congestion state (present per arc, path-node use) equals the one
  recomputed from the paths in the device path store;
* the context stays usable: with the limits restored the same job routes
  exactly like a fresh router.

Host-side failures are injected in the ctypes shim (_lib.inject_fault).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def nets(nx, ny, n, seed):
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        x0, x1 = rng.integers(0, nx, size=2)
        y0, y1 = rng.integers(0, ny, size=2)
        d = abs(int(x1) - int(x0)) + abs(int(y1) - int(y0))
        if 5 <= d <= 160:
            out.append((f"N{len(out)}", int(y0) * nx + int(x0), int(y1) * nx + int(x1)))
    return out


def router(mode="persistent"):
    from orthoroute_gb300 import Lattice
    from orthoroute_gb300.router import PathFinderConfig, PathFinderRouter
    R = PathFinderRouter(PathFinderConfig(max_iterations=3), mode=mode, full_engine="grid")
    R.initialize_lattice(Lattice(140, 40, 6))
    return R


REQS = nets(140, 40, 40, 5)


def stored_paths(R):
    L = R.store.length.cpu().numpy()
    P = R.store.path.cpu().numpy()
    return [P[k, :L[k]].astype(np.int64) for k in range(len(L)) if L[k] >= 2]


def assert_state_matches_store(R):
    """present = both arcs of every hop of every stored path; path-node use =
    distinct stored paths per node."""
    N, E = R.N, R.E
    src = R.g.edge_src.cpu().numpy().astype(np.int64)
    dst = R.g.indices.cpu().numpy().astype(np.int64)
    key = src * N + dst
    order = np.argsort(key)
    paths = stored_paths(R)
    want = np.zeros(E, dtype=np.int64)
    use = np.zeros(N, dtype=np.int64)
    for p in paths:
        for a, b in ((p[:-1], p[1:]), (p[1:], p[:-1])):
            k = a * N + b
            pos = np.searchsorted(key[order], k)
            assert np.array_equal(key[order][pos], k)
            np.add.at(want, order[pos], 1)
        use[np.unique(p)] += 1
    np.testing.assert_array_equal(R.s.present.cpu().numpy().astype(np.int64), want)
    np.testing.assert_array_equal(R.s.path_node_use.cpu().numpy().astype(np.int64), use)
    return len(paths)


def reference_paths():
    R = router()
    return {k: list(v) for k, v in R.route_multiple_nets(REQS)["paths"].items()}


@pytest.mark.parametrize("limit,status", [((1, 0), "grid barrier timed out"),
                                          ((0, 3), "iteration limit reached")])
def test_bounded_wait_runs_out_and_state_stays_consistent(limit, status):
    from orthoroute_gb300 import _lib
    want = reference_paths()
    assert any(abs(s % 140 - d % 140) + abs(s // 140 - d // 140) >= 125 for _, s, d in REQS)
    R = router()
    try:
        _lib.debug_limits(*limit)
        with pytest.raises(RuntimeError, match=status):
            R.route_multiple_nets(REQS)
    finally:
        _lib.debug_limits(0, 0)
    assert_state_matches_store(R)
    # the context is usable and a new job routes exactly like a fresh router
    assert {k: list(v) for k, v in R.route_multiple_nets(REQS)["paths"].items()} == want


def test_injected_pass_failure_raises_and_leaves_state_unchanged():
    from orthoroute_gb300 import _lib
    want = reference_paths()
    R = router()
    with _lib.inject_fault("ogr_route_pass", _lib.OGR_ERR_CUDA):
        with pytest.raises(RuntimeError, match="CUDA"):
            R.route_multiple_nets(REQS)
    assert R.s.present.abs().sum().item() == 0
    assert {k: list(v) for k, v in R.route_multiple_nets(REQS)["paths"].items()} == want


def test_injected_search_failure_in_plain_mode():
    from orthoroute_gb300 import _lib
    R = router("plain")
    with _lib.inject_fault("ogr_find_path", _lib.OGR_ERR_ITER_CAP):
        with pytest.raises(RuntimeError, match="iteration limit"):
            R.route_multiple_nets(REQS)
