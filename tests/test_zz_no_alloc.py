"""The allocation-free search entry point, ``ogr_find_path_noalloc``.

It serves hosts that cannot give the library a device workspace (a plugin
living inside an application that owns the GPU allocator, or a serving
process that fixes its memory budget at start-up).  Its scratch is a fixed
array inside the library, shared by every call, so this test checks through
the C ABI that

* two calls in a row return exactly the paths and heap statistics of the
  workspace-based ``ogr_find_path`` on the same inputs, and the oracle's;
* a call on a large lattice followed by calls on a small one (the array
  keeps the larger call's contents) still matches;
* a lattice above the array's node limit and out-of-range terminals are
  refused before anything runs.

This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(nx=48, ny=40, nz=6, seed=2024):
    import torch
    from orthoroute_gb300 import Lattice, _lib
    from orthoroute_gb300.device import DeviceGraph, DeviceState, Ops
    g = DeviceGraph(Lattice(nx, ny, nz))
    s = DeviceState(g)
    ops = Ops(g, s)
    rng = np.random.default_rng(seed)
    costs = (0.12 + rng.random(g.E) * 0.05).astype(np.float32)
    s.total_cost.copy_(torch.from_numpy(costs))
    hist = (rng.integers(0, 3, size=g.N) * 0.5).astype(np.float32)
    s.node_history.copy_(torch.from_numpy(hist))
    return torch, _lib, g, s, ops, rng, costs, hist


def _noalloc(lib, g, s, net, out, stats=None):
    n = C.c_int32(0)
    rc = lib.ogr_find_path_noalloc(C.byref(g.cgraph()), C.byref(s.cstate()), C.byref(net), out.data_ptr(),
                                   int(out.numel()), C.byref(n), None if stats is None else stats.data_ptr(), None)
    return rc, n.value


def _check_calls(torch, _lib, g, s, ops, rng, nx, ny, calls, costs=None, hist=None):
    lib = _lib.load()
    out = torch.empty(g.N, dtype=torch.int32, device=g.device)
    stats = torch.zeros(4, dtype=torch.int64, device=g.device)
    for call in range(calls):
        src, dst = (int(v) for v in rng.integers(0, nx * ny, size=2))
        from oracle.roi import roi_radius
        depth = min(int(roi_radius(src, dst, nx, nx * ny, 0.0)), 80)   # the reference's BFS depth, no stagnation
        net = ops.net_args(3, src, dst, max_depth=depth, halo=2, pres_fac=1.5, penalty=True)
        ops.stats.zero_()
        want = ops.find_path(net)
        want_stats = ops.stats.cpu().tolist()
        stats.zero_()
        rc, n = _noalloc(lib, g, s, net, out, stats)
        assert rc in (_lib.OGR_OK, _lib.OGR_NO_PATH), rc
        got = out[:n].cpu().tolist() if rc == _lib.OGR_OK and n > 1 else None
        assert got == want, f"call {call}"
        assert stats.cpu().tolist() == want_stats, f"call {call}"
        if costs is not None and want is not None:
            from oracle.lattice import LatticeSpec, build_csr
            from oracle.roi import extract_roi
            from oracle.dijkstra import find_path_roi
            from oracle.tallies import NodeState
            ref = build_csr(LatticeSpec(nx, ny, g.lattice.nz))
            roi, g2r = extract_roi(ref.indptr, ref.indices, ref.num_nodes, nx, nx * ny, src, dst)
            ns = NodeState(ref.num_nodes, 1, 1)
            ns.node_history[:] = hist
            pen = ns.owner_penalty(roi, 3, 1.5)
            assert find_path_roi(ref.indptr, ref.indices, src, dst, costs, roi, g2r, node_penalty=pen) == got


def test_noalloc_matches_workspace_search_twice():
    torch, _lib, g, s, ops, rng, costs, hist = _setup()
    _check_calls(torch, _lib, g, s, ops, rng, 48, 40, 2, costs, hist)


def test_noalloc_large_lattice_then_small():
    """The shared array after a 240,000-node call, then two 11,520-node calls."""
    torch, _lib, g, s, ops, rng, _, _ = _setup(200, 150, 8, seed=7)
    _check_calls(torch, _lib, g, s, ops, rng, 200, 150, 1)
    torch, _lib, g, s, ops, rng, _, _ = _setup(48, 40, 6, seed=8)
    _check_calls(torch, _lib, g, s, ops, rng, 48, 40, 2)


def test_noalloc_rejects_bad_terminals():
    torch, _lib, g, s, ops, rng, _, _ = _setup()
    lib = _lib.load()
    out = torch.empty(g.N, dtype=torch.int32, device=g.device)
    for src, dst in [(-1, 5), (5, g.N), (g.N + 3, 0)]:
        net = ops.net_args(3, 0, 1, max_depth=80, halo=2, pres_fac=1.5, penalty=True)
        net.src, net.dst = src, dst
        assert _noalloc(lib, g, s, net, out)[0] == _lib.OGR_ERR_ARG


def test_noalloc_rejects_lattices_above_its_limit():
    import torch
    from orthoroute_gb300 import _lib
    lib = _lib.load()
    N = _lib.OGR_NOALLOC_MAX_NODES + 1
    g = _lib.Graph(N, 1, 1, N, 0, None, None, None, None)
    st = _lib.State()
    net = _lib.NetArgs(0, 0, 1, 0, 10, 2, 75000.0, 50000, 0.0, 0.0, 0.0, 0)
    n = C.c_int32(0)
    dummy = torch.empty(4, dtype=torch.int32, device="cuda")
    assert lib.ogr_find_path_noalloc(C.byref(g), C.byref(st), C.byref(net), dummy.data_ptr(), 4, C.byref(n),
                                     None, None) == _lib.OGR_ERR_CAPACITY
