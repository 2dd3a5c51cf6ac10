"""The multi-source multi-sink search (ogr_find_path_multi) against the
reference's own outputs (golden vectors) and the oracle's restatement of
``find_path_multisource_multisink``: paths, entry/exit layers, and the
nodes popped / arcs scanned by the heap search."""
import ctypes as C
import os

import numpy as np
import pytest
import torch

from oracle.dijkstra import find_path_multisource
from oracle.lattice import LatticeSpec, build_csr
from oracle.roi import extract_roi

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(__file__), "golden")


def _ops(nx, ny, nz):
    from orthoroute_gb300 import Lattice
    from orthoroute_gb300.device import DeviceGraph, DeviceState, Ops
    g = DeviceGraph(Lattice(nx, ny, nz))
    return g, Ops(g, DeviceState(g))


def test_multisource_golden_cases():
    from test_oracle_golden import multisource_case
    nx, ny, nz = 40, 36, 6
    ref = build_csr(LatticeSpec(nx, ny, nz, allow_any_layer_via=True))
    g, ops = _ops(nx, ny, nz)
    assert np.array_equal(g.indices.cpu().numpy(), ref.indices)
    z = np.load(os.path.join(G, "multisource.npz"))
    for i in range(10):
        costs, roi, _, seeds, targets, pen = multisource_case(ref, z, i)
        res = ops.find_path_multi(seeds, targets, torch.from_numpy(costs).to(g.device), roi, pen)
        path, ent, exl = res if res else ([], -1, -1)
        np.testing.assert_array_equal(np.asarray(path, dtype=np.int32), z[f"m{i}_path"], err_msg=f"case {i}")
        assert [ent, exl] == z[f"m{i}_layers"].tolist()


def _random_sets(rng, nodes, k_seeds, k_targets):
    pick = rng.choice(nodes, size=k_seeds + k_targets, replace=False)
    seeds = [(int(n), float(np.round(rng.random() * 0.6, 3))) for n in pick[:k_seeds]]
    targets = [(int(n), float(np.round(rng.random() * 0.6, 3))) for n in pick[k_seeds:]]
    return seeds, targets


@pytest.mark.parametrize("seed", range(6))
def test_multisource_matches_oracle_with_stats(seed):
    nx, ny, nz = 30, 22, 6
    ref = build_csr(LatticeSpec(nx, ny, nz, allow_any_layer_via=True))
    g, ops = _ops(nx, ny, nz)
    rng = np.random.default_rng(900 + seed)
    E, N = len(ref.indices), ref.num_nodes
    for case in range(6):
        costs = (0.12 + rng.random(E) * 0.05).astype(np.float32)
        if case % 3 == 1:
            costs = (0.12 + rng.integers(0, 3, size=E) * 0.01).astype(np.float32)   # ties
        if case % 3 == 2:
            costs[rng.random(E) < 0.1] = np.float32("inf")
        if case % 2 == 0:
            roi = np.arange(N, dtype=np.int32)                                 # the whole lattice
        else:
            s, d = (int(v) for v in rng.integers(0, nx * ny, size=2))
            roi, _ = extract_roi(ref.indptr, ref.indices, N, ref.nx, ref.plane, s, d)
        g2r = np.full(N, -1, dtype=np.int32)
        g2r[roi] = np.arange(len(roi), dtype=np.int32)
        seeds, targets = _random_sets(rng, roi, int(rng.integers(1, 7)), int(rng.integers(1, 7)))
        if case == 3:
            targets.append((seeds[0][0], 0.9))                                 # a seed that is a target
        pen = (rng.integers(0, 3, size=len(roi)) * 0.2).astype(np.float32) if case % 2 else None
        st = {}
        want = find_path_multisource(ref.indptr, ref.indices, seeds, targets, costs, roi, g2r, node_penalty=pen,
                                     plane=ref.plane, stats=st)
        ops.stats.zero_()
        got = ops.find_path_multi(seeds, targets, torch.from_numpy(costs).to(g.device), roi, pen)
        assert got == (tuple(want) if want else None), (seed, case)
        if want is not None:
            s = ops.stats.cpu().numpy()
            assert int(s[0]) == st["scanned"] and int(s[1]) == st["settled"], (seed, case, s, st)


def test_multisource_edge_cases():
    nx, ny, nz = 12, 10, 4
    ref = build_csr(LatticeSpec(nx, ny, nz, allow_any_layer_via=True))
    g, ops = _ops(nx, ny, nz)
    N = ref.num_nodes
    costs = torch.full((len(ref.indices),), 0.4, dtype=torch.float32, device=g.device)
    roi = np.arange(N, dtype=np.int32)
    # no seed or no target in the ROI: no path
    assert ops.find_path_multi([(5, 0.0)], [(7, 0.0)], costs, roi[:5]) is None
    assert ops.find_path_multi([], [(7, 0.0)], costs, roi) is None
    # the cheapest target wins over a nearer dearer one, which is not expanded
    a = nx * ny + 1
    res = ops.find_path_multi([(a, 0.0)], [(a + 1, 5.0), (a + 3, 0.0)], costs, roi)
    assert res is not None and res[0][-1] == a + 3
    # a repeated seed is an argument error at the C boundary
    from orthoroute_gb300 import _lib
    dev = g.device
    sd = torch.tensor([a, a], dtype=torch.int32, device=dev)
    sc = torch.zeros(2, dtype=torch.float64, device=dev)
    td = torch.tensor([a + 3], dtype=torch.int32, device=dev)
    tc = torch.zeros(1, dtype=torch.float64, device=dev)
    r = torch.from_numpy(roi).to(dev)
    ws = ops.multi_workspace()
    n = C.c_int32(0)
    gc = g.cgraph()
    rc = ops.lib.ogr_find_path_multi(C.byref(gc), costs.data_ptr(), r.data_ptr(), N, None, sd.data_ptr(),
                                     sc.data_ptr(), 2, td.data_ptr(), tc.data_ptr(), 1, ws.data_ptr(),
                                     ops.multi_ws_bytes, ops.path_buf.data_ptr(), int(ops.path_buf.numel()),
                                     C.byref(n), None, None)
    assert rc == _lib.OGR_ERR_ARG
    # the workspace stays usable after the error
    assert ops.find_path_multi([(a, 0.0)], [(a + 3, 0.0)], costs, roi)[0][-1] == a + 3


@pytest.mark.parametrize("seed", range(6))
def test_full_lattice_multisource_matches_oracle(seed):
    """ogr_find_path_full_multi (the whole-lattice seeded search on all SMs)
    against the oracle's find_path_multisource on the identity ROI: paths,
    layers, nodes settled and arcs scanned, with the state's node penalty,
    ties, blocked arcs and a seed that is also a target."""
    from test_gpu_kernels import _costs, _penalty_state, make
    dims = [(40, 30, 6), (64, 48, 8), (90, 60, 4)][seed % 3]
    g, s, ops, ref = make(*dims)
    rng = np.random.default_rng(300 + seed)
    N = g.N
    ident = np.arange(N, dtype=np.int32)
    for case in range(4):
        costs = _costs((seed + case) % 4, g.E, rng)
        s.total_cost.copy_(torch.from_numpy(costs))
        ns = _penalty_state(s, N, rng, 3) if case % 2 == 0 else None
        pres_fac = float(rng.choice([1.0, 2.3]))
        pen = ns.owner_penalty(ident, 3, pres_fac) if ns is not None else None
        seeds, targets = _random_sets(rng, ident, int(rng.integers(1, 9)), int(rng.integers(1, 9)))
        if case == 1:
            targets.append((seeds[0][0], 0.9))
        st = {}
        want = find_path_multisource(ref.indptr, ref.indices, seeds, targets, costs, ident, ident, node_penalty=pen,
                                     plane=ref.plane, stats=st)
        ops.stats.zero_()
        net = ops.net_args(3, 0, 1, full_graph=True, pres_fac=pres_fac, penalty=ns is not None)
        got = ops.find_path_full_multi(seeds, targets, net)
        assert got == (tuple(want) if want else None), (seed, case)
        if want is not None:
            arcs, pops = ops.stats.cpu().tolist()[:2]
            assert (arcs, pops) == (st["scanned"], st["settled"]), (seed, case)
    # the per-node seed / target marks are restored: a plain search right after is unaffected
    from oracle.dijkstra import find_path_roi_c
    costs = _costs(3, g.E, rng)
    s.total_cost.copy_(torch.from_numpy(costs))
    for _ in range(2):
        a, b = (int(v) for v in rng.integers(0, ref.plane, size=2))
        want = find_path_roi_c(ref.indptr, ref.indices, a, b, costs, ident, ident)
        assert ops.find_path(ops.net_args(0, a, b, full_graph=True, penalty=False), engine="grid") == want


def test_full_lattice_multisource_edge_cases():
    from orthoroute_gb300 import _lib
    from test_gpu_kernels import make
    g, s, ops, ref = make(24, 20, 4)
    s.total_cost.fill_(0.4)
    net = ops.net_args(0, 0, 1, full_graph=True, penalty=False)
    plane = ref.plane
    a = plane + 1
    # the cheapest target wins over a nearer dearer one, which is not expanded
    res = ops.find_path_full_multi([(a, 0.0)], [(a + 1, 5.0), (a + 3, 0.0)], net)
    assert res is not None and res[0][-1] == a + 3 and res[0][0] == a
    # a target walled in by other targets is unreachable
    assert ops.find_path_full_multi([(a, 0.0)], [(a, float("inf"))], net) is None
    # argument errors at the C boundary: repeated target, negative seed cost
    for seeds, targets in (([(a, 0.0)], [(a + 2, 0.0), (a + 2, 1.0)]), ([(a, -1.0)], [(a + 2, 0.0)])):
        sd = torch.tensor([n for n, _ in seeds], dtype=torch.int32, device=g.device)
        sc = torch.tensor([c for _, c in seeds], dtype=torch.float64, device=g.device)
        td = torch.tensor([n for n, _ in targets], dtype=torch.int32, device=g.device)
        tc = torch.tensor([c for _, c in targets], dtype=torch.float64, device=g.device)
        n = C.c_int32(0)
        ws = ops.full_workspace()
        rc = ops.lib.ogr_find_path_full_multi(C.byref(g.cgraph()), C.byref(s.cstate()), C.byref(net),
                                              sd.data_ptr(), sc.data_ptr(), 1, td.data_ptr(), tc.data_ptr(),
                                              len(targets), ws.data_ptr(), ops.full_ws_bytes,
                                              ops.path_buf.data_ptr(), int(ops.path_buf.numel()), C.byref(n), None,
                                              None)
        assert rc == _lib.OGR_ERR_ARG
    # after the refused calls the marks are clean: the first case routes as before
    res2 = ops.find_path_full_multi([(a, 0.0)], [(a + 1, 5.0), (a + 3, 0.0)], net)
    assert res2 == res
