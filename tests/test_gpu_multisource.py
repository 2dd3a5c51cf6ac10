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
