"""Pin the CPU oracle against golden fixtures produced by the reference itself.

The fixtures under ``tests/golden`` were written by ``make_golden.py``, which
drives the reference's own ``Lattice3D``, ``EdgeAccountant``,
``ROIExtractor`` and ``SimpleDijkstra`` on seeded inputs.  Every comparison
here is exact (bit-for-bit arrays, identical paths).
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import accounting as acc
from oracle.dijkstra import find_path_roi
from oracle.lattice import LatticeSpec, build_csr
from oracle.roi import extract_roi, roi_radius, extract_roi_bfs

G = os.path.join(os.path.dirname(__file__), "golden")
META = json.load(open(os.path.join(G, "golden.json")))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("tag", ["l0", "l1", "l2", "l3", "l4", "l5"])
def test_lattice_matches_reference(tag):
    m = META[tag]
    csr = build_csr(LatticeSpec(m["nx"], m["ny"], m["nz"], allow_any_layer_via=m["any"]))
    assert len(csr.indices) == m["E"]
    got = [sha(csr.indptr), sha(csr.indices), sha(csr.base_costs), sha(csr.edge_layer), sha(csr.edge_kind)]
    assert got == m["sha"]
    z = np.load(os.path.join(G, "lattice.npz"))
    if f"{tag}_indptr" in z:
        np.testing.assert_array_equal(csr.indptr, z[f"{tag}_indptr"])
        np.testing.assert_array_equal(csr.indices, z[f"{tag}_indices"])
        np.testing.assert_array_equal(csr.base_costs, z[f"{tag}_base"])


def test_edge_count_formula():
    """Lateral 2·Ny·(Nx−1) per H layer / 2·Nx·(Ny−1) per V layer + 2·pairs·Nx·Ny vias."""
    for nx, ny, nz, anyv in [(20, 10, 12, True), (20, 10, 12, False), (15, 7, 6, True)]:
        csr = build_csr(LatticeSpec(nx, ny, nz, allow_any_layer_via=anyv))
        lat = sum(2 * ny * (nx - 1) if z % 2 == 1 else 2 * nx * (ny - 1) for z in range(1, nz - 1))
        r = nz - 2
        pairs = (r * (r - 1) // 2 + r) if anyv else (nz - 2)
        assert len(csr.indices) == lat + 2 * pairs * nx * ny


@pytest.fixture(scope="module")
def acc_lattice():
    return build_csr(LatticeSpec(14, 12, 6, allow_any_layer_via=True))


@pytest.mark.parametrize("case", [0, 1, 2])
def test_accounting_matches_reference(acc_lattice, case):
    g = acc_lattice
    z = np.load(os.path.join(G, "accounting.npz"))
    pres_fac, hw, vmult, bw = META[f"acc_c{case}"]
    E = len(g.indices)
    A = acc.Accountant(E)
    A.present[:] = z["present"]
    A.present_ema[:] = z["present_ema"]
    A.history[:] = z["history"]
    A.update_costs(g.base_costs, pres_fac, hw, via_cost_multiplier=vmult, base_cost_weight=bw,
                   edge_layer=g.edge_layer, layer_bias_per_layer=z["layer_bias"], edge_kind=g.edge_kind)
    np.testing.assert_array_equal(A.total_cost, z[f"c{case}_total"])
    A.begin_live_present_costs()
    np.testing.assert_array_equal(A.total_cost, z[f"c{case}_live"])
    touched = z[f"c{case}_touched"].tolist()
    A.commit_path(touched)
    A.refresh_live_present_costs(touched)
    np.testing.assert_array_equal(A.total_cost, z[f"c{case}_after_commit"])
    np.testing.assert_array_equal(A.present, z[f"c{case}_present_after_commit"])
    A.clear_path(touched[:20])
    A.refresh_live_present_costs(touched[:20])
    np.testing.assert_array_equal(A.total_cost, z[f"c{case}_after_clear"])
    np.testing.assert_array_equal(A.present, z[f"c{case}_present_after_clear"])
    A.update_history(1.2 if case == 2 else 0.2, base_costs=g.base_costs, history_cap_multiplier=15.0,
                     decay_factor=1.0 if case != 1 else 0.98, use_raw_present=True)
    np.testing.assert_array_equal(A.history, z[f"c{case}_history"])
    A.update_present_ema(0.4)
    np.testing.assert_array_equal(A.present_ema, z[f"c{case}_ema"])


@pytest.fixture(scope="module")
def roi_lattice():
    nx, ny, nz = META["roi_lattice"]
    return build_csr(LatticeSpec(nx, ny, nz, allow_any_layer_via=True))


def test_roi_matches_reference(roi_lattice):
    g = roi_lattice
    z = np.load(os.path.join(G, "roi.npz"))
    N = g.num_nodes
    for i, (s, d, bonus, maxn) in enumerate(META["roi_cases"]):
        r = roi_radius(s, d, g.nx, g.plane, bonus)
        roi, g2r = extract_roi_bfs(g.indptr, g.indices, N, s, d, initial_radius=r,
                                   stagnation_bonus=bonus, max_nodes=maxn)
        np.testing.assert_array_equal(roi, z[f"roi{i}"], err_msg=f"case {i}")
        assert g2r[roi[5]] == 5


def _sssp_inputs(g, i):
    rng = np.random.default_rng(1300 + i)
    E = len(g.indices)
    costs = (0.12 + rng.random(E) * 0.05).astype(np.float32)
    if i % 3 == 1:
        costs = (0.12 + rng.integers(0, 4, size=E) * 0.01).astype(np.float32)
    if i % 5 == 4:
        costs[rng.choice(E, size=E // 20, replace=False)] = np.float32("inf")
    s = int(rng.integers(0, g.nx * g.ny))
    d = int(rng.integers(0, g.nx * g.ny))
    assert [s, d] == META["sssp_cases"][i]
    roi, g2r = extract_roi(g.indptr, g.indices, g.num_nodes, g.nx, g.plane, s, d)
    pen = None
    if i % 2 == 0:
        pen = (rng.integers(0, 3, size=len(roi)) * 0.5 * (i + 1)).astype(np.float32)
    return s, d, costs, roi, g2r, pen


@pytest.mark.parametrize("i", range(10))
def test_sssp_matches_reference(roi_lattice, i):
    g = roi_lattice
    z = np.load(os.path.join(G, "sssp.npz"))
    s, d, costs, roi, g2r, pen = _sssp_inputs(g, i)
    path = find_path_roi(g.indptr, g.indices, s, d, costs, roi, g2r, node_penalty=pen)
    np.testing.assert_array_equal(np.asarray(path if path else [], dtype=np.int32), z[f"s{i}_path"])


def test_sssp_net_trace_matches_reference():
    """Replay every recorded find_path_roi call of a real reference routing run."""
    m = META["r0"]
    g = build_csr(LatticeSpec(m["nx"], m["ny"], m["nz"]))
    z = np.load(os.path.join(G, "runs.npz"))
    N = g.num_nodes
    for j in range(m["n_trace"]):
        s, d = z[f"r0_t{j}_sd"].tolist()
        roi = z[f"r0_t{j}_roi"]
        g2r = np.full(N, -1, dtype=np.int32)
        g2r[roi] = np.arange(len(roi), dtype=np.int32)
        pen = z[f"r0_t{j}_pen"] if f"r0_t{j}_pen" in z else None
        path = find_path_roi(g.indptr, g.indices, s, d, z[f"r0_t{j}_costs"], roi, g2r, node_penalty=pen)
        np.testing.assert_array_equal(np.asarray(path or [], dtype=np.int32), z[f"r0_t{j}_path"])
        # The recorded ROI is what the oracle's BFS extracts too.
        roi2, _ = extract_roi(g.indptr, g.indices, N, g.nx, g.plane, s, d)
        np.testing.assert_array_equal(roi2, roi)


@pytest.mark.parametrize("i", range(10))
def test_c_heap_dijkstra_matches_reference(roi_lattice, i):
    """The C restatement used by the CPU baseline gives the same paths."""
    from oracle.dijkstra import find_path_roi_c
    g = roi_lattice
    z = np.load(os.path.join(G, "sssp.npz"))
    s, d, costs, roi, g2r, pen = _sssp_inputs(g, i)
    st_py, st_c = {}, {}
    p1 = find_path_roi(g.indptr, g.indices, s, d, costs, roi, g2r, node_penalty=pen, stats=st_py)
    p2 = find_path_roi_c(g.indptr, g.indices, s, d, costs, roi, g2r, node_penalty=pen, stats=st_c)
    np.testing.assert_array_equal(np.asarray(p2 or [], dtype=np.int32), z[f"s{i}_path"])
    assert p1 == p2 and st_py == st_c


def multisource_case(g, z, i):
    """Inputs of golden multi-source case i (arc costs regenerated from the seed)."""
    from tests.golden.make_multisource_golden import multisource_costs
    costs = multisource_costs(len(g.indices), i)
    roi = z[f"m{i}_roi"]
    g2r = np.full(g.num_nodes, -1, dtype=np.int32)
    g2r[roi] = np.arange(len(roi), dtype=np.int32)
    seeds = list(zip(z[f"m{i}_seeds"].tolist(), z[f"m{i}_seed_cost"].tolist()))
    targets = list(zip(z[f"m{i}_targets"].tolist(), z[f"m{i}_target_cost"].tolist()))
    pen = z[f"m{i}_pen"] if f"m{i}_pen" in z else None
    return costs, roi, g2r, seeds, targets, pen


@pytest.mark.parametrize("i", range(10))
def test_multisource_matches_reference(roi_lattice, i):
    """find_path_multisource_multisink of the reference on portal-like seed columns."""
    from oracle.dijkstra import find_path_multisource
    g = roi_lattice
    z = np.load(os.path.join(G, "multisource.npz"))
    costs, roi, g2r, seeds, targets, pen = multisource_case(g, z, i)
    res = find_path_multisource(g.indptr, g.indices, seeds, targets, costs, roi, g2r, node_penalty=pen,
                                plane=g.plane)
    path, ent, exl = res if res else ([], -1, -1)
    np.testing.assert_array_equal(np.asarray(path, dtype=np.int32), z[f"m{i}_path"])
    assert [ent, exl] == z[f"m{i}_layers"].tolist()
