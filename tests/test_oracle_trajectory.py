"""CPU checks of the oracle trajectories committed for the benchmarked
workloads, and of the C heap search's whole-lattice fast path."""
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
G = os.path.join(ROOT, "tests", "golden")


def test_c0_trajectory_fixture_reproduces(tmp_path):
    """tests/golden/make_c1_trajectory.py --config c0 writes the committed
    fixture byte for byte (the oracle loop is deterministic under the fixed
    hash seed)."""
    out = tmp_path / "c0.json.gz"
    r = subprocess.run([sys.executable, os.path.join(G, "make_c1_trajectory.py"), "--config", "c0",
                        "--out", str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    from orthoroute_gb300.trajectory import load
    got, want = load(str(out)), load(os.path.join(G, "c0_trajectory.json.gz"))
    for k in ("wall_s", "record_wall_s", "host"):
        got.pop(k, None)
        want.pop(k, None)
    assert got == want


def test_c1_trajectory_fixture_is_consistent():
    """The committed c1 fixture: one record per iteration (plus detail-pass
    rounds), the first routes every net, metrics per iteration."""
    path = os.path.join(G, "c1_trajectory.json.gz")
    if not os.path.exists(path):
        return
    from orthoroute_gb300.trajectory import load
    doc = load(path)
    assert doc["lattice"] == [600, 400, 12] and doc["nets"] == 2000 and doc["max_iterations"] == 40
    assert len(doc["records"]) >= len(doc["iteration_metrics"]) == doc["result"]["iterations"]
    assert len(doc["records"][0]["changed"]) == 2000
    assert doc["searches"] >= 2000


def test_c_heap_whole_lattice_equals_python_heap():
    """The C heap search skips the global->ROI map when the ROI is the whole
    lattice in id order; paths and heap counters equal the Python restatement
    (with and without node penalties)."""
    from oracle.dijkstra import find_path_roi, find_path_roi_c
    from oracle.lattice import LatticeSpec, build_csr
    g = build_csr(LatticeSpec(30, 24, 6))
    n = g.num_nodes
    ident = np.arange(n, dtype=np.int32)
    rng = np.random.default_rng(3)
    for k in range(6):
        costs = (0.3 + rng.random(len(g.indices)) * 0.2).astype(np.float32)
        pen = (rng.random(n) * 0.5).astype(np.float32) if k % 2 else None
        s, d = (int(v) for v in rng.integers(0, 30 * 24, size=2))
        st_c, st_p = {}, {}
        a = find_path_roi_c(g.indptr, g.indices, s, d, costs, ident, ident, node_penalty=pen, stats=st_c)
        b = find_path_roi(g.indptr, g.indices, s, d, costs, ident, ident, node_penalty=pen, stats=st_p)
        assert a == b and st_c == st_p
        # a proper prefix ROI is not the identity: the map is used
        roi = ident[: n // 2]
        g2r = np.full(n, -1, dtype=np.int32)
        g2r[roi] = np.arange(len(roi), dtype=np.int32)
        a = find_path_roi_c(g.indptr, g.indices, s, d, costs, roi, g2r, node_penalty=None, stats=None)
        b = find_path_roi(g.indptr, g.indices, s, d, costs, roi, g2r, node_penalty=None)
        assert a == b
