"""Pin the oracle's negotiation loop against full routing runs of the reference.

``make_golden.py`` ran the reference ``PathFinderRouter.route_multiple_nets``
(CPU path, portals off) on seeded tuple requests and recorded every net's
path at each history update (each negotiation iteration, then each detail
pass iteration), the iteration metrics and the final result.  The oracle
loop must reproduce all of it exactly.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle.lattice import LatticeSpec
from oracle.loop import Config, OracleRouter

G = os.path.join(os.path.dirname(__file__), "golden")
META = json.load(open(os.path.join(G, "golden.json")))


def board_bounds(nx, ny, pitch=0.4):
    sx = (nx - 1) * pitch - 6.0 + 1e-6
    sy = (ny - 1) * pitch - 6.0 + 1e-6
    return (7.0, 7.0, 10.0 + sx + 3.0, 10.0 + sy + 3.0)


def flat(paths):
    out = []
    for name in sorted(paths, key=lambda s: int(s[1:])):
        out.append(len(paths[name]))
        out.extend(paths[name])
    return np.asarray(out, dtype=np.int64)


@pytest.mark.parametrize("tag", ["r0", "r1"])
def test_loop_matches_reference_run(tag):
    m = META[tag]
    z = np.load(os.path.join(G, "runs.npz"))
    tasks = {f"N{int(r[0])}": (int(r[1]), int(r[2])) for r in z[f"{tag}_reqs"]}
    R = OracleRouter(LatticeSpec(m["nx"], m["ny"], m["nz"]), board_bounds(m["nx"], m["ny"]),
                     Config(max_iterations=m["iters"]))
    R.trace = []
    res = R.route(tasks)
    n_ref = sum(1 for k in z.files if k.startswith(f"{tag}_it"))
    assert len(R.trace) == n_ref
    for j, tr in enumerate(R.trace):
        np.testing.assert_array_equal(flat(tr), z[f"{tag}_it{j}_paths"], err_msg=f"{tag} record {j}")
    for a, b in zip(res["iteration_metrics"], m["metrics"]):
        assert a == b
    ref = m["result"]
    assert bool(res["success"]) == bool(ref["success"])
    for k in ("barrel_conflicts", "overuse_sum", "failed_nets", "iterations"):
        if ref.get(k) is not None:
            assert res[k] == ref[k], k
    got_sha = hashlib.sha256(flat(R.net_paths).tobytes()).hexdigest()
    assert got_sha == m["final_paths_sha"]


@pytest.mark.parametrize("tag", ["r0", "r1"])
def test_fast_loop_matches_reference_run(tag):
    """The loop with the C heap Dijkstra (CPU baseline) is the same restatement."""
    m = META[tag]
    z = np.load(os.path.join(G, "runs.npz"))
    tasks = {f"N{int(r[0])}": (int(r[1]), int(r[2])) for r in z[f"{tag}_reqs"]}
    R = OracleRouter(LatticeSpec(m["nx"], m["ny"], m["nz"]), board_bounds(m["nx"], m["ny"]),
                     Config(max_iterations=m["iters"]), fast=True)
    R.route(tasks)
    assert hashlib.sha256(flat(R.net_paths).tobytes()).hexdigest() == m["final_paths_sha"]
