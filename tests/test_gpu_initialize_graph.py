"""The drop-in entry ``PathFinderRouter.initialize_graph(board)``
(unified_pathfinder.py:2800): a board object with the attributes the
reference reads (nets with pads and positions, layer_count) gives the same
lattice as the reference's own run of the same board, and routing that
run's requests through it reproduces every path of every iteration."""
import hashlib
import json
import os
from types import SimpleNamespace as NS

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(__file__), "golden")


def board(nx, ny, nz, pitch=0.4):
    """The two-corner-pad board of the golden runs: pad bbox + 3 mm margin
    spans exactly nx x ny sites."""
    sx = (nx - 1) * pitch - 6.0 + 1e-6
    sy = (ny - 1) * pitch - 6.0 + 1e-6
    p1 = NS(id="a", position=NS(x=10.0, y=10.0), layer="F.Cu")
    p2 = NS(id="b", position=NS(x=10.0 + sx, y=10.0 + sy), layer="F.Cu")
    return NS(id="b", name="b", layer_count=nz, nets=[NS(id="n", name="BOUNDS", pads=[p1, p2])])


def flat(paths):
    out = []
    for name in sorted(paths, key=lambda s: int(s[1:])):
        out.append(len(paths[name]))
        out.extend(paths[name])
    return np.asarray(out, dtype=np.int64)


@pytest.mark.parametrize("tag", ["r0", "r1"])
def test_initialize_graph_from_board_reproduces_reference_run(tag):
    from orthoroute_gb300.router import PathFinderConfig, PathFinderRouter
    m = json.load(open(os.path.join(G, "golden.json")))[tag]
    z = np.load(os.path.join(G, "runs.npz"))
    nx, ny, nz = m["nx"], m["ny"], m["nz"]
    cfg = PathFinderConfig(max_iterations=m["iters"])
    cfg.preferred_layer_directions = ['v'] + ['h' if k % 2 == 1 else 'v' for k in range(1, nz)]
    R = PathFinderRouter(cfg)
    assert R.initialize_graph(board(nx, ny, nz)) is True
    assert (R.nx, R.ny, R.nz) == (nx, ny, nz)
    from oracle.lattice import LatticeSpec, build_csr
    assert R.E == len(build_csr(LatticeSpec(nx, ny, nz)).indices)
    reqs = [(f"N{int(r[0])}", int(r[1]), int(r[2])) for r in z[f"{tag}_reqs"]]
    R.trace = []
    res = R.route_multiple_nets(reqs)
    n_ref = sum(1 for k in z.files if k.startswith(f"{tag}_it"))
    assert len(R.trace) == n_ref
    for j, tr in enumerate(R.trace):
        np.testing.assert_array_equal(flat(tr), z[f"{tag}_it{j}_paths"], err_msg=f"{tag} record {j}")
    assert hashlib.sha256(flat(R.net_paths).tobytes()).hexdigest() == m["final_paths_sha"]
    for a, b in zip(res["iteration_metrics"], m["metrics"]):
        assert {k: a[k] for k in b} == b


def test_initialize_graph_derives_layer_axes_from_demand():
    """Without preferred directions the layer axes come from the pads' x/y
    demand (board_analyzer.py:65-105): a wide board gets more horizontal
    inner layers; F.Cu stays vertical."""
    from orthoroute_gb300.router import PathFinderConfig, PathFinderRouter
    b = board(40, 30, 8)
    wide = [NS(id=f"w{k}", name=f"W{k}", pads=[NS(position=NS(x=10.0, y=12.0 + k)),
                                               NS(position=NS(x=20.0, y=12.0 + k))]) for k in range(5)]
    b.nets = b.nets + wide
    R = PathFinderRouter(PathFinderConfig(max_iterations=1))
    R.initialize_graph(b)
    dirs = R.lattice.layer_dirs
    assert dirs[0] == "v" and dirs.count("h") > dirs[1:-1].count("v")
