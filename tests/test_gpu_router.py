"""End-to-end parity of the GPU router with the CPU oracle loop and with the
reference's own recorded routing runs (every path of every iteration)."""
import hashlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

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


def gpu_router(nx, ny, nz, iters, mode="persistent", full_engine="grid", window_slots=32):
    from orthoroute_gb300 import Lattice
    from orthoroute_gb300.router import PathFinderConfig, PathFinderRouter
    R = PathFinderRouter(PathFinderConfig(max_iterations=iters), mode=mode, full_engine=full_engine,
                         window_slots=window_slots)
    R.initialize_lattice(Lattice(nx, ny, nz), board_bounds(nx, ny))
    return R


@pytest.mark.parametrize("mode,windows", [("persistent", 32), ("persistent", 0), ("plain", 0)])
@pytest.mark.parametrize("tag", ["r0", "r1"])
def test_gpu_router_matches_reference_runs(tag, mode, windows):
    m = META[tag]
    z = np.load(os.path.join(G, "runs.npz"))
    reqs = [(f"N{int(r[0])}", int(r[1]), int(r[2])) for r in z[f"{tag}_reqs"]]
    R = gpu_router(m["nx"], m["ny"], m["nz"], m["iters"], mode, window_slots=windows)
    R.trace = []
    res = R.route_multiple_nets(reqs)
    n_ref = sum(1 for k in z.files if k.startswith(f"{tag}_it"))
    assert len(R.trace) == n_ref
    for j, tr in enumerate(R.trace):
        np.testing.assert_array_equal(flat(tr), z[f"{tag}_it{j}_paths"], err_msg=f"{tag} record {j}")
    for a, b in zip(res["iteration_metrics"], m["metrics"]):
        assert {k: a[k] for k in b} == b
    assert hashlib.sha256(flat(R.net_paths).tobytes()).hexdigest() == m["final_paths_sha"]
    # F4: the emitted geometry equals the reference's on the same final paths
    geo = json.load(open(os.path.join(G, "geometry.json")))[tag]
    R.emit_geometry()
    prov = R.get_provisional_geometry()
    key = lambda d: json.dumps(d, sort_keys=True)
    assert sorted(map(key, prov.tracks)) == sorted(map(key, geo["tracks"]))
    assert sorted(map(key, prov.vias)) == sorted(map(key, geo["vias"]))


def seeded_nets(nx, ny, n, seed, dmin=5, dmax=80):
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        x0, x1 = rng.integers(0, nx, size=2)
        y0, y1 = rng.integers(0, ny, size=2)
        d = abs(int(x1) - int(x0)) + abs(int(y1) - int(y0))
        if dmin <= d <= dmax:
            out.append((f"N{len(out)}", int(y0) * nx + int(x0), int(y1) * nx + int(x1)))
    return out


CASES = [((40, 36, 6), 60, 8, 7, 160, "grid"), ((48, 40, 8), 90, 10, 11, 160, "grid"),
         ((140, 40, 6), 40, 6, 5, 160, "grid"), ((140, 40, 6), 40, 6, 5, 160, "cta"),
         ((260, 60, 8), 50, 6, 3, 300, "grid"), ((260, 60, 8), 50, 6, 3, 300, "auto")]


@pytest.mark.parametrize("mode", ["persistent", "plain"])
@pytest.mark.parametrize("dims,n_nets,iters,seed,dmax,engine", CASES)
def test_gpu_router_matches_oracle_loop(dims, n_nets, iters, seed, dmax, engine, mode, tmp_path, monkeypatch):
    monkeypatch.setenv("ORTHOROUTE_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    nx, ny, nz = dims
    reqs = seeded_nets(nx, ny, n_nets, seed, dmin=5, dmax=dmax)
    R = gpu_router(nx, ny, nz, iters, mode, engine)
    R.trace = []
    res = R.route_multiple_nets(reqs)
    O = OracleRouter(LatticeSpec(nx, ny, nz), board_bounds(nx, ny), Config(max_iterations=iters), fast=True)
    O.trace = []
    ores = O.route({n: (s, d) for n, s, d in reqs})
    assert len(R.trace) == len(O.trace)
    for j, (a, b) in enumerate(zip(R.trace, O.trace)):
        np.testing.assert_array_equal(flat(a), flat(b), err_msg=f"record {j}")
    assert bool(res["success"]) == bool(ores["success"])
    for k in ("barrel_conflicts", "overuse_sum", "failed_nets"):
        if k in ores and k in res:
            assert res[k] == ores[k], k
    if engine == "auto":
        assert R.tuning is not None and R.full_engine == R.tuning.full_engine


@pytest.mark.parametrize("mode", ["persistent", "plain"])
def test_gpu_router_trivial_and_skipped_requests(mode):
    """Requests with src == dst are routed trivially (a one-node path, no
    task), non-int endpoints are skipped, as the reference parses them; the
    run equals the oracle loop started with the trivial paths in place."""
    nx, ny, nz, iters = 40, 36, 6, 6
    reqs = seeded_nets(nx, ny, 50, 21, dmin=5, dmax=160)
    trivial = [(f"N{50 + k}", reqs[k][1], reqs[k][1]) for k in range(0, 12, 3)]
    skipped = [("N99", np.int64(5), 9)]
    R = gpu_router(nx, ny, nz, iters, mode)
    R.trace = []
    seen = []
    res = R.route_multiple_nets(reqs + trivial + skipped,
                                iteration_cb=lambda it, tr, vi, osum, ocnt: seen.append((it, tr, vi)))
    assert [it for it, _, _ in seen] == list(range(1, len(seen) + 1)) and len(seen) == res["iterations"]
    assert all(t["net"] in R.net_paths for _, tr, _ in seen for t in tr) and seen[-1][1]   # provisional geometry
    assert "N99" not in R.net_paths
    assert all(R.net_paths[n] == [s] for n, s, _ in trivial)
    O = OracleRouter(LatticeSpec(nx, ny, nz), board_bounds(nx, ny), Config(max_iterations=iters), fast=True)
    O.trace = []
    for n, s, _ in trivial:
        O.net_paths[n] = [s]
    ores = O.route({n: (s, d) for n, s, d in reqs})
    assert len(R.trace) == len(O.trace)
    for j, (a, b) in enumerate(zip(R.trace, O.trace)):
        np.testing.assert_array_equal(flat(a), flat(b), err_msg=f"record {j}")
    for k in ("barrel_conflicts", "overuse_sum", "failed_nets"):
        if k in ores and k in res:
            assert res[k] == ores[k], k


def test_gpu_router_no_routable_nets():
    R = gpu_router(20, 16, 6, 4)
    assert R.route_multiple_nets([]) == {}
    res = R.route_multiple_nets([("A", 7, 7), ("B", 3.0, 9)])
    assert res["error_code"] == "NO-ROUTABLE-NETS" and res["excluded_net_ids"] == ["A", "B"]
    assert res["failed_nets"] == 2 and not res["success"]


@pytest.mark.parametrize("mode", ["persistent", "plain"])
def test_gpu_router_multipin_star_matches_oracle_loop(mode):
    """Multi-pin nets (2-16 pins in a box) as star requests: every sink of every
    net in the persistent pass, paths identical to the oracle loop's."""
    from orthoroute_gb300.multipin import seeded_multipin_nets, star_requests
    nx, ny, nz, iters = 60, 50, 6, 6
    reqs = star_requests(seeded_multipin_nets(nx, ny, 25, 8, box=20))
    R = gpu_router(nx, ny, nz, iters, mode)
    R.trace = []
    res = R.route_multiple_nets(reqs)
    O = OracleRouter(LatticeSpec(nx, ny, nz), board_bounds(nx, ny), Config(max_iterations=iters), fast=True)
    O.trace = []
    for n, s, d in reqs:
        if s == d:
            O.net_paths[n] = [s]
    ores = O.route({n: (s, d) for n, s, d in reqs if s != d})
    key = lambda paths: {k: list(v) for k, v in paths.items()}
    assert len(R.trace) == len(O.trace)
    for j, (a, b) in enumerate(zip(R.trace, O.trace)):
        assert key(a) == key(b), f"record {j}"
    for k in ("barrel_conflicts", "overuse_sum", "failed_nets"):
        if k in ores and k in res:
            assert res[k] == ores[k], k
