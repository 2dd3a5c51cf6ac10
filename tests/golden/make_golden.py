"""Generate the golden fixtures that pin the CPU oracle to the reference.

Run in a container where the reference source tree is available (it is read
only and never copied):

    python tests/golden/make_golden.py /path/to/OrthoRoute

The script imports the reference's own classes (``Lattice3D``,
``EdgeAccountant``, ``ROIExtractor``, ``SimpleDijkstra``,
``PathFinderRouter``), drives them on seeded synthetic inputs and writes the
inputs that cannot be regenerated cheaply plus every output into
``tests/golden/*.npz``.  The test suite never imports the reference: it only
reads these fixtures.
"""
from __future__ import annotations

import hashlib
import json
import logging
import os
import random
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def sha(a) -> str:
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.tobytes()).hexdigest()


def default_dirs(nz):
    return ['v'] + ['h' if z % 2 == 1 else 'v' for z in range(1, nz)]


def make_board(Board, Component, Coordinate, Net, Pad, nx, ny, nz, pitch=0.4):
    """Two corner pads whose bbox + 3 mm margin yields exactly nx × ny sites."""
    b = Board(id="b", name="b")
    b.layer_count = nz
    sx = (nx - 1) * pitch - 6.0 + 1e-6
    sy = (ny - 1) * pitch - 6.0 + 1e-6
    p1 = Pad(id="a", component_id="c", position=Coordinate(x=10.0, y=10.0), layer="F.Cu",
             size=(0.2, 0.2), net_id=None)
    p2 = Pad(id="b", component_id="c", position=Coordinate(x=10.0 + sx, y=10.0 + sy), layer="F.Cu",
             size=(0.2, 0.2), net_id=None)
    c = Component(id="c", reference="U", value="v", footprint="f", position=Coordinate(x=10.0, y=10.0))
    c.pads += [p1, p2]
    b.add_component(c)
    b.add_net(Net(id="n", name="BOUNDS", pads=[p1, p2]))
    return b


def seeded_two_pin_nets(nx, ny, nz, n_nets, seed, dmin=5, dmax=80):
    """Two-pin nets with endpoints on layer 0 (same generator as the tests)."""
    rng = np.random.default_rng(seed)
    plane = nx * ny
    out = []
    while len(out) < n_nets:
        x0, x1 = rng.integers(0, nx, size=2)
        y0, y1 = rng.integers(0, ny, size=2)
        d = abs(int(x1) - int(x0)) + abs(int(y1) - int(y0))
        if dmin <= d <= dmax:
            out.append((f"N{len(out)}", int(y0) * nx + int(x0), int(y1) * nx + int(x1)))
    return out


def main(ref_root):
    sys.path.insert(0, ref_root)
    logging.disable(logging.WARNING)
    os.environ.setdefault("PYTHONHASHSEED", "0")
    from orthoroute.algorithms.manhattan import unified_pathfinder as up
    from orthoroute.domain.models.board import Board, Component, Coordinate, Net, Pad

    meta = {}

    # ---------------------------------------------------------------- A1 lattice
    lat = {}
    for tag, (nx, ny, nz, anyv) in {
        "l0": (7, 5, 6, True), "l1": (6, 4, 5, False), "l2": (9, 8, 12, True),
        "l3": (5, 5, 4, True), "l4": (30, 20, 8, True), "l5": (12, 10, 20, False),
    }.items():
        dirs = default_dirs(nz)
        L = up.Lattice3D((0, 0, (nx - 1) * 0.4 + 1e-6, (ny - 1) * 0.4 + 1e-6), 0.4, nz,
                         preferred_layer_directions=dirs)
        g = L.build_graph(0.7, allow_any_layer_via=anyv, min_via_center_spacing=0.4)
        assert (L.x_steps, L.y_steps) == (nx, ny)
        meta[tag] = dict(nx=nx, ny=ny, nz=nz, any=anyv, E=int(len(g.indices)),
                         sha=[sha(g.indptr), sha(g.indices), sha(g.base_costs),
                              sha(g.edge_layer), sha(g.edge_kind)])
        if nx * ny * nz <= 1000:
            lat[f"{tag}_indptr"] = g.indptr
            lat[f"{tag}_indices"] = g.indices
            lat[f"{tag}_base"] = g.base_costs
    np.savez_compressed(os.path.join(HERE, "lattice.npz"), **lat)

    # ------------------------------------------------------- A2–A4 accounting
    nx, ny, nz = 14, 12, 6
    dirs = default_dirs(nz)
    L = up.Lattice3D((0, 0, (nx - 1) * 0.4 + 1e-6, (ny - 1) * 0.4 + 1e-6), 0.4, nz,
                     preferred_layer_directions=dirs)
    g = L.build_graph(0.7, allow_any_layer_via=True, min_via_center_spacing=0.4)
    E = len(g.indices)
    rng = np.random.default_rng(7)
    acc_in = dict(
        present=rng.integers(0, 4, size=E).astype(np.float32),
        present_ema=(rng.random(E) * 3).astype(np.float32),
        history=(rng.random(E) * 0.5).astype(np.float32),
        layer_bias=(1.0 + rng.random(nz) * 0.6).astype(np.float32),
    )
    acc_out = {}
    for case, (pres_fac, hw, vmult, bw) in enumerate([(1.0, 12.0, 1.0, 0.3), (3.7, 9.6, 1.5, 0.3),
                                                      (57.3, 14.4, 0.5, 0.01)]):
        A = up.EdgeAccountant(E)
        A.present[:] = acc_in["present"]
        A.present_ema[:] = acc_in["present_ema"]
        A.history[:] = acc_in["history"]
        A.update_costs(g.base_costs, pres_fac, hw, via_cost_multiplier=vmult, base_cost_weight=bw,
                       edge_layer=g.edge_layer, layer_bias_per_layer=acc_in["layer_bias"],
                       edge_kind=g.edge_kind)
        acc_out[f"c{case}_total"] = A.total_cost.copy()
        A.begin_live_present_costs()
        acc_out[f"c{case}_live"] = A.total_cost.copy()
        touched = rng.choice(E, size=50, replace=False).tolist()
        acc_out[f"c{case}_touched"] = np.asarray(touched, dtype=np.int64)
        A.commit_path(touched)
        A.refresh_live_present_costs(touched)
        acc_out[f"c{case}_after_commit"] = A.total_cost.copy()
        acc_out[f"c{case}_present_after_commit"] = A.present.copy()
        A.clear_path(touched[:20])
        A.refresh_live_present_costs(touched[:20])
        acc_out[f"c{case}_after_clear"] = A.total_cost.copy()
        acc_out[f"c{case}_present_after_clear"] = A.present.copy()
        A.update_history(1.2 if case == 2 else 0.2, base_costs=g.base_costs, history_cap_multiplier=15.0,
                         decay_factor=1.0 if case != 1 else 0.98, use_raw_present=True)
        acc_out[f"c{case}_history"] = A.history.copy()
        A.update_present_ema(0.4)
        acc_out[f"c{case}_ema"] = A.present_ema.copy()
        meta[f"acc_c{case}"] = [pres_fac, hw, vmult, bw]
    np.savez_compressed(os.path.join(HERE, "accounting.npz"), **acc_in, **acc_out)

    # ----------------------------------------------------------------- A6 ROI
    roi_out = {}
    nx, ny, nz = 40, 36, 6
    dirs = default_dirs(nz)
    L = up.Lattice3D((0, 0, (nx - 1) * 0.4 + 1e-6, (ny - 1) * 0.4 + 1e-6), 0.4, nz,
                     preferred_layer_directions=dirs)
    g = L.build_graph(0.7, allow_any_layer_via=True, min_via_center_spacing=0.4)
    R = up.ROIExtractor(g, lattice=L)
    rng = np.random.default_rng(11)
    cases = []
    for i in range(8):
        s = int(rng.integers(0, nx * ny))
        d = int(rng.integers(0, nx * ny))
        bonus = [0.0, 0.6, 3.0, 9.6][i % 4]
        if i == 5:
            R.max_roi_nodes = 3000          # exercise truncation
        else:
            R.max_roi_nodes = 50_000
        roi, g2r = R.extract_roi(s, d, stagnation_bonus=bonus)
        cases.append([s, d, bonus, int(R.max_roi_nodes)])
        roi_out[f"roi{i}"] = np.asarray(roi, dtype=np.int32)
    meta["roi_cases"] = cases
    meta["roi_lattice"] = [nx, ny, nz]
    np.savez_compressed(os.path.join(HERE, "roi.npz"), **roi_out)

    # ----------------------------------------------------------------- A7 SSSP
    sssp = {}
    S = up.SimpleDijkstra(g, L)
    E = len(g.indices)
    scases = []
    for i in range(10):
        rng = np.random.default_rng(1300 + i)
        costs = (0.12 + rng.random(E) * 0.05).astype(np.float32)
        if i % 3 == 1:
            costs = (0.12 + rng.integers(0, 4, size=E) * 0.01).astype(np.float32)   # many ties
        if i % 5 == 4:
            costs[rng.choice(E, size=E // 20, replace=False)] = np.float32("inf")
        s = int(rng.integers(0, nx * ny))
        d = int(rng.integers(0, nx * ny))
        R.max_roi_nodes = 50_000
        roi, g2r = R.extract_roi(s, d, stagnation_bonus=0.0)
        pen = None
        if i % 2 == 0:
            pen = (rng.integers(0, 3, size=len(roi)) * 0.5 * (i + 1)).astype(np.float32)
        path = S.find_path_roi(s, d, costs, roi, g2r, node_penalty=pen)
        sssp[f"s{i}_path"] = np.asarray(path if path else [], dtype=np.int32)
        scases.append([s, d])
    meta["sssp_cases"] = scases
    np.savez_compressed(os.path.join(HERE, "sssp.npz"), **sssp)

    # ------------------------------------------------------------ full runs
    runs = {}
    for tag, (nx, ny, nz, n_nets, iters, seed) in {
        "r0": (24, 24, 6, 24, 6, 101),
        "r1": (28, 24, 8, 36, 8, 202),
    }.items():
        cfg = up.PathFinderConfig()
        cfg.use_gpu = False
        cfg.portal_enabled = False
        cfg.max_iterations = iters
        cfg.preferred_layer_directions = default_dirs(nz)
        router = up.PathFinderRouter(config=cfg, use_gpu=False)
        router.initialize_graph(make_board(Board, Component, Coordinate, Net, Pad, nx, ny, nz))
        assert (router.lattice.x_steps, router.lattice.y_steps) == (nx, ny)
        reqs = seeded_two_pin_nets(nx, ny, nz, n_nets, seed, dmin=4, dmax=40)
        per_iter = []
        trace = []
        orig_find = router.solver.find_path_roi
        orig_hist = router.accounting.update_history

        def find_hook(src, dst, costs, roi_nodes, global_to_roi, node_penalty=None):
            p = orig_find(src, dst, costs, roi_nodes, global_to_roi, node_penalty=node_penalty)
            if len(trace) < (10 if tag == "r0" else 0):
                trace.append(dict(src=src, dst=dst, costs=np.array(costs, copy=True),
                                  roi=np.array(roi_nodes, dtype=np.int32, copy=True),
                                  pen=None if node_penalty is None else np.array(node_penalty, copy=True),
                                  path=list(p) if p else []))
            return p

        def hist_hook(*a, **k):
            r = orig_hist(*a, **k)
            per_iter.append(dict(
                it=router.iteration,
                paths={k_: list(v) for k_, v in router.net_paths.items()},
                barrel=int(getattr(router, "_last_barrel_conflict_count", 0)),
                node_over=int(getattr(router, "_last_path_node_overuse_total", 0)),
                present_sha=sha(router.accounting.present),
                history_sha=sha(router.accounting.history),
            ))
            return r

        router.solver.find_path_roi = find_hook
        router.accounting.update_history = hist_hook
        res = router.route_multiple_nets(reqs)
        runs[f"{tag}_reqs"] = np.asarray([[int(r[0][1:]), r[1], r[2]] for r in reqs], dtype=np.int64)
        for j, pi in enumerate(per_iter):
            flat = []
            for name in sorted(pi["paths"], key=lambda s: int(s[1:])):
                p = pi["paths"][name]
                flat.append(len(p))
                flat.extend(p)
            runs[f"{tag}_it{j}_paths"] = np.asarray(flat, dtype=np.int64)
        for j, t in enumerate(trace):
            runs[f"{tag}_t{j}_costs"] = t["costs"]
            runs[f"{tag}_t{j}_roi"] = t["roi"]
            if t["pen"] is not None:
                runs[f"{tag}_t{j}_pen"] = t["pen"]
            runs[f"{tag}_t{j}_path"] = np.asarray(t["path"], dtype=np.int32)
            runs[f"{tag}_t{j}_sd"] = np.asarray([t["src"], t["dst"]], dtype=np.int64)
        meta[tag] = dict(
            nx=nx, ny=ny, nz=nz, n_nets=n_nets, iters=iters, seed=seed,
            n_trace=len(trace),
            per_iter=[dict(it=p["it"], barrel=p["barrel"], node_over=p["node_over"],
                           present_sha=p["present_sha"], history_sha=p["history_sha"]) for p in per_iter],
            metrics=res.get("iteration_metrics", []),
            result={k: res.get(k) for k in ("success", "converged", "overuse_sum", "overuse_edges",
                                            "barrel_conflicts", "failed_nets", "iterations",
                                            "path_node_overuse_sum", "best_iteration")},
            final_paths_sha=sha(np.asarray(
                [x for name in sorted(router.net_paths, key=lambda s: int(s[1:]))
                 for x in [len(router.net_paths[name])] + list(router.net_paths[name])], dtype=np.int64)),
        )
        for m in meta[tag]["metrics"]:
            m.pop("iter_time_s", None)
            m.pop("total_time_s", None)
    np.savez_compressed(os.path.join(HERE, "runs.npz"), **runs)

    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
