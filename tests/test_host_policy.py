"""Host-side policy helpers of the router (no GPU): the vectorised via-pool
membership and usage, barrel node expansion, barrel ownership and conflicts,
shared path nodes and per-net overuse sums agree with the per-hop loops they
replace (the reference's own formulation, as the oracle restates it)."""
from collections import defaultdict
from types import SimpleNamespace

import numpy as np
import pytest
import torch

from orthoroute_gb300 import router as R
from oracle.accounting import ViaPools as OracleViaPools
from oracle.tallies import NodeState, detect_barrel_conflicts


class _Host:
    """Just the attributes the helpers read."""


def _host(nx=9, ny=7, nz=8, seg_z=6):
    h = _Host()
    h.nx, h.ny, h.nz, h.plane = nx, ny, nz, nx * ny
    h.pools = type("Pools", (), {"segZ": seg_z})()
    return h


def _rand_path(rng, h, n):
    p = [int(rng.integers(0, h.plane * h.nz))]
    for _ in range(n):
        z, r = divmod(p[-1], h.plane)
        if rng.random() < 0.4:
            z2 = int(rng.integers(0, h.nz))
            p.append((z2 if z2 != z else (z + 1) % h.nz) * h.plane + r)
        else:
            p.append(z * h.plane + (r + 1) % h.plane)
    return p


def _coord(h, n):
    z, r = divmod(int(n), h.plane)
    y, x = divmod(r, h.nx)
    return x, y, z


def _router(nx=9, ny=7, nz=8):
    """A router object with the host state only (no device)."""
    h = object.__new__(R.PathFinderRouter)
    h.nx, h.ny, h.nz, h.plane, h.N = nx, ny, nz, nx * ny, nx * ny * nz
    h.config = R.PathFinderConfig()
    h.pools = R._ViaPools(nx, ny, nz)
    h.node_use = np.zeros(h.N, dtype=np.int16)
    h._via_owner = np.full(h.N, -1, dtype=np.int64)
    h._via_owner_set = np.zeros(0, dtype=np.int64)
    h.node_history = np.zeros(h.N, dtype=np.float32)
    h._hist_iter = None
    h._hist_mask = np.zeros(h.N, dtype=bool)
    h._flat_view = None
    h.net_paths = {}
    h.net_to_edges = {}
    h._eidx = None
    h.net_id_map = {}
    h.iteration = 1
    h.s = SimpleNamespace(node_history=torch.zeros(h.N, dtype=torch.float32))
    h.g = SimpleNamespace(device="cpu")
    h._reset_policy_state()
    return h


def _walk(rng, h, n, box):
    """A simple path (no repeated node) of lateral steps and via hops in a small box."""
    x, y = int(rng.integers(0, box)), int(rng.integers(0, box))
    z = int(rng.integers(0, h.nz))
    p, seen = [z * h.plane + y * h.nx + x], set()
    seen.add(p[0])
    for _ in range(n):
        for _try in range(8):
            if rng.random() < 0.35:
                z2 = int(rng.integers(0, h.nz))
                if z2 == z:
                    continue
                cand = (x, y, z2)
            else:
                dx, dy = [(1, 0), (-1, 0), (0, 1), (0, -1)][int(rng.integers(0, 4))]
                cand = (min(max(x + dx, 0), box - 1), min(max(y + dy, 0), box - 1), z)
            node = cand[2] * h.plane + cand[1] * h.nx + cand[0]
            if node not in seen:
                break
        else:
            break
        x, y, z = cand
        seen.add(node)
        p.append(node)
    return p


def _routed(seed, nets=40, box=5):
    rng = np.random.default_rng(seed)
    h = _router()
    paths = {}
    for i in range(nets):
        p = _walk(rng, h, int(rng.integers(0, 25)), box)
        # empty (failed) nets, and one-node paths: trivially routed nets (src == dst)
        paths[f"N{(i * 7) % nets}"] = [] if i % 9 == 0 else (p[:1] if i % 11 == 3 else p)
    arcs_src, arcs_dst, edges = [], [], {}
    for name, p in paths.items():
        h._net_id(name)
        if len(p) >= 2:
            h._mark_nodes(name, p, +1)
            ids = []
            for u, v in list(zip(p, p[1:])) + list(zip(p[::-1], p[::-1][1:])):
                ids.append(len(arcs_src))
                arcs_src.append(u)
                arcs_dst.append(v)
            edges[name] = ids
        h.net_paths[name] = p
    return h, paths, np.asarray(arcs_src, dtype=np.int64), np.asarray(arcs_dst, dtype=np.int64), edges


@pytest.mark.parametrize("seed", range(6))
def test_barrel_conflicts_match_oracle_loops(seed):
    h, paths, esrc, edst, edges = _routed(seed)
    ns = NodeState(h.N, h.nx, h.plane)
    ns.rebuild_owner([(h.net_id_map[n], p) for n, p in paths.items()])
    for p in paths.values():          # commits mark node use; trivially routed nets are never committed
        if len(p) >= 2:
            ns.mark_use(p)
    assert any(len(p) == 1 for p in paths.values())
    np.testing.assert_array_equal(h.node_use, ns.path_node_use)
    for rep in range(2):          # the second call sees this iteration's history marks
        got = h._detect_barrels()
        want, info = detect_barrel_conflicts(esrc, edst, ns, paths, edges, h.net_id_map, h.iteration)
        assert got == want
        assert info["exact"] > 0 and info["path_node"] > 0
        assert h.barrel_victim_nets == info["victim_nets"]
        assert h.barrel_owner_nets == info["owner_nets"]
        assert h.barrel_conflict_nets == info["conflict_nets"]
        assert h.exact_pairs == info["exact_pairs"]
        assert h.path_node_pairs == info["path_node_pairs"]
        assert h.path_node_scores == info["path_node_scores"]
        assert dict(h.physical_scores) == dict(info["scores"])
        np.testing.assert_array_equal(h.node_history, ns.node_history)
        np.testing.assert_array_equal(h.s.node_history.numpy(), ns.node_history)
        own = h._via_owner_of(h._flat())
        np.testing.assert_array_equal(own, ns.owner)
    # rip up some nets and reroute others: the flat view follows every change
    for name in list(paths)[:10]:
        if paths[name]:
            h._mark_nodes(name, paths[name], -1)
            ns.clear_use(paths[name])
        h.net_paths[name] = []
        paths[name] = []
    h.iteration = 2
    ns.rebuild_owner([(h.net_id_map[n], p) for n, p in paths.items()])
    got = h._detect_barrels()
    want, info = detect_barrel_conflicts(esrc, edst, ns, paths, edges, h.net_id_map, 2)
    assert got == want and h.exact_pairs == info["exact_pairs"]
    assert dict(h.physical_scores) == dict(info["scores"])
    np.testing.assert_array_equal(h._via_owner_of(h._flat()), ns.owner)
    np.testing.assert_array_equal(h.node_history, ns.node_history)


@pytest.mark.parametrize("seed", range(4))
def test_via_usage_rebuild_matches_oracle_loop(seed):
    h, paths, *_ = _routed(seed, nets=60, box=6)
    h._rebuild_via_usage()
    ref = OracleViaPools(h.nx, h.ny, h.nz)
    ref.rebuild(list(paths.values()))
    assert ref.col_use.sum() > 0 and ref.seg_use.sum() > 0
    np.testing.assert_array_equal(h.pools.col_use, ref.col_use)
    np.testing.assert_array_equal(h.pools.seg_use, ref.seg_use)


def test_path_dict_versions_and_arrays():
    d = R._PathDict({"a": [1, 2]})
    v = d.version
    d["b"] = [3, 4, 5]
    assert d.version > v and d.array("b").tolist() == [3, 4, 5]
    d.set_path("b", [6, 7], np.asarray([6, 7], dtype=np.int64))
    assert d.array("b").tolist() == [6, 7]
    for op in (lambda: d.update({"c": [1, 2]}), lambda: d.pop("c"), lambda: d.setdefault("e", [8, 9]),
               lambda: d.__delitem__("e"), d.clear):
        v = d.version
        op()
        assert d.version > v
    assert d.array("a").size == 0
    h = _router()
    h.net_paths = {"x": [0, h.plane, 2 * h.plane]}
    assert isinstance(h.net_paths, R._PathDict)
    f = h._flat()
    assert f.names == ["x"] and f.hops.tolist() == [0, 1] and h._flat() is f
    h.net_paths["y"] = [5, 6]
    assert h._flat() is not f and h._flat().names == ["x", "y"]


@pytest.mark.parametrize("seed", range(4))
def test_via_pool_members_match_hop_loop(seed):
    rng = np.random.default_rng(seed)
    h = _router()
    h.net_paths = {f"N{i}": _rand_path(rng, h, int(rng.integers(1, 30))) for i in range(40)}
    h.net_paths["N5"] = []
    col_over = rng.random((h.nx, h.ny)) < 0.3
    seg_over = rng.random((h.nx, h.ny, h.pools.segZ)) < 0.3
    got = R.PathFinderRouter._via_pool_members(h, col_over, seg_over)
    want = defaultdict(set)
    for name, path in h.net_paths.items():
        if not path or len(path) < 2:
            continue
        res = set()
        for u, v in zip(path, path[1:]):
            xu, yu, zu = _coord(h, u)
            xv, yv, zv = _coord(h, v)
            if xu != xv or yu != yv or zu == zv:
                continue
            if col_over[xu, yu]:
                res.add(("col", xu, yu))
            zl = max(1, min(min(zu, zv), h.nz - 2))
            zh = max(1, min(max(zu, zv), h.nz - 2))
            for z in range(zl, zh):
                if 0 <= z - 1 < h.pools.segZ and seg_over[xu, yu, z - 1]:
                    res.add(("seg", xu, yu, z - 1))
        for r in res:
            want[r].add(name)
    assert dict(got) == dict(want)


def test_via_members_match_hop_loop():
    """Every node spanned by a net's via hops, with the net's id (the flat view)."""
    from oracle.tallies import via_nodes_for_path
    rng = np.random.default_rng(7)
    h = _router()
    want = set()
    for i in range(50):
        path = _rand_path(rng, h, int(rng.integers(0, 25)))
        name = f"N{i}"
        h.net_paths[name] = path if len(path) >= 2 else []
        if len(path) >= 2:
            nid = h._net_id(name)
            want |= {(n, nid) for n in via_nodes_for_path(path, h.nx, h.plane)}
    vn, vid = h._flat().via_members()
    assert set(zip(vn.tolist(), vid.tolist())) == want
    assert np.all(np.diff(vn) >= 0)


def test_edge_over_sums_match_generator_sums():
    rng = np.random.default_rng(3)
    h = _host()
    h.E = 500
    h._eidx = None
    h.net_to_edges = {f"N{i}": rng.integers(0, 500, size=int(rng.integers(0, 40))).astype(np.int64)
                      for i in range(30)}
    h._edge_index = lambda: R.PathFinderRouter._edge_index(h)
    over_idx = np.unique(rng.integers(0, 500, size=60)).astype(np.int64)
    over_val = (rng.random(over_idx.size).astype(np.float32) * 3).astype(np.float64)
    over_map = dict(zip(over_idx.tolist(), over_val.tolist()))
    names, sums, hit = R.PathFinderRouter._edge_over(h, over_idx, over_val)
    again = R.PathFinderRouter._edge_over(h, over_idx, over_val)
    assert again[0] is names and again[1] is sums                          # reused while nothing changed
    assert not h._over_mask.any() and not h._over_dense.any()              # scratch left clean
    for i, n in enumerate(names):
        edges = h.net_to_edges[n].tolist()
        assert sums[i] == sum(float(over_map[e]) for e in edges if e in over_map)
        assert sums[i] == sum(float(over_map.get(e, 0.0)) for e in edges)
        assert bool(hit[i]) == any(e in over_map for e in edges)


def test_parse_requests_like_the_reference():
    """``_parse_requests`` (:4386-4467) for tuples: src == dst is a trivially
    routed one-node path and no task; non-int endpoints are skipped; nets
    given by pads raise; and a request list without a task gives the
    reference's NO-ROUTABLE-NETS result."""
    h = _router()
    tasks = h._parse_requests([("A", 3, 9), ("B", 4, 4), ("C", np.int64(1), 2), ("D", 1.0, 2), ("E", 5, 7, 1)])
    assert tasks == {"A": (3, 9)}
    assert h.net_paths == {"B": [4]}
    with pytest.raises(TypeError):
        h._parse_requests([SimpleNamespace(name="N", pads=[1, 2])])
    assert R.PathFinderRouter._no_routable_nets([]) == {}
    res = R.PathFinderRouter._no_routable_nets([("X", 2, 2), ("Y", 1.5, 3)])
    assert res["error_code"] == "NO-ROUTABLE-NETS" and res["excluded_net_ids"] == ["X", "Y"]
    assert res["total_nets"] == 2 and not res["success"]


def _scan_lists(h, paths, task_names):
    """What ogr_barrel_scan returns for these stored paths (its semantics in
    numpy): conflicting hops; (endpoint, net id) per conflicting endpoint;
    (node, owner count, owner xor) per distinct conflict node; (node, net id)
    of the via hops spanning a conflict node owned by several nets; (node,
    slot) per stored-path node used more than once."""
    cnt = np.zeros(h.N, dtype=np.int64)
    xr = np.zeros(h.N, dtype=np.int64)
    spans = {}
    for n in task_names:
        p = paths[n]
        if len(p) < 2:
            continue
        nid = h.net_id_map[n]
        nodes = set()
        for u, v in zip(p, p[1:]):
            zu, ru = divmod(u, h.plane)
            zv, rv = divmod(v, h.plane)
            if ru == rv and zu != zv:
                nodes.update(z * h.plane + ru for z in range(min(zu, zv), max(zu, zv) + 1))
        spans[n] = nodes
        for nd in nodes:
            cnt[nd] += 1
            xr[nd] ^= nid
    owner = np.where(cnt == 0, -1, np.where(cnt == 1, xr, -2))
    exact, occ, cnodes, seen = 0, [], [], set()
    for n in task_names:
        p = paths[n]
        if len(p) < 2:
            continue
        en = h.net_id_map[n]
        for u, v in zip(p, p[1:]):
            sc = owner[u] != -1 and owner[u] != en
            dc = owner[v] != -1 and owner[v] != en
            exact += int(sc or dc)
            for x, c in ((u, sc), (v, dc)):
                if c:
                    occ.append((x, en))
                    if x not in seen:
                        seen.add(x)
                        cnodes.append((x, int(cnt[x]), int(xr[x])))
    members = [(nd, h.net_id_map[n]) for n in task_names if len(paths[n]) >= 2
               for nd in spans[n] if nd in seen and cnt[nd] >= 2]
    shared = [(x, k) for k, n in enumerate(task_names) if len(paths[n]) >= 2
              for x in paths[n] if h.node_use[x] > 1]
    arr = lambda rows, w: np.asarray(rows, dtype=np.int64).reshape(-1, w)
    return exact, arr(occ, 2), arr(cnodes, 3), arr(members, 2), arr(shared, 2)


@pytest.mark.parametrize("seed", range(4))
def test_barrel_lists_from_the_device_give_the_host_result(seed):
    """_detect_barrels's persistent-mode branch (the device scan's lists, then
    sorts on the host) against its flat-view branch and the oracle's loops."""
    h, paths, esrc, edst, edges = _routed(seed)
    task_names = [n for n, p in paths.items() if len(p) != 1]   # one-node nets are routed trivially
    h._task_names = task_names
    lists = _scan_lists(h, paths, task_names)
    assert lists[0] > 0 and len(lists[3]) > 0 and len(lists[4]) > 0
    results = []
    for device in (False, True):
        h._hist_mask.fill(False)
        h._hist_iter = None
        h.node_history.fill(0)
        h.s.node_history.zero_()
        h.store = object() if device else None
        if device:
            h._barrel_scan = lambda: lists
        got = h._detect_barrels()
        results.append((got, set(h.barrel_victim_nets), set(h.barrel_owner_nets), set(h.barrel_conflict_nets),
                        set(h.exact_pairs), set(h.path_node_pairs), dict(h.path_node_scores),
                        dict(h.physical_scores), h.node_history.copy()))
    host, dev = results
    for a, b in zip(host, dev):
        if isinstance(a, np.ndarray):
            np.testing.assert_array_equal(a, b)
        else:
            assert a == b
    ns = NodeState(h.N, h.nx, h.plane)
    ns.rebuild_owner([(h.net_id_map[n], p) for n, p in paths.items()])
    for p in paths.values():
        if len(p) >= 2:
            ns.mark_use(p)
    want, info = detect_barrel_conflicts(esrc, edst, ns, paths, edges, h.net_id_map, h.iteration)
    assert dev[0] == want and dev[4] == info["exact_pairs"] and dev[3] == info["conflict_nets"]


def test_batched_node_use_marks_equal_per_path_marks():
    """The pass epilogue marks every old path off and every new path on in one
    batch each; a path's distinct nodes count once, as _mark_nodes counts them."""
    rng = np.random.default_rng(5)
    a, b = _router(), _router()
    paths = [rng.integers(0, a.N, size=int(rng.integers(1, 40))).astype(np.int64) for _ in range(50)]
    paths.append(np.asarray([3, 3, 7, 3], dtype=np.int64))          # repeated nodes count once
    for p in paths:
        a._mark_nodes("x", None, +1, p)
    b._mark_many(paths, +1)
    np.testing.assert_array_equal(a.node_use, b.node_use)
    off = paths[::3]
    for p in off:
        a._mark_nodes("x", None, -1, p)
    b._mark_many(off, -1)
    np.testing.assert_array_equal(a.node_use, b.node_use)
    assert a.node_use.min() >= 0 and a.node_use.sum() > 0


def test_net_table_cache_equals_the_per_pass_loop():
    """The per-net search parameters (_net_table, extract_roi :2240-2255): the
    cached and vectorised table equals the per-net formula for every
    stagnation bonus, and net ids keep their first-use order (this pass's
    order first, then task order)."""
    rng = np.random.default_rng(8)
    h = _router(nx=300, ny=200, nz=4)
    names = [f"N{i}" for i in range(60)]
    h._tasks_all = {n: (int(rng.integers(0, h.plane)), int(rng.integers(0, h.plane))) for n in names}
    h._task_names = list(names)
    h._table_cache = None
    ordered = names[::-1][:20]                      # this pass routes 20 nets, in reverse order
    for n in ordered:
        h._net_id(n)
    for bonus in (0.0, 0.0, 0.6, 3.0, 0.6):
        t = h._net_table(bonus)
        for i, n in enumerate(names):
            s_, d_ = h._tasks_all[n]
            dist = h._manhattan(s_, d_)
            assert int(t["src"][i]) == s_ and int(t["dst"][i]) == d_
            assert int(t["full"][i]) == (1 if dist >= R.ROI_THRESHOLD_STEPS else 0) == int(t["full_host"][i])
            assert int(t["id"][i]) == h.net_id_map[n]
            for j, b in enumerate((bonus, bonus * 2)):
                radius = max(60, int(dist * 0.75 + b * 2.0))
                assert int(t["depth"][2 * i + j]) == min(int(radius + b * 2.0), 80)
                assert int(t["halo"][2 * i + j]) == min(16, 2 + int(max(0.0, b) / 0.6))
    # ids: the pass's nets in its order, then the rest in task order
    want = {n: k for k, n in enumerate(ordered)}
    for n in names:
        want.setdefault(n, len(want))
    assert h.net_id_map == want
