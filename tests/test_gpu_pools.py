"""Device via pools and per-net overuse against the oracle on random paths.

* ogr_via_pools_rebuild / ogr_via_pools_presence against oracle.accounting.
  ViaPools (the restatement of _accumulate_via_usage_for_path :4470-4546 and
  the EMA / z prefix :6279-6303): column and segment use, the spatial
  overuse sum, the over-full list, and two EMA steps bit for bit.
* ogr_nets_overuse against numpy sums over each net's arcs.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def rand_paths(rng, nx, ny, nz, n_paths, max_len):
    """Paths of lateral and via hops, with via runs up and down a column and
    columns revisited after a lateral step."""
    plane = nx * ny
    out = []
    for _ in range(n_paths):
        x, y, z = (int(rng.integers(0, nx)), int(rng.integers(0, ny)), int(rng.integers(0, nz)))
        p = [z * plane + y * nx + x]
        for _ in range(int(rng.integers(1, max_len))):
            r = rng.random()
            if r < 0.45:
                z2 = int(rng.integers(0, nz))
                z = z2 if z2 != z else (z + 1) % nz
            elif r < 0.7:
                x = min(nx - 1, max(0, x + int(rng.choice([-1, 1]))))
            else:
                y = min(ny - 1, max(0, y + int(rng.choice([-1, 1]))))
            n = z * plane + y * nx + x
            if n != p[-1]:
                p.append(n)
        out.append(p)
    return out


def store(paths, slot_cap, dev):
    L = torch.zeros(len(paths), dtype=torch.int32)
    P = torch.zeros((len(paths), slot_cap), dtype=torch.int32)
    for k, p in enumerate(paths):
        L[k] = len(p)
        P[k, :len(p)] = torch.tensor(p, dtype=torch.int32)
    return L.to(dev), P.to(dev)


@pytest.mark.parametrize("nx,ny,nz,seed", [(12, 9, 8, 1), (20, 16, 12, 2), (7, 5, 3, 3), (16, 12, 2, 4)])
def test_device_via_pools_match_oracle(nx, ny, nz, seed):
    from oracle.accounting import ViaPools
    from orthoroute_gb300 import _lib
    lib = _lib.load()
    dev = "cuda"
    rng = np.random.default_rng(seed)
    segZ = max(0, nz - 2)
    ref = ViaPools(nx, ny, nz)
    col_cap = torch.from_numpy(ref.col_cap).to(dev)
    seg_cap = torch.from_numpy(ref.seg_cap).to(dev) if segZ else None
    col_use = torch.zeros((nx, ny), dtype=torch.int16, device=dev)
    seg_use = torch.zeros((nx, ny, max(segZ, 1)), dtype=torch.int16, device=dev)
    col_pres = torch.zeros((nx, ny), dtype=torch.float32, device=dev)
    seg_pres = torch.zeros((nx, ny, max(segZ, 1)), dtype=torch.float32, device=dev)
    seg_prefix = torch.zeros_like(seg_pres)
    scratch = torch.zeros(nx * ny * (1 + segZ), dtype=torch.int32, device=dev)
    spatial = torch.zeros(1, dtype=torch.int64, device=dev)
    over = torch.zeros(5 * 8192, dtype=torch.int32, device=dev)
    over_n = torch.zeros(1, dtype=torch.int32, device=dev)
    for step in range(2):
        paths = rand_paths(rng, nx, ny, nz, 60, 40)
        L, P = store(paths, 64, dev)
        rc = lib.ogr_via_pools_rebuild(L.data_ptr(), P.data_ptr(), len(paths), 64, nx, ny, nz, scratch.data_ptr(),
                                       col_use.data_ptr(), seg_use.data_ptr() if segZ else None, col_cap.data_ptr(),
                                       seg_cap.data_ptr() if segZ else None, spatial.data_ptr(), over.data_ptr(),
                                       8192, over_n.data_ptr(), None)
        assert rc == _lib.OGR_OK
        rc = lib.ogr_via_pools_presence(nx, ny, nz, col_use.data_ptr(), col_cap.data_ptr(),
                                        seg_use.data_ptr() if segZ else None, seg_cap.data_ptr() if segZ else None,
                                        col_pres.data_ptr(), seg_pres.data_ptr() if segZ else None,
                                        seg_prefix.data_ptr() if segZ else None, None)
        assert rc == _lib.OGR_OK
        ref.rebuild(paths)
        ref.update_presence()
        np.testing.assert_array_equal(col_use.cpu().numpy(), ref.col_use)
        assert int(spatial.item()) == ref.spatial_overuse_total()
        n = int(over_n.item())
        got = {tuple(r) for r in over[:5 * n].view(n, 5).cpu().numpy().tolist()}
        want = {(0, x, y, 0, int(ref.col_use[x, y])) for x, y in zip(*np.nonzero(ref.col_use > ref.col_cap))}
        np.testing.assert_array_equal(col_pres.cpu().numpy(), ref.col_pres)
        if segZ:
            np.testing.assert_array_equal(seg_use.cpu().numpy(), ref.seg_use)
            want |= {(1, x, y, s, int(ref.seg_use[x, y, s]))
                     for x, y, s in zip(*np.nonzero(ref.seg_use > ref.seg_cap))}
            np.testing.assert_array_equal(seg_pres.cpu().numpy(), ref.seg_pres)
            np.testing.assert_array_equal(seg_prefix.cpu().numpy(), ref.seg_prefix)
        assert got == want, step


@pytest.mark.parametrize("canonical", [0, 1])
def test_nets_overuse_matches_numpy(canonical):
    from orthoroute_gb300 import _lib
    lib = _lib.load()
    dev = "cuda"
    rng = np.random.default_rng(7 + canonical)
    E, K, cap = 5000, 300, 40
    present = rng.integers(0, 4, size=E).astype(np.float32)
    capacity = np.ones(E, dtype=np.float32)
    src = rng.integers(0, 900, size=E).astype(np.int32)
    dst = rng.integers(0, 900, size=E).astype(np.int32)
    lens = rng.integers(0, cap // 2 + 1, size=K).astype(np.int32)
    arcs = np.zeros((K, cap), dtype=np.int32)
    for k in range(K):
        na = 2 * (lens[k] - 1) if lens[k] >= 2 else 0
        arcs[k, :na] = rng.integers(0, E, size=na)
    # the device copies must outlive the asynchronous launch: keep them named
    d = {k: torch.from_numpy(v).to(dev) for k, v in dict(lens=lens, arcs=arcs, present=present, capacity=capacity,
                                                          src=src, dst=dst).items()}
    sums = torch.zeros(K, dtype=torch.float64, device=dev)
    hit = torch.zeros(K, dtype=torch.uint8, device=dev)
    rc = lib.ogr_nets_overuse(d["lens"].data_ptr(), d["arcs"].data_ptr(), K, cap, d["present"].data_ptr(),
                              d["capacity"].data_ptr(), d["src"].data_ptr(), d["dst"].data_ptr(), canonical,
                              sums.data_ptr(), hit.data_ptr(), None)
    assert rc == _lib.OGR_OK
    torch.cuda.synchronize()
    over = np.maximum(0, present - capacity).astype(np.float64)
    for k in range(K):
        na = 2 * (lens[k] - 1) if lens[k] >= 2 else 0
        a = arcs[k, :na]
        if canonical:
            a = a[src[a] < dst[a]]
        assert sums[k].item() == over[a].sum()
        assert bool(hit[k].item()) == bool((over[a] > 0).any())


@pytest.mark.parametrize("canonical", [0, 1])
def test_per_net_overuse_after_restore_reads_restored_arcs(canonical):
    """A best-state restore re-commits every path in one launch
    (ogr_paths_commit).  The per-net overuse the stagnation rip-up ranks by
    (ogr_nets_overuse over the path store's arcs) must then be that of the
    restored paths, not of the paths the store held before."""
    from orthoroute_gb300 import Lattice
    from orthoroute_gb300.router import PathFinderConfig, PathFinderRouter
    nx, ny, nz = 40, 30, 4
    rng = np.random.default_rng(11)
    reqs = []
    while len(reqs) < 90:
        x0, x1 = rng.integers(5, 35, size=2)
        y0, y1 = rng.integers(5, 25, size=2)
        if abs(int(x1) - int(x0)) + abs(int(y1) - int(y0)) >= 6:
            reqs.append((f"N{len(reqs)}", int(y0) * nx + int(x0), int(y1) * nx + int(x1)))
    R = PathFinderRouter(PathFinderConfig(max_iterations=1), mode="persistent", full_engine="grid")
    R.initialize_lattice(Lattice(nx, ny, nz))
    R.route_multiple_nets(reqs)
    first = R._capture()
    R.config = PathFinderConfig(max_iterations=4)
    R.route_multiple_nets(reqs)
    later = R._capture()
    assert any(first.get(n) != later.get(n) for n in later), "the states must differ for the check to bite"
    R._restore(first)
    names, sums, hit = R._edge_over_device(canonical)
    src = R.g.edge_src.cpu().numpy().astype(np.int64)
    dst = R.g.indices.cpu().numpy().astype(np.int64)
    arc_of = {(int(a), int(b)): e for e, (a, b) in enumerate(zip(src, dst))}
    over = np.maximum(0.0, R.s.present.cpu().numpy() - R.s.capacity.cpu().numpy()).astype(np.float64)
    assert over.sum() > 0
    got = dict(zip(names, zip(sums.tolist(), hit.tolist())))
    assert set(got) == {n for n, p in first.items() if p and len(p) >= 2}
    for n, (s_, h_) in got.items():
        p = first[n]
        arcs = [arc_of[(u, v)] for u, v in zip(p[:-1], p[1:])] + [arc_of[(v, u)] for u, v in zip(p[:-1], p[1:])]
        if canonical:
            arcs = [e for e in arcs if src[e] < dst[e]]
        assert s_ == float(over[arcs].sum()), n
        assert bool(h_) == bool((over[arcs] > 0).any()), n
