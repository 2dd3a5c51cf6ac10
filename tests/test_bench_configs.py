"""The bench's seeded workloads have the shapes their descriptions state (CPU)."""
import numpy as np
import pytest

import bench


def _coords(n, nx):
    return n % nx, n // nx


@pytest.mark.parametrize("name", ["c0", "c1"])
def test_two_pin_workloads(name):
    cfg = bench.CONFIGS[name]
    reqs = bench.make_requests(cfg)
    nx, ny = cfg["nx"], cfg["ny"]
    assert len(reqs) == cfg["nets"] and len({r[0] for r in reqs}) == len(reqs)
    for _, s, d in reqs:
        assert 0 <= s < nx * ny and 0 <= d < nx * ny and s != d       # endpoints on layer 0
    if name == "c0":
        dist = [abs(s % nx - d % nx) + abs(s // nx - d // nx) for _, s, d in reqs]
        assert 5 <= min(dist) and max(dist) <= 80
    assert bench.make_requests(cfg) == reqs                            # seeded


def test_multipin_workload():
    cfg = bench.CONFIGS["c2"]
    reqs = bench.make_requests(cfg)
    nets = {r[0].split("#")[0] for r in reqs}
    assert len(nets) == cfg["nets"] and len(reqs) == 4135


def test_bga_backplane_workload():
    cfg = bench.CONFIGS["c3"]
    nx, ny = cfg["nx"], cfg["ny"]
    conn = bench.connector_pins(nx, ny)
    assert len(conn) == 8000 and len(set(conn)) == 8000
    for p in conn:
        x, y = _coords(p, nx)
        assert x < 3 or x >= nx - 3 or y < 2 or y >= ny - 2               # on the board's edge bands
    reqs = bench.make_requests(cfg)
    assert len(reqs) == 4800
    pins = [s for _, s, _ in reqs] + [d for _, _, d in reqs]
    assert len(set(pins)) == len(pins) == 9600                          # every pin used once
    balls = [s for n, s, _ in reqs if n.startswith("B")]
    assert len(balls) == 1600
    xs = np.array([_coords(b, nx)[0] for b in balls])
    ys = np.array([_coords(b, nx)[1] for b in balls])
    assert abs(xs.mean() - nx / 2) < 2 and abs(ys.mean() - ny / 2) < 2  # centred 40x40 field
    assert xs.max() - xs.min() == pytest.approx(39 * 2.5, abs=1)
