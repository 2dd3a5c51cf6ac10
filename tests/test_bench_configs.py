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


def test_cpu_sample_scales_by_measured_counts_or_a_lower_bound():
    """The CPU baseline's job time = time per sampled search x the job's
    searches + policy time per iteration; the count is the oracle's own (the
    committed trajectory), else this GPU run's, else only the first
    iteration's searches (every net once), which can only understate it."""
    cs = object.__new__(bench.CpuSample)
    cs.small = False
    cs.timed_search_s, cs.timed_searches, cs.policy_s = 10.0, 20, 2.0
    cs.name, cs.cfg, cs.tasks = "c1", bench.CONFIGS["c1"], {f"N{i}": (0, 1) for i in range(2000)}
    fx = bench.trajectory_fixture("c1")
    assert fx is not None
    v, desc = cs.estimate()
    assert v == pytest.approx(0.5 * fx["searches"] + 2.0 * fx["result"]["iterations"])
    assert "oracle's own run" in desc
    cs.name, cs.cfg, cs.tasks = "c3", bench.CONFIGS["c3"], {f"N{i}": (0, 1) for i in range(4800)}
    v, desc = cs.estimate(gpu_counts=(7000, 2))
    assert v == pytest.approx(0.5 * 7000 + 2.0 * 2) and "GPU run" in desc
    v, desc = cs.estimate()
    assert v == pytest.approx(0.5 * 4800 + 2.0 * bench.CONFIGS["c3"]["iters"]) and "lower bound" in desc
