"""Multi-pin nets as star two-pin requests (host logic, no GPU)."""
import numpy as np

from orthoroute_gb300.multipin import group_paths, net_of, seeded_multipin_nets, star_requests


def test_star_requests_keep_two_pin_nets_and_name_sinks():
    reqs = star_requests([("A", [5, 9]), ("B", [1, 2, 3, 2, 1]), ("C", [4]), ("D#x", [7, 8, 9])])
    assert reqs == [("A", 5, 9), ("B", 1, 2), ("B#2", 1, 3), ("B#3", 1, 1), ("D#x", 7, 8), ("D#x#2", 7, 9)]
    assert [net_of(n) for n, _, _ in reqs] == ["A", "B", "B", "B", "D#x", "D#x"]


def test_group_paths_follows_request_order():
    paths = {"B": [1, 2], "A": [5, 6], "B#2": [1, 3], "B#3": [1]}
    assert group_paths(paths) == {"B": [[1, 2], [1, 3], [1]], "A": [[5, 6]]}


def test_seeded_multipin_nets_shape():
    nx, ny = 600, 400
    nets = seeded_multipin_nets(nx, ny, 1500, 2468)
    k = np.array([len(p) for _, p in nets])
    assert k.min() >= 2 and k.max() <= 16 and 3.0 < k.mean() < 4.5
    for _, pins in nets:
        xs = [p % nx for p in pins]
        ys = [p // nx for p in pins]
        assert max(xs) - min(xs) < 50 and max(ys) - min(ys) < 50
        assert all(0 <= p < nx * ny for p in pins)       # layer 0
    assert nets == seeded_multipin_nets(nx, ny, 1500, 2468)
