"""Multi-pin nets as two-pin requests (star decomposition).

The reference routes only the first two pads of a net
(``_parse_requests``, unified_pathfinder.py:4397-4404;
``board_analyzer.py:67-71``).  This build defines a multi-pin net
``(name, [p0, p1, ..., pk])`` as the k two-pin nets ``p0 -> pi``: the first
keeps the net's name (so a two-pin net is the reference's request
unchanged), the others are named ``name#i``.  They are ordinary tuple
requests, so the reference's negotiation routes them as it routes any
tuple nets and the oracle reproduces every path; the persistent routing
pass searches all sinks of every net in its single launch.  A sink equal
to the source is a trivially routed request, as for any tuple net, and a
repeated sink is dropped.
"""
from __future__ import annotations

from typing import Dict, Iterable, List, Sequence, Tuple

import numpy as np

SEP = "#"


def star_requests(nets: Iterable[Tuple[str, Sequence[int]]]) -> List[Tuple[str, int, int]]:
    """(name, pins) -> [(name, p0, p1), (name#2, p0, p2), ...]."""
    out = []
    for name, pins in nets:
        pins = [int(p) for p in pins]
        if len(pins) < 2:
            continue
        seen = set()
        k = 0
        for p in pins[1:]:
            if p in seen:
                continue
            seen.add(p)
            k += 1
            out.append((name if k == 1 else f"{name}{SEP}{k}", pins[0], p))
    return out


def net_of(request_name: str) -> str:
    """The multi-pin net a request belongs to."""
    base, sep, tail = str(request_name).rpartition(SEP)
    return base if sep and tail.isdigit() else str(request_name)


def group_paths(net_paths: Dict[str, List[int]]) -> Dict[str, List[List[int]]]:
    """Routed sub-net paths per multi-pin net, sinks in request order."""
    out: Dict[str, List[List[int]]] = {}
    for name, path in net_paths.items():
        out.setdefault(net_of(name), []).append(list(path))
    return out


def seeded_multipin_nets(nx: int, ny: int, n: int, seed: int, box: int = 50, p: float = 0.35,
                         max_pins: int = 16) -> List[Tuple[str, List[int]]]:
    """Nets of 2..max_pins pins (1 + geometric(p) pins, clipped), pins uniform
    on layer 0 inside a seeded box x box cell window per net (numpy
    default_rng)."""
    rng = np.random.default_rng(seed)
    nets = []
    for i in range(n):
        k = int(min(max_pins, max(2, 1 + rng.geometric(p))))
        x0 = int(rng.integers(0, max(1, nx - box + 1)))
        y0 = int(rng.integers(0, max(1, ny - box + 1)))
        xs = rng.integers(x0, min(nx, x0 + box), size=k)
        ys = rng.integers(y0, min(ny, y0 + box), size=k)
        nets.append((f"M{i}", [int(y) * nx + int(x) for x, y in zip(xs, ys)]))
    return nets
