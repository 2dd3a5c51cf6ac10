"""The allocation-free search entry point, ``ogr_find_path_noalloc``.

It serves hosts that cannot give the library a device workspace (a plugin
living inside an application that owns the GPU allocator, or a serving
process that fixes its memory budget at start-up).  Its scratch is a fixed
array inside the library, so this test checks, through the C ABI, that two
calls in a row return exactly the paths of the workspace-based
``ogr_find_path`` on the same inputs, and that a lattice above the array's
node limit is refused before anything runs.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup():
    import torch
    from orthoroute_gb300 import Lattice, _lib
    from orthoroute_gb300.device import DeviceGraph, DeviceState, Ops
    g = DeviceGraph(Lattice(48, 40, 6))
    s = DeviceState(g)
    ops = Ops(g, s)
    rng = np.random.default_rng(2024)
    costs = (0.12 + rng.random(g.E) * 0.05).astype(np.float32)
    s.total_cost.copy_(torch.from_numpy(costs))
    hist = (rng.integers(0, 3, size=g.N) * 0.5).astype(np.float32)
    s.node_history.copy_(torch.from_numpy(hist))
    return torch, _lib, g, s, ops, rng


def test_noalloc_matches_workspace_search_twice():
    torch, _lib, g, s, ops, rng = _setup()
    lib = _lib.load()
    plane = 48 * 40
    out = torch.empty(g.N, dtype=torch.int32, device=g.device)
    for call in range(2):                      # two calls in a row share the array
        src, dst = (int(v) for v in rng.integers(0, plane, size=2))
        net = ops.net_args(3, src, dst, max_depth=80, halo=2, pres_fac=1.5, penalty=True)
        want = ops.find_path(net)
        n = C.c_int32(0)
        rc = lib.ogr_find_path_noalloc(C.byref(g.cgraph()), C.byref(s.cstate()), C.byref(net), out.data_ptr(),
                                       g.N, C.byref(n), None, None)
        assert rc in (_lib.OGR_OK, _lib.OGR_NO_PATH), rc
        got = out[: n.value].cpu().tolist() if rc == _lib.OGR_OK and n.value > 1 else None
        assert got == want, f"call {call}"


def test_noalloc_rejects_lattices_above_its_limit():
    import torch
    from orthoroute_gb300 import _lib
    lib = _lib.load()
    N = _lib.OGR_NOALLOC_MAX_NODES + 1
    g = _lib.Graph(N, 1, 1, N, 0, None, None, None, None)
    st = _lib.State()
    net = _lib.NetArgs(0, 0, 1, 0, 10, 2, 75000.0, 50000, 0.0, 0.0, 0.0, 0)
    n = C.c_int32(0)
    dummy = torch.empty(4, dtype=torch.int32, device="cuda")
    assert lib.ogr_find_path_noalloc(C.byref(g), C.byref(st), C.byref(net), dummy.data_ptr(), 4, C.byref(n),
                                     None, None) == _lib.OGR_ERR_CAPACITY
