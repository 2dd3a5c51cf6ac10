"""ctypes binding of ``include/orthoroute_gb300.h``.

The library is built in-tree by ``orthoroute_gb300._build``.  There is no CPU
fallback: if the shared library is missing or a CUDA device is absent, the
routing entry points raise.
"""
from __future__ import annotations

import contextlib
import ctypes as C
import os

from . import _build

OGR_OK = 0
OGR_NO_PATH = 1
OGR_ERR_ARG = -1
OGR_ERR_CUDA = -2
OGR_ERR_CAPACITY = -3
OGR_ERR_ITER_CAP = -4
OGR_ERR_NUMERIC = -5
OGR_ERR_TIMEOUT = -6
OGR_NOALLOC_MAX_NODES = 262144
ERRORS = {-1: "bad argument", -2: "CUDA error", -3: "buffer capacity exceeded",
          -4: "device loop iteration limit reached", -5: "exactness precondition violated",
          -6: "grid barrier timed out"}

EXPORTED = [
    "ogr_csr_num_edges", "ogr_csr_workspace_bytes", "ogr_csr_build",
    "ogr_costs_update", "ogr_live_begin", "ogr_present_ema", "ogr_history_update",
    "ogr_tally", "ogr_route_workspace_bytes", "ogr_route_workspace_init",
    "ogr_find_path", "ogr_path_apply", "ogr_extract_roi", "ogr_via_pools_apply", "ogr_overused_arcs",
    "ogr_find_path_noalloc", "ogr_route_pass", "ogr_search_profile", "ogr_bfs_workspace_bytes",
    "ogr_bfs_workspace_init", "ogr_full_workspace_bytes", "ogr_find_path_full",
    "ogr_full_profile", "ogr_full_workspace_init", "ogr_find_path_roi", "ogr_reverse_costs",
    "ogr_window_workspace_bytes", "ogr_window_workspace_init", "ogr_window_ctl_bytes",
    "ogr_multi_workspace_bytes", "ogr_find_path_multi", "ogr_full_grid", "ogr_search_lanes",
    "ogr_paths_commit", "ogr_full_lanes", "ogr_full_reuse", "ogr_window_lookahead",
    "ogr_full_tile", "ogr_tile_profile", "ogr_debug_limits", "ogr_nets_overuse",
    "ogr_via_pools_rebuild", "ogr_via_pools_presence", "ogr_barrel_scan", "ogr_find_path_full_multi",
]

P = C.c_void_p
I32 = C.c_int32
I64 = C.c_int64
F32 = C.c_float


class LatticeDesc(C.Structure):
    _fields_ = [("nx", I32), ("ny", I32), ("nz", I32), ("lateral_cost", F32), ("wrong_way_cost", F32),
                ("layer_axis", P), ("partner_ptr", P), ("partner_z", P), ("partner_cost", P),
                ("partner_site", P)]


class CostArgs(C.Structure):
    _fields_ = [("num_edges", I64), ("base_costs", P), ("edge_layer", P), ("edge_kind", P),
                ("present_ema", P), ("capacity", P), ("history", P), ("blocked", P), ("layer_bias", P),
                ("via_cost_multiplier", F32), ("base_cost_weight", F32), ("pres_fac", F32),
                ("hist_weight", F32), ("add_jitter", I32)]


class Graph(C.Structure):
    _fields_ = [("nx", I32), ("ny", I32), ("nz", I32), ("num_nodes", I32), ("num_edges", I64),
                ("indptr", P), ("indices", P), ("rev", P), ("blocked", P)]


class State(C.Structure):
    _fields_ = [("total_cost", P), ("live_static", P), ("present", P), ("capacity", P), ("layer_bias", P),
                ("edge_layer", P), ("edge_kind", P), ("path_node_use", P), ("owner_count", P),
                ("owner_xor", P), ("node_history", P), ("rcost", P)]


class NetArgs(C.Structure):
    _fields_ = [("net_id", I32), ("src", I32), ("dst", I32), ("full_graph", I32), ("bfs_max_depth", I32),
                ("bfs_halo", I32), ("bfs_stop_count", C.c_double), ("max_roi_nodes", I32),
                ("owner_weight", F32), ("path_weight", F32), ("history_weight", F32),
                ("penalty_enabled", I32)]


class NetTable(C.Structure):
    _fields_ = [("num_nets", I32), ("slot_cap", I32), ("store_len", P), ("store_path", P), ("store_arcs", P),
                ("net_src", P), ("net_dst", P), ("net_id", P), ("net_full", P), ("net_depth", P), ("net_halo", P)]


class PassArgs(C.Structure):
    _fields_ = [("order", P), ("count", I32), ("fallback_quota", I32), ("max_roi_nodes", I32),
                ("bfs_stop_count", C.c_double), ("owner_weight", F32), ("path_weight", F32),
                ("history_weight", F32), ("penalty_enabled", I32), ("pres_fac", F32), ("live", I32),
                ("net_status", P), ("stats", P)]


class RoiBatch(C.Structure):
    _fields_ = [("slots", I32), ("slot_bytes", C.c_size_t), ("qcap", I64), ("bfs_ws", P), ("roi_pool", P),
                ("roi_len", P), ("roi_cap", I32), ("next", P), ("roi_box", P)]


class WindowArgs(C.Structure):
    _fields_ = [("slots", I32), ("slot_bytes", C.c_size_t), ("ws", P), ("scratch", P), ("ctl", P),
                ("discarded", P)]


_LIB = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the shared library (building it first if it is absent)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing; run orthoroute_gb300._build.build()")
        _build.build()
    lib = C.CDLL(path)
    sig = {
        "ogr_csr_num_edges": [C.POINTER(LatticeDesc), C.POINTER(I64)],
        "ogr_csr_workspace_bytes": [C.POINTER(LatticeDesc)],
        "ogr_csr_build": [C.POINTER(LatticeDesc), P, P, P, P, P, P, P, P, C.c_size_t, P],
        "ogr_costs_update": [C.POINTER(CostArgs), P, P],
        "ogr_live_begin": [C.POINTER(CostArgs), P, P, P, P],
        "ogr_present_ema": [I64, P, P, F32, F32, P],
        "ogr_history_update": [I64, P, P, P, P, P, F32, F32, F32, I32, P],
        "ogr_tally": [I64, I32, I32, P, P, P, P, P, P, P, I32, P, P, P],
        "ogr_route_workspace_bytes": [I32],
        "ogr_route_workspace_init": [P, C.c_size_t, I32, P],
        "ogr_find_path": [C.POINTER(Graph), C.POINTER(State), C.POINTER(NetArgs), P, C.c_size_t, P, I32,
                          C.POINTER(I32), P, P],
        "ogr_path_apply": [C.POINTER(Graph), C.POINTER(State), P, I32, I32, I32, F32, I32, P, P, P],
        "ogr_extract_roi": [C.POINTER(Graph), C.POINTER(NetArgs), P, C.c_size_t, P, I32, C.POINTER(I32), P],
        "ogr_via_pools_apply": [I64, I32, I32, I32, P, P, P, P, P, P, P, P, P, P, F32, F32, F32, I32, I32, P, P],
        "ogr_overused_arcs": [I64, P, P, P, P, I32, P, P],
        "ogr_find_path_noalloc": [C.POINTER(Graph), C.POINTER(State), C.POINTER(NetArgs), P, I32,
                                  C.POINTER(I32), P, P],
        "ogr_search_profile": [P, I32],
        "ogr_route_pass": [C.POINTER(Graph), C.POINTER(State), C.POINTER(NetTable), C.POINTER(PassArgs),
                           C.POINTER(RoiBatch), P, C.c_size_t, P, P, C.c_size_t, C.POINTER(WindowArgs),
                           C.POINTER(I32), P],
        "ogr_window_workspace_bytes": [I32, I32, I32],
        "ogr_window_workspace_init": [P, I32, I32, I32, P],
        "ogr_window_ctl_bytes": [I32],
        "ogr_full_workspace_bytes": [I32, I64],
        "ogr_find_path_roi": [C.POINTER(Graph), P, P, I32, P, I32, I32, P, C.c_size_t, P, I32, C.POINTER(I32), P, P],
        "ogr_multi_workspace_bytes": [I32],
        "ogr_full_grid": [I32, C.POINTER(I32), C.POINTER(I32)],
        "ogr_search_lanes": [I32, C.POINTER(I32)],
        "ogr_full_lanes": [I32, C.POINTER(I32)],
        "ogr_full_reuse": [I32, C.POINTER(I32)],
        "ogr_window_lookahead": [I32, C.POINTER(I32)],
        "ogr_paths_commit": [C.POINTER(Graph), C.POINTER(State), P, P, P, I32, P, P, P, P, P, I32, P, P],
        "ogr_find_path_multi": [C.POINTER(Graph), P, P, I32, P, P, P, I32, P, P, I32, P, C.c_size_t, P, I32,
                                C.POINTER(I32), P, P],
        "ogr_full_profile": [P, I32],
        "ogr_full_tile": [I32, C.c_double, I32, I32, C.POINTER(I32), C.POINTER(C.c_double)],
        "ogr_tile_profile": [P, I32],
        "ogr_debug_limits": [I32, I32, C.POINTER(I32), C.POINTER(I32)],
        "ogr_nets_overuse": [P, P, I32, I64, P, P, P, P, I32, P, P, P],
        "ogr_via_pools_rebuild": [P, P, I32, I64, I32, I32, I32, P, P, P, P, P, P, P, I32, P, P],
        "ogr_via_pools_presence": [I32, I32, I32, P, P, P, P, P, P, P, P],
        "ogr_barrel_scan": [P, P, P, I32, I64, I32, I32, P, P, P, P, I32, I64, P, P, P, P, P, P],
        "ogr_reverse_costs": [I64, P, P, P, P],
        "ogr_full_workspace_init": [P, C.c_size_t, I32, I64, P],
        "ogr_find_path_full": [C.POINTER(Graph), C.POINTER(State), C.POINTER(NetArgs), P, C.c_size_t, P, I32,
                               C.POINTER(I32), P, P],
        "ogr_find_path_full_multi": [C.POINTER(Graph), C.POINTER(State), C.POINTER(NetArgs), P, P, I32, P, P, I32,
                                     P, C.c_size_t, P, I32, C.POINTER(I32), P, P],
        "ogr_bfs_workspace_bytes": [I32, I64, I32],
        "ogr_bfs_workspace_init": [P, I32, I64, I32, P],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_size_t if name.endswith("_bytes") else C.c_int
    _LIB = lib
    return lib


@contextlib.contextmanager
def inject_fault(name: str, rc: int):
    """Test hook for failure handling: inside the block, calls of the entry
    point `name` return the status `rc` without running (a stand-in for a
    device or driver failure reported by that call)."""
    lib = load()
    real = getattr(lib, name)

    def fake(*_args, **_kw):
        return rc
    setattr(lib, name, fake)
    try:
        yield
    finally:
        setattr(lib, name, real)


def debug_limits(barrier_spin: int = -1, max_phases: int = -1):
    """Set (>= 0) or read (-1) the whole-lattice search's failure-test limits
    (ogr_debug_limits): (barrier spin, phase cap), 0 = default."""
    a, b = C.c_int32(0), C.c_int32(0)
    check(load().ogr_debug_limits(int(barrier_spin), int(max_phases), C.byref(a), C.byref(b)), "ogr_debug_limits")
    return int(a.value), int(b.value)


def check(rc: int, what: str) -> int:
    if rc < 0:
        raise RuntimeError(f"{what} failed: {ERRORS.get(rc, rc)} ({rc})")
    return rc
