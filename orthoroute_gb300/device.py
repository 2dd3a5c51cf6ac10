"""Device-resident lattice and congestion state, and thin wrappers over the C ABI.

PyTorch tensors provide the device memory; every computation on them is a
hand-written kernel in ``csrc/``.  Arrays (E arcs, N nodes):

* CSR: indptr int32[N+1], indices int32[E], base_costs f32[E],
  edge_layer u8[E], edge_kind u8[E], edge_src int32[E], rev int32[E]
* accounting: present, present_ema, history, capacity, total_cost,
  live_static f32[E]; layer_bias f32[Nz]
* nodes: path_node_use, owner_count, owner_xor int32[N], node_history f32[N]
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _lib
from .lattice import Lattice


def _p(t: Optional[torch.Tensor]) -> Optional[int]:
    return None if t is None else t.data_ptr()


def _stream_ptr(stream: Optional[torch.cuda.Stream]) -> Optional[int]:
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("orthoroute_gb300 needs a CUDA device (GB300, sm_103a); there is no CPU path")


class DeviceGraph:
    """CSR lattice built on the device by ``ogr_csr_build``."""

    def __init__(self, lattice: Lattice, device="cuda", stream=None):
        require_cuda()
        self.lib = _lib.load()
        self.lattice = lattice
        self.device = torch.device(device)
        desc, keep = lattice.descriptor()
        E = C.c_int64(0)
        _lib.check(self.lib.ogr_csr_num_edges(C.byref(desc), C.byref(E)), "ogr_csr_num_edges")
        self.E = int(E.value)
        self.N = lattice.num_nodes
        dev = self.device
        self.indptr = torch.empty(self.N + 1, dtype=torch.int32, device=dev)
        self.indices = torch.empty(self.E, dtype=torch.int32, device=dev)
        self.base_costs = torch.empty(self.E, dtype=torch.float32, device=dev)
        self.edge_layer = torch.empty(self.E, dtype=torch.uint8, device=dev)
        self.edge_kind = torch.empty(self.E, dtype=torch.uint8, device=dev)
        self.edge_src = torch.empty(self.E, dtype=torch.int32, device=dev)
        self.rev = torch.empty(self.E, dtype=torch.int32, device=dev)
        ws_bytes = int(self.lib.ogr_csr_workspace_bytes(C.byref(desc)))
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
        _lib.check(self.lib.ogr_csr_build(C.byref(desc), _p(self.indptr), _p(self.indices), _p(self.base_costs),
                                          _p(self.edge_layer), _p(self.edge_kind), _p(self.edge_src),
                                          _p(self.rev), _p(ws), ws_bytes, _stream_ptr(stream)),
                   "ogr_csr_build")
        self.blocked = None
        del keep

    def cgraph(self) -> _lib.Graph:
        L = self.lattice
        return _lib.Graph(L.nx, L.ny, L.nz, self.N, self.E, _p(self.indptr), _p(self.indices), _p(self.rev),
                          _p(self.blocked))


class DeviceState:
    """Congestion state of one routing job (EdgeAccountant + node maps)."""

    def __init__(self, graph: DeviceGraph):
        self.g = graph
        dev, E, N = graph.device, graph.E, graph.N
        self.present = torch.zeros(E, dtype=torch.float32, device=dev)
        self.present_ema = torch.zeros(E, dtype=torch.float32, device=dev)
        self.history = torch.zeros(E, dtype=torch.float32, device=dev)
        self.capacity = torch.ones(E, dtype=torch.float32, device=dev)
        self.total_cost = torch.zeros(E, dtype=torch.float32, device=dev)
        self.live_static = torch.zeros(E, dtype=torch.float32, device=dev)
        self.layer_bias = torch.ones(graph.lattice.nz, dtype=torch.float32, device=dev)
        self.use_layer_bias = False
        self.path_node_use = torch.zeros(N, dtype=torch.int32, device=dev)
        self.owner_count = torch.zeros(N, dtype=torch.int32, device=dev)
        self.owner_xor = torch.zeros(N, dtype=torch.int32, device=dev)
        self.node_history = torch.zeros(N, dtype=torch.float32, device=dev)
        self.rcost = None   # reverse costs, kept in sync once enabled (see enable_rcost)

    def enable_rcost(self):
        """Keep rcost[e] = total_cost[rev[e]] in HBM: the searches then read the
        cost into each row's node directly.  Every writer of total_cost must be
        followed by Ops.sync_rcost (the path-apply kernels keep it in sync)."""
        if self.rcost is None:
            self.rcost = torch.empty_like(self.total_cost)

    def cstate(self) -> _lib.State:
        g = self.g
        return _lib.State(_p(self.total_cost), _p(self.live_static), _p(self.present), _p(self.capacity),
                          _p(self.layer_bias) if self.use_layer_bias else None, _p(g.edge_layer), _p(g.edge_kind),
                          _p(self.path_node_use), _p(self.owner_count), _p(self.owner_xor), _p(self.node_history),
                          _p(self.rcost))

    def cost_args(self, pres_fac, hist_weight, via_mult, base_weight, add_jitter=True) -> _lib.CostArgs:
        g = self.g
        return _lib.CostArgs(g.E, _p(g.base_costs), _p(g.edge_layer), _p(g.edge_kind), _p(self.present_ema),
                             _p(self.capacity), _p(self.history), _p(g.blocked),
                             _p(self.layer_bias) if self.use_layer_bias else None,
                             float(np.float32(via_mult)), float(np.float32(base_weight)),
                             float(np.float32(pres_fac)), float(np.float32(hist_weight)), int(bool(add_jitter)))


class Ops:
    """Typed wrappers over the kernels for one graph / state pair."""

    def __init__(self, graph: DeviceGraph, state: DeviceState, slots: int = 1, stream=None):
        self.g, self.s = graph, state
        self.lib = graph.lib
        self.stream = stream
        self.ws_bytes = int(self.lib.ogr_route_workspace_bytes(graph.N))
        self.ws = [torch.empty(self.ws_bytes, dtype=torch.uint8, device=graph.device) for _ in range(slots)]
        for w in self.ws:
            _lib.check(self.lib.ogr_route_workspace_init(_p(w), self.ws_bytes, graph.N, self._sp()),
                       "ogr_route_workspace_init")
        self.path_buf = torch.empty(max(graph.N, 2), dtype=torch.int32, device=graph.device)
        self.stats = torch.zeros(4, dtype=torch.int64, device=graph.device)
        # {searches, arcs, pops} of window searches whose results were undone
        self.discarded = torch.zeros(3, dtype=torch.int64, device=graph.device)
        self.status = torch.zeros(1, dtype=torch.int32, device=graph.device)
        self.tally_out = torch.zeros(5, dtype=torch.int64, device=graph.device)
        self.layer_units = torch.zeros(graph.lattice.nz, dtype=torch.int64, device=graph.device)
        self.counters = dict(launches=0, h2d_bytes=0, d2h_bytes=0, search_launches=0, search_ms=0.0)
        self._full_ws = None
        self.full_ws_bytes = 0
        self._ev0 = torch.cuda.Event(enable_timing=True)
        self._ev1 = torch.cuda.Event(enable_timing=True)

    def reset_counters(self):
        for k in self.counters:
            self.counters[k] = 0.0 if k == "search_ms" else 0

    def _sp(self):
        return _stream_ptr(self.stream)

    # -- A2–A4 ----------------------------------------------------------------
    def update_costs(self, pres_fac, hist_weight, via_mult, base_weight, layer_bias: Optional[np.ndarray]):
        s = self.s
        s.use_layer_bias = layer_bias is not None
        if layer_bias is not None:
            s.layer_bias.copy_(torch.from_numpy(np.asarray(layer_bias, dtype=np.float32)))
        a = s.cost_args(pres_fac, hist_weight, via_mult, base_weight)
        _lib.check(self.lib.ogr_costs_update(C.byref(a), _p(s.total_cost), self._sp()), "ogr_costs_update")
        self.counters["launches"] += 1
        self.sync_rcost()
        if layer_bias is not None:
            self.counters["h2d_bytes"] += 4 * len(layer_bias)

    def live_begin(self, pres_fac):
        s = self.s
        a = s.cost_args(pres_fac, 0.0, 1.0, 1.0)
        _lib.check(self.lib.ogr_live_begin(C.byref(a), _p(s.present), _p(s.total_cost), _p(s.live_static),
                                           self._sp()), "ogr_live_begin")
        self.counters["launches"] += 1
        self.sync_rcost()

    def sync_rcost(self):
        """Re-derive the reverse costs after a full-array change of total_cost."""
        s, g = self.s, self.g
        if s.rcost is None:
            return
        _lib.check(self.lib.ogr_reverse_costs(g.E, _p(g.rev), _p(s.total_cost), _p(s.rcost), self._sp()),
                   "ogr_reverse_costs")
        self.counters["launches"] += 1

    def present_ema(self, beta=0.40):
        s = self.s
        _lib.check(self.lib.ogr_present_ema(self.g.E, _p(s.present), _p(s.present_ema), float(np.float32(beta)),
                                            float(np.float32(1.0 - beta)), self._sp()), "ogr_present_ema")
        self.counters["launches"] += 1

    def update_history(self, gain, cap_mult=15.0, decay=1.0, use_cap=True, use_raw_present=True):
        s = self.s
        _lib.check(self.lib.ogr_history_update(self.g.E, _p(s.history), _p(s.present), _p(s.present_ema),
                                               _p(s.capacity), _p(self.g.base_costs) if use_cap else None,
                                               float(np.float32(gain)), float(np.float32(cap_mult)),
                                               float(np.float32(decay)), int(use_raw_present), self._sp()),
                   "ogr_history_update")
        self.counters["launches"] += 1

    def tally(self, canonical_only=True):
        """Returns (over_sum, over_cnt, node_over_sum, node_over_cnt, layer_units[nz])."""
        s, g = self.s, self.g
        _lib.check(self.lib.ogr_tally(g.E, g.N, g.lattice.nz, _p(s.present), _p(s.present_ema), _p(s.capacity),
                                      _p(g.edge_src), _p(g.indices), _p(g.edge_layer), _p(s.path_node_use),
                                      int(canonical_only), _p(self.tally_out), _p(self.layer_units), self._sp()),
                   "ogr_tally")
        out = self.tally_out.cpu().numpy()
        self.counters["launches"] += 1
        self.counters["d2h_bytes"] += 8 * (5 + g.lattice.nz)
        if out[4]:
            raise RuntimeError("present EMA off the 2^-23 grid: per-layer sums would not be exact")
        return int(out[0]), int(out[1]), int(out[2]), int(out[3]), self.layer_units.cpu().numpy()

    # -- A6–A8 ----------------------------------------------------------------
    def net_args(self, net_id, src, dst, *, full_graph=False, max_depth=80, halo=2, max_roi_nodes=50_000,
                 pres_fac=1.0, owner_base=25.0, path_base=25.0, hist_pen=5.0, freeze_weight=None,
                 penalty=True) -> _lib.NetArgs:
        w = float(owner_base) * float(pres_fac)
        if freeze_weight is not None:
            w = max(w, float(freeze_weight))
        return _lib.NetArgs(int(net_id), int(src), int(dst), int(bool(full_graph)), int(max_depth), int(halo),
                            float(max_roi_nodes) * 1.5, int(max_roi_nodes), float(np.float32(w)),
                            float(np.float32(float(path_base) * float(pres_fac))), float(np.float32(hist_pen)),
                            int(bool(penalty)))

    def full_workspace(self) -> torch.Tensor:
        """Workspace of the whole-lattice search (allocated on first use)."""
        if self._full_ws is None:
            self.full_ws_bytes = int(self.lib.ogr_full_workspace_bytes(self.g.N, self.g.E))
            self._full_ws = torch.empty(self.full_ws_bytes, dtype=torch.uint8, device=self.g.device)
            _lib.check(self.lib.ogr_full_workspace_init(_p(self._full_ws), self.full_ws_bytes, self.g.N, self.g.E,
                                                        self._sp()), "ogr_full_workspace_init")
        return self._full_ws

    def find_path(self, net: _lib.NetArgs, slot: int = 0, engine: str = "auto") -> Optional[List[int]]:
        """Search one net.  engine: "grid" = whole-lattice search on all SMs
        (full-graph nets), "cta" = one CTA, "auto" = grid for full-graph nets."""
        g = self.g.cgraph()
        st = self.s.cstate()
        n = C.c_int32(0)
        stream = self.stream if self.stream is not None else torch.cuda.current_stream()
        grid = engine == "grid" or (engine == "auto" and bool(net.full_graph))
        if grid:
            ws = self.full_workspace()
        self._ev0.record(stream)
        if grid:
            rc = self.lib.ogr_find_path_full(C.byref(g), C.byref(st), C.byref(net), _p(ws), self.full_ws_bytes,
                                             _p(self.path_buf), int(self.path_buf.numel()), C.byref(n),
                                             _p(self.stats), self._sp())
        else:
            rc = self.lib.ogr_find_path(C.byref(g), C.byref(st), C.byref(net), _p(self.ws[slot]), self.ws_bytes,
                                        _p(self.path_buf), int(self.path_buf.numel()), C.byref(n),
                                        _p(self.stats), self._sp())
        self._ev1.record(stream)
        _lib.check(rc, "ogr_find_path_full" if grid else "ogr_find_path")
        self._ev1.synchronize()
        self.counters["search_ms"] += self._ev0.elapsed_time(self._ev1)
        self.counters["search_launches"] += 1
        self.counters["launches"] += 1
        self.counters["d2h_bytes"] += 16 + 4 * max(0, n.value)
        if rc == _lib.OGR_NO_PATH or n.value < 2:
            return None
        return self.path_buf[: n.value].cpu().tolist()

    def find_path_given_roi(self, src: int, dst: int, costs: torch.Tensor, roi_nodes, roi_penalty=None,
                            slot: int = 0) -> Optional[List[int]]:
        """``SimpleDijkstra.find_path_roi`` seam: search a caller-given ROI with
        caller-given arc costs (device f32[E]) and ROI-local penalties."""
        dev = self.g.device
        roi = torch.as_tensor(np.asarray(roi_nodes, dtype=np.int32)).to(dev)
        pen = None if roi_penalty is None else torch.as_tensor(np.asarray(roi_penalty, dtype=np.float32)).to(dev)
        g = self.g.cgraph()
        n = C.c_int32(0)
        rc = self.lib.ogr_find_path_roi(C.byref(g), _p(costs), _p(roi), int(roi.numel()), _p(pen), int(src),
                                        int(dst), _p(self.ws[slot]), self.ws_bytes, _p(self.path_buf),
                                        int(self.path_buf.numel()), C.byref(n), _p(self.stats), self._sp())
        _lib.check(rc, "ogr_find_path_roi")
        self.counters["launches"] += 1
        if rc == _lib.OGR_NO_PATH or n.value < 2:
            return None
        return self.path_buf[: n.value].cpu().tolist()

    def multi_workspace(self) -> torch.Tensor:
        """Scratch of the multi-source search (allocated on first use)."""
        if getattr(self, "_multi_ws", None) is None:
            self.multi_ws_bytes = int(self.lib.ogr_multi_workspace_bytes(self.g.N))
            self._multi_ws = torch.empty(self.multi_ws_bytes, dtype=torch.uint8, device=self.g.device)
            _lib.check(self.lib.ogr_route_workspace_init(_p(self._multi_ws), self.multi_ws_bytes, self.g.N,
                                                         self._sp()), "ogr_route_workspace_init")
        return self._multi_ws

    def find_path_multi(self, src_seeds, dst_targets, costs: torch.Tensor, roi_nodes, roi_penalty=None):
        """``SimpleDijkstra.find_path_multisource_multisink`` seam: seeds and
        targets are ``(global node, cost)`` pairs; a repeated target keeps its
        last cost (the reference builds a dict).  Returns ``(path,
        entry_layer, exit_layer)`` or None."""
        dev = self.g.device
        tg = dict((int(n), float(c)) for n, c in dst_targets)
        seeds = [(int(n), float(c)) for n, c in src_seeds]
        if len({n for n, _ in seeds}) != len(seeds):
            raise ValueError("repeated seed node")
        if not seeds or not tg:
            return None
        roi = torch.as_tensor(np.asarray(roi_nodes, dtype=np.int32)).to(dev)
        pen = None if roi_penalty is None else torch.as_tensor(np.asarray(roi_penalty, dtype=np.float32)).to(dev)
        sd = torch.as_tensor(np.asarray([n for n, _ in seeds], dtype=np.int32)).to(dev)
        sc = torch.as_tensor(np.asarray([c for _, c in seeds], dtype=np.float64)).to(dev)
        td = torch.as_tensor(np.asarray(list(tg), dtype=np.int32)).to(dev)
        tc = torch.as_tensor(np.asarray(list(tg.values()), dtype=np.float64)).to(dev)
        ws = self.multi_workspace()
        g = self.g.cgraph()
        n = C.c_int32(0)
        rc = self.lib.ogr_find_path_multi(C.byref(g), _p(costs), _p(roi), int(roi.numel()), _p(pen), _p(sd), _p(sc),
                                          int(sd.numel()), _p(td), _p(tc), int(td.numel()), _p(ws),
                                          self.multi_ws_bytes, _p(self.path_buf), int(self.path_buf.numel()),
                                          C.byref(n), _p(self.stats), self._sp())
        _lib.check(rc, "ogr_find_path_multi")
        self.counters["launches"] += 1
        if rc == _lib.OGR_NO_PATH or n.value < 2:
            return None
        path = self.path_buf[: n.value].cpu().tolist()
        plane = self.g.lattice.plane
        return path, path[0] // plane, path[-1] // plane

    def find_path_full_multi(self, src_seeds, dst_targets, net: _lib.NetArgs):
        """Whole-lattice multi-source multi-sink search (ogr_find_path_full_multi)
        on the state's costs and node penalty: seeds and targets are
        ``(global node, cost)`` pairs; a repeated target keeps its last cost
        (the reference builds a dict).  Returns ``(path, entry_layer,
        exit_layer)`` or None."""
        dev = self.g.device
        tg = dict((int(n), float(c)) for n, c in dst_targets)
        seeds = [(int(n), float(c)) for n, c in src_seeds]
        if len({n for n, _ in seeds}) != len(seeds):
            raise ValueError("repeated seed node")
        if not seeds or not tg:
            return None
        sd = torch.as_tensor(np.asarray([n for n, _ in seeds], dtype=np.int32)).to(dev)
        sc = torch.as_tensor(np.asarray([c for _, c in seeds], dtype=np.float64)).to(dev)
        td = torch.as_tensor(np.asarray(list(tg), dtype=np.int32)).to(dev)
        tc = torch.as_tensor(np.asarray(list(tg.values()), dtype=np.float64)).to(dev)
        ws = self.full_workspace()
        g = self.g.cgraph()
        st = self.s.cstate()
        n = C.c_int32(0)
        rc = self.lib.ogr_find_path_full_multi(C.byref(g), C.byref(st), C.byref(net), _p(sd), _p(sc), int(sd.numel()),
                                               _p(td), _p(tc), int(td.numel()), _p(ws), self.full_ws_bytes,
                                               _p(self.path_buf), int(self.path_buf.numel()), C.byref(n),
                                               _p(self.stats), self._sp())
        _lib.check(rc, "ogr_find_path_full_multi")
        self.counters["launches"] += 1
        self.counters["search_launches"] += 1
        self.counters["h2d_bytes"] += 12 * (len(seeds) + len(tg))
        self.counters["d2h_bytes"] += 16 + 4 * max(0, n.value)
        if rc == _lib.OGR_NO_PATH or n.value < 2:
            return None
        path = self.path_buf[: n.value].cpu().tolist()
        plane = self.g.lattice.plane
        return path, path[0] // plane, path[-1] // plane

    def extract_roi(self, net: _lib.NetArgs, slot: int = 0) -> np.ndarray:
        g = self.g.cgraph()
        out = torch.empty(self.g.N, dtype=torch.int32, device=self.g.device)
        n = C.c_int32(0)
        _lib.check(self.lib.ogr_extract_roi(C.byref(g), C.byref(net), _p(self.ws[slot]), self.ws_bytes, _p(out),
                                            self.g.N, C.byref(n), self._sp()), "ogr_extract_roi")
        return out[: n.value].cpu().numpy()

    def commit_paths(self, paths: Sequence[np.ndarray], net_ids: Sequence[int], store: "PathStore" = None,
                     slots: Optional[Sequence[int]] = None) -> List[np.ndarray]:
        """Commit many paths (>= 2 nodes each) in one launch, no live refresh
        (a best-state restore); optionally into `store` slots.  Returns each
        path's arcs (forward then reverse) as int64 arrays."""
        n = len(paths)
        if n == 0:
            return []
        lens = np.fromiter((len(p) for p in paths), dtype=np.int64, count=n)
        if lens.min() < 2:
            raise ValueError("commit_paths takes paths of two or more nodes")
        off = np.zeros(n + 1, dtype=np.int32)
        off[1:] = np.cumsum(lens)
        flat = np.concatenate([np.asarray(p, dtype=np.int32) for p in paths])
        dev = self.g.device
        d_nodes = torch.from_numpy(flat).to(dev)
        d_off = torch.from_numpy(off).to(dev)
        d_ids = torch.from_numpy(np.asarray(net_ids, dtype=np.int32)).to(dev)
        arcs = torch.empty(int(2 * (lens - 1).sum()), dtype=torch.int32, device=dev)
        d_slots = None if store is None else torch.from_numpy(np.asarray(slots, dtype=np.int32)).to(dev)
        g = self.g.cgraph()
        st = self.s.cstate()
        _lib.check(self.lib.ogr_paths_commit(C.byref(g), C.byref(st), _p(d_nodes), _p(d_off), _p(d_ids), n, _p(arcs),
                                             _p(store.path) if store is not None else None,
                                             _p(store.length) if store is not None else None,
                                             _p(store.arcs) if store is not None else None, _p(d_slots),
                                             store.slot_cap if store is not None else 0, _p(self.status),
                                             self._sp()), "ogr_paths_commit")
        a = arcs.cpu().numpy().astype(np.int64)
        self.counters["launches"] += 1
        self.counters["h2d_bytes"] += flat.nbytes + off.nbytes + 4 * n * (2 if store is not None else 1)
        self.counters["d2h_bytes"] += 4 * a.size + 4
        bad = int(self.status.item())
        if bad:
            raise ValueError("path hop is not a graph edge" if bad == 1 else "path longer than the path-store slot")
        aoff = 2 * (off[:-1].astype(np.int64) - np.arange(n))
        return [a[aoff[k]: aoff[k] + 2 * (lens[k] - 1)] for k in range(n)]

    def apply_path(self, path: Sequence[int], net_id: int, sign: int, pres_fac: float, live: bool = True):
        """Commit (+1) or rip up (-1); returns the arc list (forward then reverse)."""
        L = len(path)
        if L < 2:
            return []
        d = torch.as_tensor(np.asarray(path, dtype=np.int32)).to(self.g.device)
        arcs = torch.empty(2 * (L - 1), dtype=torch.int32, device=self.g.device)
        g = self.g.cgraph()
        st = self.s.cstate()
        _lib.check(self.lib.ogr_path_apply(C.byref(g), C.byref(st), _p(d), L, int(net_id), int(sign),
                                           float(np.float32(pres_fac)), int(bool(live)), _p(arcs),
                                           _p(self.status), self._sp()), "ogr_path_apply")
        out = arcs.cpu().tolist()
        self.counters["launches"] += 1
        self.counters["h2d_bytes"] += 4 * L
        self.counters["d2h_bytes"] += 4 * (2 * (L - 1) + 1)
        if int(self.status.item()) != 0:
            raise ValueError("path hop is not a graph edge")
        return out


class PathStore:
    """Device-resident current path of every net of a job (one fixed slot each),
    plus the per-net ROI pool and BFS slots of the batched ROI extraction."""

    def __init__(self, graph: DeviceGraph, num_nets: int, slot_cap: int = 8192, max_roi_nodes: int = 50_000,
                 bfs_slots: int = 64, window_slots: int = 0):
        dev = graph.device
        lib = graph.lib
        self.num_nets = num_nets
        self.slot_cap = slot_cap
        self.length = torch.zeros(num_nets, dtype=torch.int32, device=dev)
        self.path = torch.zeros((num_nets, slot_cap), dtype=torch.int32, device=dev)
        self.arcs = torch.zeros((num_nets, 2 * slot_cap), dtype=torch.int32, device=dev)
        N = graph.N
        self.roi_cap = int(min(max_roi_nodes, N))
        self.roi_pool = torch.zeros((num_nets, self.roi_cap), dtype=torch.int32, device=dev)
        self.roi_len = torch.zeros(num_nets, dtype=torch.int32, device=dev)
        self.next = torch.zeros(1, dtype=torch.int32, device=dev)
        self.bfs_slots = int(max(1, min(bfs_slots, num_nets)))
        self.qcap = int(min(N, max(4 * max_roi_nodes, 1 << 18)))
        per = int(lib.ogr_bfs_workspace_bytes(N, self.qcap, 1))
        self.slot_bytes = per
        self.bfs_ws = torch.empty(per * self.bfs_slots, dtype=torch.uint8, device=dev)
        _lib.check(lib.ogr_bfs_workspace_init(_p(self.bfs_ws), N, self.qcap, self.bfs_slots, _stream_ptr(None)),
                   "ogr_bfs_workspace_init")
        self.roi_box = torch.zeros(4 * num_nets, dtype=torch.int32, device=dev)
        # batched disjoint-ROI windows: one search slot, scratch path and CTA per window member
        self.window_slots = int(max(0, window_slots))
        if self.window_slots:
            self.win_slot_bytes = int(lib.ogr_window_workspace_bytes(N, max_roi_nodes, 1))
            self.win_ws = torch.empty(self.win_slot_bytes * self.window_slots, dtype=torch.uint8, device=dev)
            _lib.check(lib.ogr_window_workspace_init(_p(self.win_ws), N, max_roi_nodes, self.window_slots,
                                                     _stream_ptr(None)),
                       "ogr_window_workspace_init")
            self.win_scratch = torch.empty((self.window_slots, slot_cap), dtype=torch.int32, device=dev)
            self.win_ctl = torch.empty(int(lib.ogr_window_ctl_bytes(self.window_slots)), dtype=torch.uint8,
                                       device=dev)

    def roi_batch(self) -> _lib.RoiBatch:
        return _lib.RoiBatch(self.bfs_slots, self.slot_bytes, self.qcap, _p(self.bfs_ws), _p(self.roi_pool),
                             _p(self.roi_len), self.roi_cap, _p(self.next), _p(self.roi_box))

    def window_args(self, discarded: Optional[torch.Tensor] = None) -> Optional[_lib.WindowArgs]:
        """discarded: device int64[3] that accumulates {searches, arcs, pops}
        of window searches whose results were undone (those nets are searched
        again)."""
        if not self.window_slots:
            return None
        return _lib.WindowArgs(self.window_slots, self.win_slot_bytes, _p(self.win_ws), _p(self.win_scratch),
                               _p(self.win_ctl), _p(discarded))

    def set_path(self, idx: int, path, arcs=None):
        """Slot idx holds `path` and its arcs (forward then reverse, as the
        commit returned them); an empty or one-node path clears the slot."""
        n = len(path)
        if n > self.slot_cap:
            raise RuntimeError("path longer than the path-store slot")
        if n >= 2:
            if arcs is None or len(arcs) != 2 * (n - 1):
                raise ValueError("a stored path needs its 2 * (len - 1) arcs")
            self.path[idx, :n] = torch.as_tensor(np.asarray(path, dtype=np.int32)).to(self.path.device)
            self.arcs[idx, :len(arcs)] = torch.as_tensor(np.asarray(arcs, dtype=np.int32)).to(self.arcs.device)
        self.length[idx] = n if n >= 2 else 0


def route_pass(ops: "Ops", store: PathStore, table: dict, order: np.ndarray, *, fallback_quota, max_roi_nodes,
               owner_weight, path_weight, history_weight, pres_fac, live, penalty=True, batch_roi=True,
               order_full: Optional[np.ndarray] = None, windows: bool = True):
    """One ``ogr_route_pass`` call; returns (per-net status flags, stats[4]).

    order_full (host, one flag per entry of order) sends the full-graph nets
    to the whole-lattice search; None keeps every net on the single-CTA pass."""
    dev = ops.g.device
    k = len(order)
    if k == 0:
        return np.zeros(0, dtype=np.int32), np.zeros(4, dtype=np.int64)
    d_order = torch.as_tensor(np.asarray(order, dtype=np.int32)).to(dev)
    status = torch.zeros(max(k, 1), dtype=torch.int32, device=dev)
    stats = torch.zeros(4, dtype=torch.int64, device=dev)
    t = _lib.NetTable(store.num_nets, store.slot_cap, _p(store.length), _p(store.path), _p(store.arcs),
                      _p(table["src"]), _p(table["dst"]), _p(table["id"]), _p(table["full"]), _p(table["depth"]),
                      _p(table["halo"]))
    a = _lib.PassArgs(_p(d_order), k, int(fallback_quota), int(max_roi_nodes), float(max_roi_nodes) * 1.5,
                      float(np.float32(owner_weight)), float(np.float32(path_weight)),
                      float(np.float32(history_weight)), int(bool(penalty)), float(np.float32(pres_fac)),
                      int(bool(live)), _p(status), _p(stats))
    g = ops.g.cgraph()
    st = ops.s.cstate()
    rc_dev = C.c_int32(0)
    stream = ops.stream if ops.stream is not None else torch.cuda.current_stream()
    ops._ev0.record(stream)
    rb = store.roi_batch() if batch_roi else None
    full_flags = None
    full_ws, full_bytes = None, 0
    if order_full is not None and np.any(order_full):
        full_flags = np.ascontiguousarray(order_full, dtype=np.uint8)
        full_ws, full_bytes = _p(ops.full_workspace()), ops.full_ws_bytes
    win = store.window_args(ops.discarded) if (batch_roi and windows) else None
    rc = ops.lib.ogr_route_pass(C.byref(g), C.byref(st), C.byref(t), C.byref(a),
                                C.byref(rb) if rb is not None else None, _p(ops.ws[0]), ops.ws_bytes,
                                full_flags.ctypes.data if full_flags is not None else None, full_ws, full_bytes,
                                C.byref(win) if win is not None else None, C.byref(rc_dev), ops._sp())
    ops._ev1.record(stream)
    _lib.check(rc, "ogr_route_pass")
    ops._ev1.synchronize()
    ops.counters["search_ms"] += ops._ev0.elapsed_time(ops._ev1)
    ops.counters["search_launches"] += 1
    n_launch = 1 if rb is not None else 0
    if full_flags is None:
        n_launch += 1
    else:
        runs = int(np.count_nonzero((full_flags[1:] == 0) & (full_flags[:-1] != 0))) + int(full_flags[0] == 0)
        n_launch += runs + 3 * int(np.count_nonzero(full_flags))
    ops.counters["launches"] += n_launch
    ops.counters["h2d_bytes"] += 4 * k
    ops.counters["d2h_bytes"] += 4 * k + 32
    return status[:k].cpu().numpy(), stats.cpu().numpy()
