// A6–A8: per-net ROI extraction, exact ROI shortest path, backtrace, and the
// commit / rip-up scatter.  One CTA (1024 threads) owns one net's search.
//
// ROI (extract_roi_bfs, unified_pathfinder.py:2257-2384): level-synchronous
// bidirectional BFS.  Within one wave step the reference's marks are a set
// function of the frontier (unseen -> wave mark, other wave -> 3 and
// "met"), so claiming nodes with atomicCAS yields the same seen[] array,
// meeting depth and early stop.  The ROI is then compacted in ascending
// global id order (np.where) by scanning the BFS bounding box, and truncated
// to max_roi_nodes with the reference's must-keep swap.  The BFS does not read
// costs, so a routing pass extracts the ROIs of all its nets in parallel on
// many SMs before the sequential part starts (roi_batch_kernel).
//
// Search (SimpleDijkstra.find_path_roi, :2451-2548): the reference pops
// (label, roi_idx) from a heap of FP64 labels, and accepts a relaxation iff
// float32(alt) < dist32[v] (numpy 2 compares a Python float with a float32
// in float32).  Hence every node ends with the FIRST candidate, in pop order
// of its relaxer, that reaches the minimal float32 value; its label is that
// candidate's FP64 alt.  Equivalently, each node takes the lexicographic
// minimum of (float32(alt), L(u), roi_idx(u)) over its relaxers u.
// We settle nodes in phases (IN-criterion): with T = the smallest tentative
// label, a node whose float32 key is below float32((T + cin) + pen) — cin
// being its cheapest in-arc from an unsettled node — can no longer change,
// and nodes whose label equals T are final as in Dijkstra.  Tentative states
// are recomputed by pulling from all settled in-neighbours, which makes the
// result independent of thread scheduling and bit-identical to the heap.
//
// Latency: before the phases, each search gathers an ROI-local adjacency
// (neighbour's ROI index and the in-arc cost, 32 slots per node, one 128-byte
// row) so a phase touches two dependent loads per arc instead of six; a
// 16-lane group handles one node's arcs in parallel; node state is packed in
// one 32-byte sector; the per-group key reduction uses shuffles.
//
// ogr_route_pass runs the reference's per-net sequence (_route_all,
// :7949-8449: rip-up, ROI search, one larger-ROI retry while the pass has
// fallbacks left, commit) for a whole ordered list of nets in one launch,
// with every net's current path kept in a device-resident store.
#include <atomic>

#include "common.cuh"
#include "fullgraph.cuh"

namespace {

constexpr int kThreads = 1024;
constexpr int kWarps = kThreads / 32;
constexpr int kSub = 16;                       // lanes per node (ROI BFS)
constexpr int kGroups = kThreads / kSub;       // nodes in flight per CTA (ROI BFS)
#ifndef OGR_SEARCH_LANES
#define OGR_SEARCH_LANES 4
#endif
constexpr int kSearchLanes = OGR_SEARCH_LANES;  // default lanes per node of the ROI search

// Lanes per node of the ROI search for the launches that follow (set by
// ogr_search_lanes; the autotuner picks it per lattice).  Every searching
// kernel exists for 2, 4, 8 and 16 lanes; results do not depend on the choice.
thread_local int g_search_lanes = kSearchLanes;

// Nets a disjoint-ROI window may skip over to take later disjoint ones
// (ogr_window_lookahead; 0 = consecutive nets only).
thread_local int g_window_look = 8;

#define OGR_WITH_LANES(LV, ...)                                \
  do {                                                         \
    switch (g_search_lanes) {                                  \
      case 2: { constexpr int LV = 2; __VA_ARGS__; } break;    \
      case 8: { constexpr int LV = 8; __VA_ARGS__; } break;    \
      case 16: { constexpr int LV = 16; __VA_ARGS__; } break;  \
      default: { constexpr int LV = 4; __VA_ARGS__; } break;   \
    }                                                          \
  } while (0)
constexpr int32_t ST_NONE = 0, ST_FRONT = 1, ST_DONE = 2, ST_SINK = 3;  // SINK: a settled target (multi-seed)
constexpr int kMaxViaNodes = 4096;
constexpr int kDMax = 32;                      // arcs per node the local adjacency holds
constexpr int kAdjCap = 65536;                 // ROI nodes the local adjacency holds
constexpr int kMaxSkip = 16;                   // nets a window may skip over (look-ahead)

struct __align__(32) NodeSt {
  double lab;      // FP64 label (tentative until settled)
  float m32;       // float32 key of the label
  float pen;       // node penalty (fixed once reached)
  float cin;       // cheapest in-arc cost from an unsettled ROI neighbour
  int32_t par;     // ROI index of the winning relaxer
  int32_t st;      // ST_NONE / ST_FRONT / ST_DONE
  int32_t stamp;   // phase in which the node was last queued for recompute
};
static_assert(sizeof(NodeSt) == 32, "NodeSt must fill one 32-byte sector");

struct Ws {
  int32_t* seen;
  int32_t* g2r;
  int32_t* q[4];
  int32_t* roi;
  NodeSt* node;
  int32_t* fr[2];
  int32_t* dl;
  int32_t* blist;
  int32_t* adj;      // [kAdjCap][kDMax] neighbour ROI index or -1
  float* acost;      // [kAdjCap][kDMax] cost of the arc neighbour -> node
  int32_t* deg;      // [kAdjCap] arcs of the node
  int64_t* result;   // [0] status, [1] path len
  int64_t qcap;
};

// Seeds and targets of a multi-source multi-sink search
// (find_path_multisource_multisink, unified_pathfinder.py:2550-2659), global
// ids with FP64 costs, mapped to ROI-indexed arrays inside the search.
struct MultiSeeds {
  const int32_t* seeds;
  const double* seed_cost;
  int32_t nseeds;
  const int32_t* targets;
  const double* target_cost;
  int32_t ntargets;
  double* init;    // [R] seed cost before the node penalty, +inf for other nodes
  double* tcost;   // [R] target cost, NaN for other nodes
};

__host__ __device__ constexpr size_t round256(size_t v) { return (v + 255) & ~(size_t)255; }
__host__ __device__ constexpr size_t min_sz(size_t a, size_t b) { return a < b ? a : b; }

// Bytes of one search slot for n nodes.
__host__ __device__ constexpr size_t ws_bytes_for(size_t n) {
  return 10 * round256(4 * n) + round256(32 * n) + 2 * round256(4 * min_sz(n, kAdjCap) * kDMax) +
         round256(4 * min_sz(n, kAdjCap)) + round256(64);
}

__host__ inline size_t ws_layout(int32_t N, char* base, Ws* w) {
  size_t off = 0;
  auto take = [&](size_t bytes) -> char* {
    char* p = base ? base + off : nullptr;
    off += round256(bytes);
    return p;
  };
  const size_t n = (size_t)N;
  const size_t a = min_sz(n, kAdjCap);
  Ws t{};
  t.seen = (int32_t*)take(4 * n);
  t.g2r = (int32_t*)take(4 * n);
  for (int i = 0; i < 4; ++i) t.q[i] = (int32_t*)take(4 * n);
  t.roi = (int32_t*)take(4 * n);
  t.fr[0] = (int32_t*)take(4 * n);
  t.fr[1] = (int32_t*)take(4 * n);
  t.dl = (int32_t*)take(4 * n);
  t.node = (NodeSt*)take(32 * n);
  t.adj = (int32_t*)take(4 * a * kDMax);
  t.acost = (float*)take(4 * a * kDMax);
  t.deg = (int32_t*)take(4 * a);
  t.blist = t.q[0];  // the BFS queues are free while the search runs
  t.result = (int64_t*)take(64);
  t.qcap = (int64_t)n;
  if (w) *w = t;
  return off;
}

// A search-only slot for the window pass: the global->ROI map and ROI-sized
// arrays (the ROI comes from the batched extraction, so no BFS state).
__host__ __device__ inline size_t ws_slot_layout(int32_t N, int32_t Rmax, char* base, Ws* w) {
  size_t off = 0;
  char* p[11];
  const size_t n = (size_t)N, r = (size_t)Rmax, ad = min_sz(r, kAdjCap);
  const size_t sz[11] = {4 * n, 32 * r, 4 * r, 4 * r, 4 * r, 4 * r, 4 * ad * kDMax, 4 * ad * kDMax, 4 * ad, 64, 0};
  for (int i = 0; i < 10; ++i) {
    p[i] = base ? base + off : nullptr;
    off += round256(sz[i]);
  }
  if (w) {
    Ws t{};
    t.g2r = (int32_t*)p[0];
    t.node = (NodeSt*)p[1];
    t.fr[0] = (int32_t*)p[2];
    t.fr[1] = (int32_t*)p[3];
    t.dl = (int32_t*)p[4];
    t.blist = (int32_t*)p[5];
    t.adj = (int32_t*)p[6];
    t.acost = (float*)p[7];
    t.deg = (int32_t*)p[8];
    t.result = (int64_t*)p[9];
    t.qcap = 0;
    *w = t;
  }
  return off;
}

// A BFS-only slot for the batched ROI extraction: seen[N] + 4 queues.
struct BfsSlot {
  int32_t* seen;
  int32_t* q[4];
  int64_t qcap;
};

__host__ inline size_t bfs_slot_bytes(int32_t N, int64_t qcap) {
  return round256(4 * (size_t)N) + 4 * round256(4 * (size_t)qcap);
}

__host__ __device__ inline BfsSlot bfs_slot_at(char* base, int32_t N, int64_t qcap) {
  BfsSlot s;
  size_t off = 0;
  s.seen = (int32_t*)(base + off);
  off += round256(4 * (size_t)N);
  for (int i = 0; i < 4; ++i) {
    s.q[i] = (int32_t*)(base + off);
    off += round256(4 * (size_t)qcap);
  }
  s.qcap = qcap;
  return s;
}

// ---- block primitives ------------------------------------------------------
__device__ __forceinline__ unsigned long long block_min_u64(unsigned long long v, unsigned long long* s) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long y = __shfl_down_sync(0xffffffffu, v, o);
    v = y < v ? y : v;
  }
  if (lane == 0) s[wid] = v;
  __syncthreads();
  if (wid == 0) {
    unsigned long long w = (lane < kWarps) ? s[lane] : ~0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long y = __shfl_down_sync(0xffffffffu, w, o);
      w = y < w ? y : w;
    }
    if (lane == 0) s[0] = w;
  }
  __syncthreads();
  unsigned long long r = s[0];
  __syncthreads();
  return r;
}

// Per-stage cycle counters of the search (a tracing aid, read with
// ogr_search_profile): [0] BFS waves, [1] ROI compaction, [2] SSSP init and
// local adjacency, [3] phase queueing, [4] recompute, [5] frontier min,
// [6] settle, [7] statistics + backtrace, [8] cleanup, [9] searches,
// [10] phases, [11] BFS waves run, [12] ROI nodes, [13] recomputed nodes,
// [14] ROIs taken from the batched extraction.
__device__ unsigned long long g_stage[16];

struct Shared {
  unsigned long long s_min[kWarps];
  int s_cnt[kWarps];
  int s_off[kWarps];
  int nq[4];
  int seen_count;
  int met;
  int overflow;
  int bx0, bx1, by0, by1;
  int pos_src, pos_dst;
  int R;
  int nfront, nnext, ndirty, nb;
  int status;
  int found;
  int len;
  int local;
};

struct StageClock {
  long long t;
  __device__ void start() { t = clock64(); }
  __device__ void mark(int k) {
    if (threadIdx.x == 0) {
      const long long now = clock64();
      atomicAdd(&g_stage[k], (unsigned long long)(now - t));
      t = now;
    }
  }
};

// ---- ROI extraction ---------------------------------------------------------
// Bidirectional BFS from src/dst on seen[] (all zero on entry, restored to
// zero on exit) with queues of qcap entries; writes the ROI (ascending id,
// truncated with the must-keep swap) into out[0..out_cap) and its size into
// sh.R.  sh.status = OGR_ERR_CAPACITY when a queue overflowed.
__device__ void roi_build(Shared& sh, const ogr_graph& g, const ogr_net_args& a, int32_t* seen, int32_t* const* q,
                          int64_t qcap, int32_t* out, int32_t out_cap, StageClock& clk) {
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int sl = tid & (kSub - 1), grp = tid / kSub;
  const int nx = g.nx, nz = g.nz;
  const int32_t plane = nx * g.ny;
  const int32_t src = a.src, dst = a.dst;
  const int32_t* __restrict__ indptr = g.indptr;
  const int32_t* __restrict__ indices = g.indices;
  if (tid == 0) {
    seen[src] = 1;
    seen[dst] = 2;
    q[0][0] = src;
    q[2][0] = dst;
    sh.nq[0] = 1;
    sh.nq[2] = 1;
    sh.seen_count = (src != dst) ? 2 : 1;
    sh.overflow = 0;
    const int sy = (src % plane) / nx, sx = (src % plane) % nx;
    const int dy = (dst % plane) / nx, dx = (dst % plane) % nx;
    sh.bx0 = min(sx, dx); sh.bx1 = max(sx, dx);
    sh.by0 = min(sy, dy); sh.by1 = max(sy, dy);
    sh.met = 0;
    sh.pos_src = -1;
    sh.pos_dst = -1;
  }
  __syncthreads();
  int depth = 0, meet = -1;
  int cur_s = 0, cur_d = 2;
  while (depth < a.bfs_max_depth && (sh.nq[cur_s] > 0 || sh.nq[cur_d] > 0)) {
    for (int wave = 0; wave < 2; ++wave) {
      const int cur = wave == 0 ? cur_s : cur_d;
      const int nxt = cur ^ 1;
      const int32_t mark = wave == 0 ? 1 : 2;
      if (tid == 0) sh.nq[nxt] = 0;
      __syncthreads();
      const int n = (int)min((int64_t)sh.nq[cur], qcap);
      const int32_t* qc = q[cur];
      int32_t* qn = q[nxt];
      int local_met = 0, local_new = 0, local_ovf = 0;
      int lx0 = 1 << 30, lx1 = -1, ly0 = 1 << 30, ly1 = -1;
      for (int i = grp; i < n; i += kGroups) {
        const int32_t u = qc[i];
        const int32_t e1 = indptr[u + 1];
        for (int32_t e = indptr[u] + sl; e < e1; e += kSub) {
          if (g.blocked != nullptr && g.blocked[e]) continue;
          const int32_t v = indices[e];
          const int32_t old = atomicCAS(&seen[v], 0, mark);
          if (old == 0) {
            const int pos = atomicAdd(&sh.nq[nxt], 1);
            if (pos < qcap) qn[pos] = v; else local_ovf = 1;
            ++local_new;
            const int32_t r = v % plane;
            const int vy = r / nx, vx = r % nx;
            lx0 = min(lx0, vx); lx1 = max(lx1, vx);
            ly0 = min(ly0, vy); ly1 = max(ly1, vy);
          } else if (old != mark) {
            seen[v] = 3;
            local_met = 1;
          }
        }
      }
      local_new = __reduce_add_sync(0xffffffffu, local_new);
      local_met = __reduce_or_sync(0xffffffffu, local_met);
      local_ovf = __reduce_or_sync(0xffffffffu, local_ovf);
      lx0 = __reduce_min_sync(0xffffffffu, lx0);
      lx1 = __reduce_max_sync(0xffffffffu, lx1);
      ly0 = __reduce_min_sync(0xffffffffu, ly0);
      ly1 = __reduce_max_sync(0xffffffffu, ly1);
      if (lane == 0) {
        if (local_met) sh.met = 1;
        if (local_ovf) sh.overflow = 1;
        if (local_new) {
          atomicAdd(&sh.seen_count, local_new);
          atomicMin(&sh.bx0, lx0); atomicMax(&sh.bx1, lx1);
          atomicMin(&sh.by0, ly0); atomicMax(&sh.by1, ly1);
        }
      }
      __syncthreads();
      if (wave == 0) cur_s = nxt; else cur_d = nxt;
    }
    ++depth;
    if (tid == 0) atomicAdd(&g_stage[11], 2ull);
    if (sh.met && meet < 0) meet = depth;
    if (meet >= 0 && depth >= meet + a.bfs_halo) break;
    if ((double)sh.seen_count > a.bfs_stop_count) break;
    if (sh.overflow) break;
  }
  __syncthreads();
  clk.mark(0);
  // Ordered compaction over the bounding box (ascending global id): each warp
  // owns a contiguous segment; count, scan the 32 counts, then write.  Only
  // positions below out_cap are stored; those of src and dst are recorded.
  const int W = sh.bx1 - sh.bx0 + 1, H = sh.by1 - sh.by0 + 1;
  const int32_t area = W * H;
  const int32_t V = area * nz;
  const int32_t seg = (((V + kWarps - 1) / kWarps) + 31) & ~31;
  const int32_t w0 = warp * seg, w1 = min(V, w0 + seg);
  const int bx0 = sh.bx0, by0 = sh.by0;
  auto gid_of = [&](int32_t i) -> int32_t {
    const int z = i / area;
    const int32_t rem = i - z * area;
    const int y = by0 + rem / W;
    const int x = bx0 + rem % W;
    return z * plane + y * nx + x;
  };
  int cnt = 0;
  for (int32_t b = w0; b < w1; b += 32) {
    const int32_t i = b + lane;
    const bool f = i < w1 && seen[gid_of(i)] != 0;
    cnt += __popc(__ballot_sync(0xffffffffu, f));
  }
  if (lane == 0) sh.s_cnt[warp] = cnt;
  __syncthreads();
  if (warp == 0) {
    const int c = sh.s_cnt[lane];
    int x = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    sh.s_off[lane] = x - c;
    if (lane == 31) sh.R = x;
  }
  __syncthreads();
  int off = sh.s_off[warp];
  for (int32_t b = w0; b < w1; b += 32) {
    const int32_t i = b + lane;
    int32_t gid = 0;
    bool f = false;
    if (i < w1) {
      gid = gid_of(i);
      f = seen[gid] != 0;
    }
    const unsigned m = __ballot_sync(0xffffffffu, f);
    if (f) {
      const int pos = off + __popc(m & ((1u << lane) - 1));
      if (pos < out_cap) out[pos] = gid;
      if (gid == src) sh.pos_src = pos;
      if (gid == dst) sh.pos_dst = pos;
    }
    off += __popc(m);
  }
  __syncthreads();
  if (tid == 0) {
    int R = sh.R;
    if (R > a.max_roi_nodes) {
      // Must-keep swap (extract_roi_bfs :2359-2379): the positions of src/dst
      // in ascending order; each one beyond the cut swaps with slot 0 / 1.
      int kp[2];
      int32_t kn[2];
      int nk = 0;
      if (src == dst) {
        kp[0] = sh.pos_src; kn[0] = src; nk = 1;
      } else {
        const bool s_first = sh.pos_src < sh.pos_dst;
        kp[0] = s_first ? sh.pos_src : sh.pos_dst; kn[0] = s_first ? src : dst;
        kp[1] = s_first ? sh.pos_dst : sh.pos_src; kn[1] = s_first ? dst : src;
        nk = 2;
      }
      for (int k = 0; k < nk; ++k)
        if (kp[k] >= a.max_roi_nodes) out[k] = kn[k];
      R = a.max_roi_nodes;
    }
    sh.R = R;
    if (sh.overflow || R > out_cap) sh.status = OGR_ERR_CAPACITY;
    atomicAdd(&g_stage[12], (unsigned long long)R);
  }
  // restore seen[] to zero over the bounding box
  for (int32_t i = tid; i < V; i += kThreads) seen[gid_of(i)] = 0;
  __syncthreads();
  clk.mark(1);
}

// ---- the search on a given ROI ---------------------------------------------------
// roi[0..R) in ROI order (ignored when full).  Writes the path (global ids,
// src first) to path_out and its length to sh.len, or a status to sh.status.
//
// With kMulti the search is the reference's multi-source multi-sink form: every
// seed starts with label seed_cost + penalty and no parent (a first relaxation
// that later ones must beat in float32), targets are settled but never
// expanded, the search runs until nothing is left, and the result is the
// settled target with the least (label + target cost), first in pop order
// (label, ROI index) among equals.
//
// kLanes lanes serve one node (its arcs, then a shuffle reduction), so a CTA
// keeps 1024 / kLanes nodes in flight per round of a phase.
// Arcs per lane that the local-adjacency stages of the ROI search load in one
// batch: the first 12 arcs of a row (a lattice node has at most 10; at most 4
// per lane, to stay in registers) are read at once, then the records they
// name at once, so a row costs two dependent round trips instead of two per
// kLanes arcs.  Slots past the degree lie in the row's 32-slot allocation and
// are loaded but never used.
constexpr int kBatchArcs = 12;
static_assert(kBatchArcs <= kDMax, "a batch stays inside a local-adjacency row");

template <bool kMulti = false, int kLanes = kSearchLanes>
__device__ void sssp_roi(Shared& sh, const ogr_graph& g, const ogr_state& st, const ogr_net_args& a, const Ws& w,
                         const int32_t* roi, int32_t R, int32_t* path_out, int32_t path_cap,
                         unsigned long long* stats_acc, StageClock& clk, const float* roi_pen = nullptr,
                         const MultiSeeds* ms = nullptr) {
  static_assert(kLanes == 2 || kLanes == 4 || kLanes == 8 || kLanes == 16 || kLanes == 32,
                "lanes per node: a power of two from 2 to 32");
  constexpr int kSub = kLanes;                  // shadows the BFS's lane count inside the search
  constexpr int kGroups = kThreads / kLanes;
  constexpr int kPerWarp = 32 / kLanes;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int sl = tid & (kSub - 1), grp = tid / kSub;
  const int32_t src = a.src, dst = a.dst;
  const bool full = a.full_graph != 0;
  const int32_t* __restrict__ indptr = g.indptr;
  const int32_t* __restrict__ indices = g.indices;
  NodeSt* __restrict__ node = w.node;
  const float kInf = __int_as_float(0x7f800000);

  if (!full)
    for (int r = tid; r < R; r += kThreads) w.g2r[roi[r]] = r;
  if (tid == 0) {
    sh.local = (!full && R <= kAdjCap) ? 1 : 0;
    sh.nfront = 0;
    sh.nb = 0;
    sh.found = 0;
    sh.len = 0;
  }
  for (int r = tid; r < R; r += kThreads) {
    node[r].st = ST_NONE;
    node[r].stamp = -1;
    if constexpr (kMulti) {
      node[r].par = -1;
      ms->init[r] = __longlong_as_double(0x7ff0000000000000ll);
      ms->tcost[r] = __longlong_as_double(0x7ff8000000000000ll);
    }
  }
  __syncthreads();
  if constexpr (kMulti) {
    // Seeds and targets outside the ROI are dropped (as the reference does);
    // a repeated seed or target id is an argument error.
    for (int i = tid; i < ms->nseeds; i += kThreads) {
      const int32_t gid = ms->seeds[i];
      if (gid < 0 || gid >= g.num_nodes) { sh.status = OGR_ERR_ARG; continue; }
      const int32_t r = full ? gid : w.g2r[gid];
      if (r < 0) continue;
      if (atomicCAS(&node[r].stamp, -1, -2) != -1) { sh.status = OGR_ERR_ARG; continue; }
      ms->init[r] = ms->seed_cost[i];
    }
    for (int i = tid; i < ms->ntargets; i += kThreads) {
      const int32_t gid = ms->targets[i];
      if (gid < 0 || gid >= g.num_nodes) { sh.status = OGR_ERR_ARG; continue; }
      const int32_t r = full ? gid : w.g2r[gid];
      if (r < 0) continue;
      if (atomicCAS(&node[r].par, -1, -3) != -1) { sh.status = OGR_ERR_ARG; continue; }
      ms->tcost[r] = ms->target_cost[i];
    }
    __syncthreads();
    for (int r = tid; r < R; r += kThreads) {
      node[r].stamp = -1;
      node[r].par = -1;
    }
  }
  __syncthreads();
  // ROI-local adjacency: neighbour ROI index and in-arc cost per slot.
  if (sh.local) {
    int too_wide = 0;
    for (int r = grp; r < R; r += kGroups) {
      const int32_t rg = roi[r];
      const int32_t e0 = indptr[rg], e1 = indptr[rg + 1];
      if (e1 - e0 > kDMax) too_wide = 1;
      // only the node's own arcs: slots past its degree are never read
      const int dr = min(e1 - e0, kDMax);
      for (int k = sl; k < dr; k += kSub) {
        const int32_t e = e0 + k;
        w.adj[(int64_t)r * kDMax + k] = w.g2r[indices[e]];
        w.acost[(int64_t)r * kDMax + k] = st.rcost ? st.rcost[e] : st.total_cost[g.rev[e]];
      }
      if (sl == 0) w.deg[r] = min(e1 - e0, kDMax);
    }
    too_wide = __reduce_or_sync(0xffffffffu, too_wide);
    if (lane == 0 && too_wide) sh.local = 0;
  }
  const int32_t rs = kMulti ? -1 : (full ? src : w.g2r[src]);
  int32_t rd = kMulti ? -1 : (full ? dst : w.g2r[dst]);
  if (!kMulti && tid == 0 && (rs < 0 || rd < 0 || rs == rd)) sh.status = OGR_NO_PATH;
  __syncthreads();
  const bool local = sh.local != 0;
  clk.mark(2);
  int phase = 0;
  bool exhausted = false;   // the frontier ran out before dst settled
  if (sh.status == OGR_OK) {
    if constexpr (kMulti) {
      // the first recompute pass takes every seed (ROI order) from its initial
      // candidate; nothing is settled yet
      if (tid == 0) sh.ndirty = 0;
      __syncthreads();
      for (int r = tid; r < R; r += kThreads)
        if (ms->init[r] < __longlong_as_double(0x7ff0000000000000ll)) w.dl[atomicAdd(&sh.ndirty, 1)] = r;
    } else if (tid == 0) {
      node[rs].st = ST_DONE;
      node[rs].lab = 0.0;
      node[rs].m32 = 0.0f;
      node[rs].par = -1;
      w.blist[0] = rs;
      sh.nb = 1;
    }
    __syncthreads();
    int cur = 0;
    const int max_phase = 2 * R + 4;
    // With statistics requested the search goes on after dst is settled until
    // every node with a label <= L(dst) is settled (T > L(dst)): the IN bound
    // can settle dst before cheaper nodes, which the heap pops earlier.
    bool dst_done = false;
    double ld_stop = 0.0;
    while (true) {
      // 1. queue the unsettled ROI neighbours of the newly settled nodes
      if (!(kMulti && phase == 0)) {
      if (tid == 0) sh.ndirty = 0;
      __syncthreads();
      const int nb = sh.nb;
      for (int i = grp; i < nb; i += kGroups) {
        const int32_t x = w.blist[i];
        if (local) {
          constexpr int kB = (kBatchArcs + kSub - 1) / kSub < 4 ? (kBatchArcs + kSub - 1) / kSub : 4;
          const int dx = w.deg[x];
          const int32_t* arow = w.adj + (int64_t)x * kDMax;
          int32_t yb[kB];
#pragma unroll
          for (int j = 0; j < kB; ++j) yb[j] = arow[sl + j * kSub];
          int32_t sb[kB];
#pragma unroll
          for (int j = 0; j < kB; ++j) {
            const bool ok = sl + j * kSub < dx && yb[j] >= 0;
            sb[j] = ok ? node[yb[j]].st : ST_DONE;
          }
#pragma unroll
          for (int j = 0; j < kB; ++j) {
            if (sb[j] >= ST_DONE) continue;
            if (atomicExch(&node[yb[j]].stamp, phase) != phase) w.dl[atomicAdd(&sh.ndirty, 1)] = yb[j];
          }
          for (int k = sl + kB * kSub; k < dx; k += kSub) {   // rows wider than a batch
            const int32_t y = arow[k];
            if (y < 0 || node[y].st >= ST_DONE) continue;
            if (atomicExch(&node[y].stamp, phase) != phase) w.dl[atomicAdd(&sh.ndirty, 1)] = y;
          }
        } else {
          const int32_t xg = full ? x : roi[x];
          const int32_t e1 = indptr[xg + 1];
          for (int32_t e = indptr[xg] + sl; e < e1; e += kSub) {
            const int32_t yg = indices[e];
            const int32_t y = full ? yg : w.g2r[yg];
            if (y < 0 || node[y].st >= ST_DONE) continue;
            if (atomicExch(&node[y].stamp, phase) != phase) w.dl[atomicAdd(&sh.ndirty, 1)] = y;
          }
        }
      }
      }
      __syncthreads();
      clk.mark(3);
      // 2. recompute each queued node from all settled in-neighbours: a
      //    kLanes-lane group per node, lanes over its arcs, shuffle reduction.
      const int nd = sh.ndirty;
      const int half = lane / kLanes;
      for (int base = warp * kPerWarp; base < nd; base += kWarps * kPerWarp) {
        const int idx = base + half;
        const bool valid = idx < nd;
        const int32_t y = valid ? w.dl[idx] : 0;
        bool fresh = false;
        float p = 0.0f;
        if (valid) {
          fresh = node[y].st == ST_NONE;
          if (sl == 0)
            p = !fresh ? node[y].pen : (roi_pen ? roi_pen[y] : ogr_node_penalty(st, a, full ? y : roi[y]));
        }
        p = __shfl_sync(0xffffffffu, p, lane & ~(kLanes - 1));
        const double pd = (double)p;
        float ba = kInf, bc = kInf;
        double bl = 0.0;
        int32_t bu = 0x7fffffff;
        float cin = kInf;
        if constexpr (kMulti) {
          // the seed's own start: relaxed before any pop, so it wins float32 ties
          if (valid && sl == 0) {
            const double s0 = ms->init[y];
            if (s0 < __longlong_as_double(0x7ff0000000000000ll)) {
              ba = __double2float_rn(s0 + pd);
              bl = -__longlong_as_double(0x7ff0000000000000ll);
              bu = -1;
            }
          }
        }
        if (valid) {
          if (local) {
            constexpr int kB = (kBatchArcs + kSub - 1) / kSub < 4 ? (kBatchArcs + kSub - 1) / kSub : 4;
            const int dy = w.deg[y];
            const int32_t* arow = w.adj + (int64_t)y * kDMax;
            const float* crow = w.acost + (int64_t)y * kDMax;
            int32_t ub[kB];
            float cb[kB];
#pragma unroll
            for (int j = 0; j < kB; ++j) {
              ub[j] = arow[sl + j * kSub];
              cb[j] = crow[sl + j * kSub];
            }
            int32_t sb[kB];
            double lb[kB];
#pragma unroll
            for (int j = 0; j < kB; ++j) {
              const bool ok = sl + j * kSub < dy && ub[j] >= 0;
              sb[j] = ok ? node[ub[j]].st : -1;
              lb[j] = ok ? node[ub[j]].lab : 0.0;
            }
            auto relax = [&](int32_t u, float c, int32_t su, double lu) {
              if (kMulti && su == ST_SINK) return;   // targets relax nothing
              if (su != ST_DONE) {
                cin = fminf(cin, c);
                return;
              }
              const float a32 = __double2float_rn((lu + (double)c) + pd);
              if (!(a32 < kInf)) return;
              if (ogr_key_lt(a32, lu, u, ba, bl, bu)) { ba = a32; bl = lu; bu = u; bc = c; }
            };
#pragma unroll
            for (int j = 0; j < kB; ++j)
              if (sb[j] >= 0) relax(ub[j], cb[j], sb[j], lb[j]);
            for (int k = sl + kB * kSub; k < dy; k += kSub) {   // rows wider than a batch
              const int32_t u = arow[k];
              if (u < 0) continue;
              relax(u, crow[k], node[u].st, node[u].lab);
            }
          } else {
            const int32_t yg = full ? y : roi[y];
            const int32_t e1 = indptr[yg + 1];
            for (int32_t e = indptr[yg] + sl; e < e1; e += kSub) {
              const int32_t ug = indices[e];
              const int32_t u = full ? ug : w.g2r[ug];
              if (u < 0) continue;
              const float c = st.rcost ? st.rcost[e] : st.total_cost[g.rev[e]];
              if (kMulti && node[u].st == ST_SINK) continue;   // targets relax nothing
              if (node[u].st != ST_DONE) {
                cin = fminf(cin, c);
                continue;
              }
              const double lu = node[u].lab;
              const float a32 = __double2float_rn((lu + (double)c) + pd);
              if (!(a32 < kInf)) continue;
              if (ogr_key_lt(a32, lu, u, ba, bl, bu)) { ba = a32; bl = lu; bu = u; bc = c; }
            }
          }
        }
#pragma unroll
        for (int o = kLanes / 2; o > 0; o >>= 1) {
          const float oa = __shfl_xor_sync(0xffffffffu, ba, o);
          const double ol = __shfl_xor_sync(0xffffffffu, bl, o);
          const int32_t ou = __shfl_xor_sync(0xffffffffu, bu, o);
          const float oc = __shfl_xor_sync(0xffffffffu, bc, o);
          if (ogr_key_lt(oa, ol, ou, ba, bl, bu)) { ba = oa; bl = ol; bu = ou; bc = oc; }
          cin = fminf(cin, __shfl_xor_sync(0xffffffffu, cin, o));
        }
        if (valid && sl == 0) {
          NodeSt& ns = node[y];
          if (fresh) ns.pen = p;
          ns.cin = cin;
          if (ba < kInf) {
            ns.m32 = ba;
            ns.lab = (kMulti && bu == -1) ? ms->init[y] + pd : (bl + (double)bc) + pd;
            ns.par = bu;
            if (fresh) {
              ns.st = ST_FRONT;
              w.fr[cur][atomicAdd(&sh.nfront, 1)] = y;
            }
          }
        }
      }
      __syncthreads();
      clk.mark(4);
      if (tid == 0) atomicAdd(&g_stage[13], (unsigned long long)nd);
      const int nf = sh.nfront;
      if (nf == 0) {
        if (!kMulti && !dst_done) exhausted = true;
        if (tid == 0 && !kMulti) {
          if (dst_done)
            sh.found = 1;
          else
            sh.status = OGR_NO_PATH;
        }
        break;
      }
      // 3. T = smallest tentative label in the frontier.
      unsigned long long mn = ~0ull;
      for (int i = tid; i < nf; i += kThreads) {
        const unsigned long long b = ogr_dbits(node[w.fr[cur][i]].lab);
        mn = b < mn ? b : mn;
      }
      mn = block_min_u64(mn, sh.s_min);
      const double T = __longlong_as_double((long long)mn);
      clk.mark(5);
      if (dst_done && T > ld_stop) {
        if (tid == 0) sh.found = 1;
        break;
      }
      // 4. settle every node whose state can no longer change.
      if (tid == 0) { sh.nb = 0; sh.nnext = 0; }
      __syncthreads();
      for (int i = tid; i < nf; i += kThreads) {
        const int32_t x = w.fr[cur][i];
        NodeSt& ns = node[x];
        bool settle = (ns.lab == T);
        if (!settle) settle = ns.m32 < __double2float_rn((T + (double)ns.cin) + (double)ns.pen);
        if (settle) {
          if (kMulti && ms->tcost[x] == ms->tcost[x]) {
            ns.st = ST_SINK;   // settled, never expanded
          } else {
            ns.st = ST_DONE;
            w.blist[atomicAdd(&sh.nb, 1)] = x;
          }
        } else {
          w.fr[cur ^ 1][atomicAdd(&sh.nnext, 1)] = x;
        }
      }
      __syncthreads();
      if (tid == 0) sh.nfront = sh.nnext;
      cur ^= 1;
      clk.mark(6);
      if (tid == 0) atomicAdd(&g_stage[10], 1ull);
      const bool done = !kMulti && !dst_done && node[rd].st == ST_DONE;
      const bool capped = phase + 1 > max_phase;
      if (done) ld_stop = node[rd].lab;
      __syncthreads();
      if (done) {
        dst_done = true;
        if (stats_acc == nullptr) {
          if (tid == 0) sh.found = 1;
          break;
        }
      }
      if (capped) {
        if (tid == 0) sh.status = OGR_ERR_ITER_CAP;
        break;
      }
      ++phase;
    }
  }
  __syncthreads();
  if constexpr (kMulti) {
    // The reference keeps the first popped target whose label + target cost is
    // strictly below the best so far: the least (total, label, ROI index).
    if (sh.status == OGR_OK) {
      unsigned long long k1 = ~0ull;
      for (int r = tid; r < R; r += kThreads) {
        if (node[r].st != ST_SINK) continue;
        const double tot = node[r].lab + ms->tcost[r];
        if (!(tot < __longlong_as_double(0x7ff0000000000000ll))) continue;
        k1 = min(k1, ogr_order_bits(tot));
      }
      k1 = block_min_u64(k1, sh.s_min);
      unsigned long long k2 = ~0ull;
      if (k1 != ~0ull)
        for (int r = tid; r < R; r += kThreads)
          if (node[r].st == ST_SINK && ogr_order_bits(node[r].lab + ms->tcost[r]) == k1)
            k2 = min(k2, ogr_order_bits(node[r].lab));
      k2 = block_min_u64(k2, sh.s_min);
      unsigned long long k3 = ~0ull;
      if (k1 != ~0ull)
        for (int r = tid; r < R; r += kThreads)
          if (node[r].st == ST_SINK && ogr_order_bits(node[r].lab + ms->tcost[r]) == k1 &&
              ogr_order_bits(node[r].lab) == k2)
            k3 = min(k3, (unsigned long long)r);
      k3 = block_min_u64(k3, sh.s_min);
      if (tid == 0) {
        if (k1 == ~0ull) {
          sh.status = OGR_NO_PATH;
        } else {
          sh.found = 1;
          sh.nb = (int)k3;   // the chosen target
        }
      }
    }
    __syncthreads();
    if (sh.found) rd = sh.nb;
    // every settled node was popped once; expanded ones scanned their row
    if (sh.status == OGR_OK && stats_acc != nullptr) {
      unsigned arcs = 0, pops = 0;
      for (int r = tid; r < R; r += kThreads) {
        const int32_t sr = node[r].st;
        if (sr < ST_DONE) continue;
        ++pops;
        if (sr == ST_DONE) {
          const int32_t rg = full ? r : roi[r];
          arcs += (unsigned)(indptr[rg + 1] - indptr[rg]);
        }
      }
      arcs = __reduce_add_sync(0xffffffffu, arcs);
      pops = __reduce_add_sync(0xffffffffu, pops);
      if (lane == 0) {
        atomicAdd(&stats_acc[0], (unsigned long long)arcs);
        atomicAdd(&stats_acc[1], (unsigned long long)pops);
      }
      if (tid == 0) {
        atomicAdd(&stats_acc[2], (unsigned long long)R);
        atomicAdd(&stats_acc[3], (unsigned long long)(phase + 1));
      }
    }
  }
  // A search that cannot reach dst pops every node it reaches and scans each
  // one's row, as the heap does before it runs empty.
  if (!kMulti && exhausted && stats_acc != nullptr) {
    unsigned arcs = 0, pops = 0;
    for (int r = tid; r < R; r += kThreads) {
      if (node[r].st != ST_DONE) continue;
      const int32_t rg = full ? r : roi[r];
      arcs += (unsigned)(indptr[rg + 1] - indptr[rg]);
      ++pops;
    }
    arcs = __reduce_add_sync(0xffffffffu, arcs);
    pops = __reduce_add_sync(0xffffffffu, pops);
    if (lane == 0) {
      atomicAdd(&stats_acc[0], (unsigned long long)arcs);
      atomicAdd(&stats_acc[1], (unsigned long long)pops);
    }
    if (tid == 0) {
      atomicAdd(&stats_acc[2], (unsigned long long)R);
      atomicAdd(&stats_acc[3], (unsigned long long)(phase + 1));
    }
  }
  // Arcs the sequential search scans before popping dst: the rows of all
  // nodes popped before it, i.e. settled with (L, idx) < (L(dst), dst).
  if (!kMulti && sh.found && stats_acc != nullptr) {
    const double ld = node[rd].lab;
    unsigned arcs = 0, pops = 0;
    for (int r = tid; r < R; r += kThreads) {
      if (node[r].st != ST_DONE) continue;
      const double lr = node[r].lab;
      if (lr < ld || (lr == ld && r < rd)) {
        const int32_t rg = full ? r : roi[r];
        arcs += (unsigned)(indptr[rg + 1] - indptr[rg]);
        ++pops;
      }
    }
    arcs = __reduce_add_sync(0xffffffffu, arcs);
    pops = __reduce_add_sync(0xffffffffu, pops);
    if (lane == 0) {
      atomicAdd(&stats_acc[0], (unsigned long long)arcs);
      atomicAdd(&stats_acc[1], (unsigned long long)pops);
    }
    if (tid == 0) {
      atomicAdd(&stats_acc[1], 1ull);
      atomicAdd(&stats_acc[2], (unsigned long long)R);
      atomicAdd(&stats_acc[3], (unsigned long long)(phase + 1));
    }
  }
  // Backtrace dst -> src.
  if (tid == 0 && sh.found && sh.status == OGR_OK) {
    int len = 0;
    for (int32_t c = rd; c != -1 && len <= R; c = node[c].par) ++len;
    if (len > R) {
      sh.status = OGR_ERR_ITER_CAP;  // a parent chain longer than the ROI is a cycle
    } else if (len > path_cap) {
      sh.status = OGR_ERR_CAPACITY;
    } else {
      int i = len - 1;
      for (int32_t c = rd; c != -1; c = node[c].par) path_out[i--] = full ? c : roi[c];
      sh.len = len;
      if (len < 2) sh.status = OGR_NO_PATH;
    }
  }
  __syncthreads();
  clk.mark(7);
  if (!full)
    for (int r = tid; r < R; r += kThreads) w.g2r[roi[r]] = -1;
  __syncthreads();
  clk.mark(8);
  if (tid == 0) atomicAdd(&g_stage[9], 1ull);
}

// Whole search for one net on one CTA (ROI extraction inline).
template <int L>
__device__ void search_net(Shared& sh, const ogr_graph& g, const ogr_state& st, const ogr_net_args& a, const Ws& w,
                           int32_t* path_out, int32_t path_cap, unsigned long long* stats_acc) {
  StageClock clk;
  clk.start();
  if (threadIdx.x == 0) {
    sh.status = OGR_OK;
    sh.len = 0;
    sh.found = 0;
  }
  __syncthreads();
  int32_t R = g.num_nodes;
  if (!a.full_graph) {
    roi_build(sh, g, a, w.seen, w.q, w.qcap, w.roi, a.max_roi_nodes, clk);
    R = sh.R;
  }
  if (sh.status != OGR_OK) return;
  sssp_roi<false, L>(sh, g, st, a, w, w.roi, R, path_out, path_cap, stats_acc, clk);
}

// ---- commit / rip-up ---------------------------------------------------------
// commit_path / clear_path (:1096-1135) + refresh_live_present_costs (:1403),
// _mark/_clear_path_node_use (:4635-4659), barrel ownership of every node a
// via hop spans (:4934-5034), arcs in _path_to_edges order (:9981-10046).
// Returns OGR_OK, OGR_ERR_ARG (a hop is not an arc) or OGR_ERR_CAPACITY.
__device__ int apply_path_dev(const ogr_graph& g, const ogr_state& st, const int32_t* path, int32_t len,
                              int32_t net_id, int32_t sign, float pres_fac, int32_t live, int32_t* arcs_out,
                              int32_t* s_via, int* s_flags) {
  const int tid = threadIdx.x, nt = blockDim.x;
  if (tid == 0) { s_flags[0] = 0; s_flags[1] = 0; }
  __syncthreads();
  const int hops = len - 1;
  const int32_t plane = g.nx * g.ny;
  for (int i = tid; i < hops; i += nt) {
    const int32_t u = path[i], v = path[i + 1];
    int32_t f = -1;
    for (int32_t e = g.indptr[u]; e < g.indptr[u + 1]; ++e)
      if (g.indices[e] == v) { f = e; break; }
    if (f < 0) { s_flags[1] = 1; continue; }
    const int32_t r = g.rev[f];
    const int j = hops - 1 - i;
    if (arcs_out) { arcs_out[i] = f; arcs_out[hops + j] = r; }
    for (int k = 0; k < 2; ++k) {
      const int32_t e = k == 0 ? f : r;
      float p = st.present[e];
      p = sign > 0 ? __fadd_rn(p, 1.0f) : fmaxf(__fsub_rn(p, 1.0f), 0.0f);
      st.present[e] = p;
      if (live) {
        const float bias = (st.layer_bias != nullptr && st.edge_kind[e] == 0) ? st.layer_bias[st.edge_layer[e]] : 1.0f;
        const float scale = st.layer_bias != nullptr ? __fmul_rn(pres_fac, bias) : pres_fac;
        const float prosp = fmaxf(0.0f, __fsub_rn(__fadd_rn(p, 1.0f), st.capacity[e]));
        const float tc = __fadd_rn(st.live_static[e], __fmul_rn(scale, prosp));
        st.total_cost[e] = tc;
        if (st.rcost) st.rcost[k == 0 ? r : f] = tc;   // the opposite arc's row entry
      }
    }
  }
  for (int i = tid; i < len; i += nt) {
    const int32_t n = path[i];
    const int32_t u = st.path_node_use[n];
    st.path_node_use[n] = sign > 0 ? u + 1 : max(u - 1, 0);
  }
  __syncthreads();
  if (tid == 0) {
    int nv = 0;
    for (int i = 0; i < hops && !s_flags[1]; ++i) {
      const int32_t u = path[i], v = path[i + 1];
      const int32_t ru = u % plane, rv = v % plane;
      const int zu = u / plane, zv = v / plane;
      if (ru != rv || zu == zv) continue;
      for (int z = min(zu, zv); z <= max(zu, zv); ++z) {
        const int32_t nd = z * plane + ru;
        bool dup = false;
        for (int k = 0; k < nv; ++k)
          if (s_via[k] == nd) { dup = true; break; }
        if (dup) continue;
        if (nv >= kMaxViaNodes) { s_flags[1] = 2; break; }
        s_via[nv++] = nd;
      }
    }
    s_flags[0] = nv;
  }
  __syncthreads();
  const int nv = s_flags[0];
  for (int k = tid; k < nv; k += nt) {
    const int32_t nd = s_via[k];
    st.owner_count[nd] += sign > 0 ? 1 : -1;
    st.owner_xor[nd] ^= net_id;
  }
  const int bad = s_flags[1];
  __syncthreads();
  return bad ? (bad == 1 ? OGR_ERR_ARG : OGR_ERR_CAPACITY) : OGR_OK;
}

// ---- kernels -------------------------------------------------------------------
template <int L>
__global__ void __launch_bounds__(kThreads, 1)
find_path_kernel(ogr_graph g, ogr_state st, ogr_net_args a, Ws w, int32_t* path_out, int32_t path_cap,
                 int64_t* stats) {
  __shared__ Shared sh;
  search_net<L>(sh, g, st, a, w, path_out, path_cap, reinterpret_cast<unsigned long long*>(stats));
  if (threadIdx.x == 0) {
    w.result[0] = sh.status;
    w.result[1] = sh.len;
  }
}

// The reference's solver seam: search a given ROI (ROI order = tie order)
// with a given ROI-local penalty array (or none).
template <int L>
__global__ void __launch_bounds__(kThreads, 1)
find_path_given_roi_kernel(ogr_graph g, ogr_state st, ogr_net_args a, Ws w, const int32_t* roi, int32_t R,
                           const float* roi_pen, int32_t* path_out, int32_t path_cap, int64_t* stats) {
  __shared__ Shared sh;
  StageClock clk;
  clk.start();
  if (threadIdx.x == 0) {
    sh.status = OGR_OK;
    sh.len = 0;
    sh.found = 0;
  }
  __syncthreads();
  sssp_roi<false, L>(sh, g, st, a, w, roi, R, path_out, path_cap, reinterpret_cast<unsigned long long*>(stats), clk,
                     roi_pen);
  if (threadIdx.x == 0) {
    w.result[0] = sh.status;
    w.result[1] = sh.len;
  }
}

// The multi-source multi-sink seam on a given ROI.
template <int L>
__global__ void __launch_bounds__(kThreads, 1)
find_path_multi_kernel(ogr_graph g, ogr_state st, ogr_net_args a, Ws w, const int32_t* roi, int32_t R,
                       const float* roi_pen, MultiSeeds ms, int32_t* path_out, int32_t path_cap, int64_t* stats) {
  __shared__ Shared sh;
  StageClock clk;
  clk.start();
  if (threadIdx.x == 0) {
    sh.status = OGR_OK;
    sh.len = 0;
    sh.found = 0;
  }
  __syncthreads();
  sssp_roi<true, L>(sh, g, st, a, w, roi, R, path_out, path_cap, reinterpret_cast<unsigned long long*>(stats), clk,
                 roi_pen, &ms);
  if (threadIdx.x == 0) {
    w.result[0] = sh.status;
    w.result[1] = sh.len;
  }
}

__global__ void __launch_bounds__(kThreads, 1)
roi_kernel(ogr_graph g, ogr_net_args a, Ws w, int32_t* roi_out, int32_t roi_cap) {
  __shared__ Shared sh;
  StageClock clk;
  clk.start();
  if (threadIdx.x == 0) sh.status = OGR_OK;
  __syncthreads();
  int R = 0;
  if (a.full_graph) {
    R = g.num_nodes;
    if (threadIdx.x == 0 && R > roi_cap) sh.status = OGR_ERR_CAPACITY;
    __syncthreads();
    if (sh.status == OGR_OK)
      for (int r = threadIdx.x; r < R; r += kThreads) roi_out[r] = r;
  } else {
    roi_build(sh, g, a, w.seen, w.q, w.qcap, roi_out, roi_cap, clk);
    R = sh.R;
  }
  if (threadIdx.x == 0) {
    w.result[0] = sh.status;
    w.result[1] = R;
  }
}

__global__ void ws_init_kernel(Ws w, int64_t N) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    w.seen[i] = 0;
    w.g2r[i] = -1;
  }
}

__global__ void bfs_init_kernel(char* base, int32_t slots, size_t slot_bytes, int32_t N, int64_t qcap) {
  for (int s = 0; s < slots; ++s) {
    BfsSlot b = bfs_slot_at(base + (size_t)s * slot_bytes, N, qcap);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
      b.seen[i] = 0;
  }
}

constexpr int kApplyThreads = 256;

__global__ void __launch_bounds__(kApplyThreads)
path_apply_kernel(ogr_graph g, ogr_state st, const int32_t* path, int32_t len, int32_t net_id, int32_t sign,
                  float pres_fac, int32_t live, int32_t* arcs_out, int32_t* status) {
  __shared__ int32_t s_via[kMaxViaNodes];
  __shared__ int s_flags[2];
  const int rc = apply_path_dev(g, st, path, len, net_id, sign, pres_fac, live, arcs_out, s_via, s_flags);
  if (threadIdx.x == 0) *status = rc;
}

// Commit many paths at once (a best-state restore, _restore_routing_state
// :7806-7838): present +1 on both arcs of every hop, path-node use +1, barrel
// ownership of every via-spanned node; no live refresh.  Commits only add
// exact small integers (and XOR ids), so paths may be applied by different
// CTAs in any order and the state equals the sequential one.  Path k is
// nodes[off[k] .. off[k+1]); its arcs go to arcs[2 * (off[k] - k) ..]; with a
// store given, the path, its length and its arcs are also written to slot
// store_slot[k] (the per-net overuse sums read the slot's arcs).
__global__ void __launch_bounds__(kApplyThreads)
paths_commit_kernel(ogr_graph g, ogr_state st, const int32_t* nodes, const int32_t* off, const int32_t* net_ids,
                    int32_t n_paths, int32_t* arcs, int32_t* store_path, int32_t* store_len,
                    int32_t* store_arcs, const int32_t* store_slot, int32_t slot_cap, int32_t* status) {
  __shared__ int32_t s_via[kMaxViaNodes];
  __shared__ int s_nv, s_bad;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int32_t plane = g.nx * g.ny;
  for (int32_t k = blockIdx.x; k < n_paths; k += gridDim.x) {
    const int32_t o = off[k], len = off[k + 1] - off[k];
    const int32_t* path = nodes + o;
    const int hops = len - 1;
    int32_t* a_out = arcs + 2 * (int64_t)(o - k);
    int32_t* a_store = (store_arcs != nullptr && len <= slot_cap)
                           ? store_arcs + (int64_t)store_slot[k] * 2 * slot_cap : nullptr;
    if (tid == 0) { s_nv = 0; s_bad = 0; }
    __syncthreads();
    for (int i = tid; i < hops; i += nt) {
      const int32_t u = path[i], v = path[i + 1];
      int32_t f = -1;
      for (int32_t e = g.indptr[u]; e < g.indptr[u + 1]; ++e)
        if (g.indices[e] == v) { f = e; break; }
      if (f < 0) { s_bad = 1; continue; }
      const int32_t r = g.rev[f];
      a_out[i] = f;
      a_out[hops + (hops - 1 - i)] = r;
      if (a_store) {
        a_store[i] = f;
        a_store[hops + (hops - 1 - i)] = r;
      }
      atomicAdd(&st.present[f], 1.0f);
      atomicAdd(&st.present[r], 1.0f);
    }
    for (int i = tid; i < len; i += nt) atomicAdd(&st.path_node_use[path[i]], 1);
    if (store_path != nullptr && len <= slot_cap)
      for (int i = tid; i < len; i += nt) store_path[(int64_t)store_slot[k] * slot_cap + i] = path[i];
    __syncthreads();
    if (tid == 0) {
      int nv = 0;
      for (int i = 0; i < hops && !s_bad; ++i) {
        const int32_t u = path[i], v = path[i + 1];
        const int32_t ru = u % plane, rv = v % plane;
        const int zu = u / plane, zv = v / plane;
        if (ru != rv || zu == zv) continue;
        for (int z = min(zu, zv); z <= max(zu, zv); ++z) {
          const int32_t nd = z * plane + ru;
          bool dup = false;
          for (int q = 0; q < nv; ++q)
            if (s_via[q] == nd) { dup = true; break; }
          if (dup) continue;
          if (nv >= kMaxViaNodes) { s_bad = 2; break; }
          s_via[nv++] = nd;
        }
      }
      s_nv = nv;
      if (store_len != nullptr) store_len[store_slot[k]] = len <= slot_cap ? len : 0;
      if (len > slot_cap && store_path != nullptr) s_bad = 2;
    }
    __syncthreads();
    for (int q = tid; q < s_nv; q += nt) {
      atomicAdd(&st.owner_count[s_via[q]], 1);
      atomicXor(&st.owner_xor[s_via[q]], net_ids[k]);
    }
    if (tid == 0 && s_bad) atomicMax(status, s_bad);
    __syncthreads();
  }
}

// Extract the (cost-independent) ROIs of every ROI net of the pass, one net
// per CTA at a time, each CTA with its own BFS slot.  roi_len[n] = -1 when a
// queue overflowed (the pass then extracts that ROI inline).
__global__ void __launch_bounds__(kThreads, 1)
roi_batch_kernel(ogr_graph g, ogr_net_table t, ogr_pass_args pa, ogr_roi_batch rb) {
  __shared__ Shared sh;
  __shared__ int s_k;
  BfsSlot slot = bfs_slot_at((char*)rb.bfs_ws + (size_t)blockIdx.x * rb.slot_bytes, g.num_nodes, rb.qcap);
  while (true) {
    if (threadIdx.x == 0) s_k = atomicAdd(rb.next, 1);
    __syncthreads();
    const int k = s_k;
    __syncthreads();
    if (k >= pa.count) break;
    const int32_t n = pa.order[k];
    if (t.net_full[n]) {
      if (threadIdx.x == 0) rb.roi_len[n] = 0;
      continue;
    }
    ogr_net_args a = ogr_pass_net_args(t, pa, n, 0);
    StageClock clk;
    clk.start();
    if (threadIdx.x == 0) sh.status = OGR_OK;
    __syncthreads();
    roi_build(sh, g, a, slot.seen, slot.q, slot.qcap, rb.roi_pool + (int64_t)n * rb.roi_cap, rb.roi_cap, clk);
    if (threadIdx.x == 0) {
      rb.roi_len[n] = (sh.status == OGR_OK) ? sh.R : -1;
      if (rb.roi_box) {
        rb.roi_box[4 * n + 0] = sh.bx0;
        rb.roi_box[4 * n + 1] = sh.bx1;
        rb.roi_box[4 * n + 2] = sh.by0;
        rb.roi_box[4 * n + 3] = sh.by1;
      }
    }
    __syncthreads();
  }
}

// One launch routes an ordered list of nets the way _route_all does.
template <int L>
__global__ void __launch_bounds__(kThreads, 1)
route_pass_kernel(ogr_graph g, ogr_state st, ogr_net_table t, ogr_pass_args pa, ogr_roi_batch rb, int use_batch,
                  Ws w) {
  __shared__ Shared sh;
  __shared__ int32_t s_via[kMaxViaNodes];
  __shared__ int s_flags[2];
  __shared__ int s_fallbacks;
  __shared__ int s_error;
  unsigned long long* stats = reinterpret_cast<unsigned long long*>(pa.stats);
  if (w.result[0] < 0) return;  // an earlier step of this pass failed
  if (threadIdx.x == 0) { s_fallbacks = (int)w.result[2]; s_error = OGR_OK; }
  __syncthreads();
  for (int k = 0; k < pa.count; ++k) {
    const int32_t n = pa.order[k];
    int32_t* slot = t.store_path + (int64_t)n * t.slot_cap;
    int32_t* arcs = t.store_arcs + (int64_t)n * 2 * t.slot_cap;
    const int32_t old_len = t.store_len[n];
    if (old_len >= 2) {
      const int rc = apply_path_dev(g, st, slot, old_len, t.net_id[n], -1, pa.pres_fac, pa.live, nullptr, s_via,
                                    s_flags);
      if (rc != OGR_OK) {
        if (threadIdx.x == 0) s_error = rc;
        break;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) t.store_len[n] = 0;
    ogr_net_args a = ogr_pass_net_args(t, pa, n, 0);
    const int pre = (use_batch && !a.full_graph) ? rb.roi_len[n] : -1;
    if (pre > 0) {
      StageClock clk;
      clk.start();
      if (threadIdx.x == 0) {
        sh.status = OGR_OK;
        atomicAdd(&g_stage[14], 1ull);
      }
      __syncthreads();
      sssp_roi<false, L>(sh, g, st, a, w, rb.roi_pool + (int64_t)n * rb.roi_cap, pre, slot, t.slot_cap, stats, clk);
    } else {
      search_net<L>(sh, g, st, a, w, slot, t.slot_cap, stats);
    }
    int flags = 0;
    const int st1 = sh.status;
    if (st1 < 0) {
      if (threadIdx.x == 0) s_error = st1;
      break;
    }
    if (st1 != OGR_OK && s_fallbacks < pa.fallback_quota) {
      a = ogr_pass_net_args(t, pa, n, 1);
      __syncthreads();
      if (threadIdx.x == 0) ++s_fallbacks;
      search_net<L>(sh, g, st, a, w, slot, t.slot_cap, stats);
      const int st2 = sh.status;
      if (st2 < 0) {
        if (threadIdx.x == 0) s_error = st2;
        break;
      }
      flags |= 2;
    }
    const int fin = sh.status;
    const int len = sh.len;
    __syncthreads();
    if (fin == OGR_OK) {
      const int rc = apply_path_dev(g, st, slot, len, t.net_id[n], +1, pa.pres_fac, pa.live, arcs, s_via, s_flags);
      if (rc != OGR_OK) {
        if (threadIdx.x == 0) s_error = rc;
        break;
      }
      if (threadIdx.x == 0) t.store_len[n] = len;
    } else {
      flags |= 1;
    }
    if (threadIdx.x == 0) pa.net_status[k] = flags;
    __syncthreads();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    w.result[2] = s_fallbacks;
    if (s_error != OGR_OK) w.result[0] = s_error;
  }
}

// ---- batched disjoint-ROI windows ---------------------------------------------
// Control block of the window pass (device scratch, cleared per launch).
struct WinCtl {
  unsigned long long bar_count;
  int32_t bar_err;
  int32_t cursor;
  int32_t wsize;
  int32_t error;
};

struct WinSlots {
  int32_t* k;                      // position in the order of the window's b-th net
  int32_t* solo;                   // 1: ROI extracted inline (the batched one overflowed)
  int32_t* st;                     // status of the b-th search
  int32_t* len;                    // path length of the b-th search
  int32_t* box;                    // [4] footprint box
  unsigned long long* stats;       // [4] the b-th search's statistics, added on acceptance
  int32_t* inorder;                // 1: no pending net precedes the b-th net
};

__host__ __device__ inline size_t win_ctl_layout(int32_t slots, char* base, WinCtl** c, WinSlots* s) {
  size_t off = round256(sizeof(WinCtl));
  const size_t k = (size_t)slots;
  char* p[7];
  const size_t sz[7] = {4 * k, 4 * k, 4 * k, 4 * k, 16 * k, 32 * k, 4 * k};
  for (int i = 0; i < 7; ++i) {
    p[i] = base ? base + off : nullptr;
    off += round256(sz[i]);
  }
  if (c) *c = (WinCtl*)base;
  if (s) {
    s->k = (int32_t*)p[0];
    s->solo = (int32_t*)p[1];
    s->st = (int32_t*)p[2];
    s->len = (int32_t*)p[3];
    s->box = (int32_t*)p[4];
    s->stats = (unsigned long long*)p[5];
    s->inorder = (int32_t*)p[6];
  }
  return off;
}

constexpr unsigned kWinBarSpin = 1u << 24;

// Bounded grid barrier (monotone arrival counter); false once any CTA gave up.
__device__ bool win_barrier(WinCtl* c, unsigned long long& target, int* s_flag) {
  __syncthreads();
  if (threadIdx.x == 0) {
    target += gridDim.x;
    int ok = 1;
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
    asm volatile("red.relaxed.gpu.global.add.u64 [%0], 1;" ::"l"(&c->bar_count) : "memory");
    unsigned it = 0;
    while (true) {
      unsigned long long v;
      asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(&c->bar_count) : "memory");
      if (v >= target) break;
      if (++it > kWinBarSpin || *(volatile int32_t*)&c->bar_err) {
        atomicExch(&c->bar_err, 1);
        ok = 0;
        break;
      }
      if (it > 64) __nanosleep(64);
    }
    *s_flag = ok;
  }
  __syncthreads();
  return *s_flag != 0;
}

__device__ __forceinline__ bool boxes_meet(const int* a, const int* b) {
  return !(a[1] < b[0] || b[1] < a[0] || a[3] < b[2] || b[3] < a[2]);
}

// Copies a path found into scratch to the net's store slot and commits it.
__device__ int commit_from(const ogr_graph& g, const ogr_state& st, const ogr_net_table& t, const ogr_pass_args& pa,
                           int32_t n, const int32_t* path, int32_t len, int32_t* s_via, int* s_flags) {
  int32_t* slot = t.store_path + (int64_t)n * t.slot_cap;
  for (int i = threadIdx.x; i < len; i += blockDim.x) slot[i] = path[i];
  __syncthreads();
  const int rc = apply_path_dev(g, st, slot, len, t.net_id[n], +1, pa.pres_fac, pa.live,
                                t.store_arcs + (int64_t)n * 2 * t.slot_cap, s_via, s_flags);
  if (threadIdx.x == 0 && rc == OGR_OK) t.store_len[n] = len;
  return rc;
}

// The ROI nets of a pass (pa.order[0..count)) in windows of mutually disjoint
// footprints.  CTA 0 forms each window; CTA b rips up and searches its net
// into scratch; then either every net commits (no failure) or CTA 0 commits in
// order up to the first failed net, undoes the later nets' rip-ups and runs
// the failed net's fallback.
template <int L>
__global__ void __launch_bounds__(kThreads, 1)
window_pass_kernel(ogr_graph g, ogr_state st, ogr_net_table t, ogr_pass_args pa, ogr_roi_batch rb, char* slot_base,
                   size_t slot_bytes, int32_t rmax, int32_t* scratch, char* ctl_base, Ws w, int32_t look,
                   unsigned long long* discarded) {
  __shared__ Shared sh;
  __shared__ int32_t s_via[kMaxViaNodes];
  __shared__ int s_flags[2];
  __shared__ int s_bar;
  __shared__ int s_box[4];
  __shared__ int s_skip[4 * kMaxSkip];
  __shared__ int s_win[4];
  WinCtl* c;
  WinSlots ws;
  win_ctl_layout(gridDim.x, ctl_base, &c, &ws);
  const int b = blockIdx.x, tid = threadIdx.x, G = gridDim.x;
  if (w.result[0] < 0) return;  // uniform: an earlier step of this pass failed
  Ws mine;
  ws_slot_layout(g.num_nodes, rmax, slot_base + (size_t)b * slot_bytes, &mine);
  int32_t* my_path = scratch + (int64_t)b * t.slot_cap;
  unsigned long long* stats = reinterpret_cast<unsigned long long*>(pa.stats);
  const int32_t plane = g.nx * g.ny;
  unsigned long long target = 0;
  while (true) {
    // 1. window formation (CTA 0).  Nets are taken in order from the first
    // pending one while their footprints (ROI box and old-path box) are
    // pairwise disjoint.  With look > 0 a clashing net is skipped (it stays
    // pending) and the scan goes on: a later net joins only if it is also
    // disjoint from every skipped net's footprint grown to the bound of its
    // fallback ROI (terminals +- fallback BFS depth + halo), so it commutes
    // with the skipped nets whatever they do when their turn comes.
    // Pending = net_status still -1 (set before the launch).
    if (b == 0) {
      if (tid == 0) {
        int cur = c->cursor;
        while (cur < pa.count && pa.net_status[cur] != -1) ++cur;
        c->cursor = cur;
        s_win[0] = cur;
      }
      __syncthreads();
      const int k0 = s_win[0];
      int W = 0, nskip = 0;
      for (int k = k0; k < pa.count && W < G && k - k0 < 4 * G; ++k) {
        if (*(volatile int32_t*)&pa.net_status[k] != -1) continue;   // done out of order earlier
        const int32_t n = pa.order[k];
        const int32_t R = rb.roi_len[n];
        if (R <= 0) {
          if (W == 0 && nskip == 0) {
            if (tid == 0) { ws.k[0] = k; ws.solo[0] = 1; ws.inorder[0] = 1; }
            W = 1;
          }
          break;
        }
        if (tid == 0) {
          for (int q = 0; q < 4; ++q) s_box[q] = rb.roi_box[4 * n + q];
        }
        __syncthreads();
        const int32_t ol = t.store_len[n];
        const int32_t* op = t.store_path + (int64_t)n * t.slot_cap;
        for (int i = tid; i < ol; i += kThreads) {
          const int32_t r = op[i] % plane;
          const int x = r % g.nx, y = r / g.nx;
          atomicMin(&s_box[0], x); atomicMax(&s_box[1], x);
          atomicMin(&s_box[2], y); atomicMax(&s_box[3], y);
        }
        __syncthreads();
        bool clash = false;
        for (int m = 0; m < W && !clash; ++m) clash = boxes_meet(s_box, ws.box + 4 * m);
        for (int q = 0; q < nskip && !clash; ++q) clash = boxes_meet(s_box, s_skip + 4 * q);
        if (clash) {
          if (nskip >= look) break;   // no look-ahead left: the window ends here
          if (tid == 0) {
            const int32_t sr = t.net_src[n] % plane, dr = t.net_dst[n] % plane;
            const int sx = sr % g.nx, sy = sr / g.nx, dx = dr % g.nx, dy = dr / g.nx;
            const int m = t.net_depth[2 * n + 1] + t.net_halo[2 * n + 1];
            int* q = s_skip + 4 * nskip;
            q[0] = min(s_box[0], min(sx, dx) - m);
            q[1] = max(s_box[1], max(sx, dx) + m);
            q[2] = min(s_box[2], min(sy, dy) - m);
            q[3] = max(s_box[3], max(sy, dy) + m);
          }
          __syncthreads();
          ++nskip;
          continue;
        }
        if (tid == 0) {
          ws.k[W] = k;
          ws.solo[W] = 0;
          ws.inorder[W] = nskip == 0 ? 1 : 0;
          for (int q = 0; q < 4; ++q) ws.box[4 * W + q] = s_box[q];
        }
        __syncthreads();
        ++W;
      }
      if (tid == 0) c->wsize = W;
    }
    if (!win_barrier(c, target, &s_bar)) break;
    const int W = *(volatile int32_t*)&c->wsize;
    if (W == 0 || *(volatile int32_t*)&c->error) break;
    // 2. rip-up and search, one net per CTA, paths into scratch
    if (b < W) {
      const int32_t k = ws.k[b];
      const int32_t n = pa.order[k];
      const int32_t ol = t.store_len[n];
      int rc = OGR_OK;
      if (ol >= 2)
        rc = apply_path_dev(g, st, t.store_path + (int64_t)n * t.slot_cap, ol, t.net_id[n], -1, pa.pres_fac,
                            pa.live, nullptr, s_via, s_flags);
      if (tid < 4) ws.stats[4 * b + tid] = 0ull;
      __syncthreads();
      if (rc == OGR_OK) {
        const ogr_net_args a = ogr_pass_net_args(t, pa, n, 0);
        if (ws.solo[b]) {
          search_net<L>(sh, g, st, a, w, my_path, t.slot_cap, ws.stats + 4 * b);
        } else {
          StageClock clk;
          clk.start();
          if (tid == 0) sh.status = OGR_OK;
          __syncthreads();
          sssp_roi<false, L>(sh, g, st, a, mine, rb.roi_pool + (int64_t)n * rb.roi_cap, rb.roi_len[n], my_path,
                             t.slot_cap,
                   ws.stats + 4 * b, clk);
        }
        if (tid == 0) {
          ws.st[b] = sh.status;
          ws.len[b] = sh.len;
          if (sh.status < 0) atomicExch(&c->error, sh.status);
        }
      } else if (tid == 0) {
        atomicExch(&c->error, rc);
      }
    }
    if (!win_barrier(c, target, &s_bar)) break;
    if (*(volatile int32_t*)&c->error) break;
    // 3. commit
    int ff = W;
    for (int m = 0; m < W; ++m)
      if (ws.st[m] != OGR_OK) { ff = m; break; }
    // With the pass's fallbacks used up (the count only grows, and only CTA 0
    // writes it, before a barrier) a failed member takes no fallback: it stays
    // unrouted with its old path ripped up, the state every member's search
    // already saw, so every member's result is the sequential pass's and all
    // of them are final -- in or out of order.
    const bool no_fallback = (int)__ldcg(reinterpret_cast<const long long*>(&w.result[2])) >= pa.fallback_quota;
    if (ff == W || no_fallback) {
      if (b < W) {
        const int32_t k = ws.k[b], n = pa.order[k];
        if (tid < 4) atomicAdd(&stats[tid], ws.stats[4 * b + tid]);
        if (ws.st[b] == OGR_OK) {
          const int rc = commit_from(g, st, t, pa, n, my_path, ws.len[b], s_via, s_flags);
          if (tid == 0) {
            pa.net_status[k] = 0;
            if (rc != OGR_OK) atomicExch(&c->error, rc);
          }
        } else if (tid == 0) {
          t.store_len[n] = 0;
          pa.net_status[k] = 1;
        }
      }
    } else if (b == 0) {
      int rc = OGR_OK;
      for (int m = 0; m < ff && rc == OGR_OK; ++m) {
        const int32_t k = ws.k[m], n = pa.order[k];
        rc = commit_from(g, st, t, pa, n, scratch + (int64_t)m * t.slot_cap, ws.len[m], s_via, s_flags);
        if (tid < 4) atomicAdd(&stats[tid], ws.stats[4 * m + tid]);
        if (tid == 0) pa.net_status[k] = 0;
        __syncthreads();
      }
      // A failed net with pending nets before it (taken out of order) must
      // not take its fallback yet: it is undone like the later members and
      // stays pending, to be searched again when its turn comes.
      const bool defer = !ws.inorder[ff];
      for (int m = defer ? ff : ff + 1; m < W && rc == OGR_OK; ++m) {   // undo the later rip-ups
        if (discarded != nullptr && tid == 0) {
          atomicAdd(&discarded[0], 1ull);
          atomicAdd(&discarded[1], ws.stats[4 * m + 0]);
          atomicAdd(&discarded[2], ws.stats[4 * m + 1]);
        }
        const int32_t n = pa.order[ws.k[m]];
        const int32_t ol = t.store_len[n];
        if (ol >= 2)
          rc = apply_path_dev(g, st, t.store_path + (int64_t)n * t.slot_cap, ol, t.net_id[n], +1, pa.pres_fac,
                              pa.live, nullptr, s_via, s_flags);
      }
      const int32_t kf = ws.k[ff], nf = pa.order[kf];
      if (defer) {
        if (tid == 0 && rc != OGR_OK) atomicExch(&c->error, rc);
      } else {
      if (tid < 4) atomicAdd(&stats[tid], ws.stats[4 * ff + tid]);
      if (tid == 0) t.store_len[nf] = 0;
      __syncthreads();
      int flags = 0, fin = ws.st[ff], len = 0;
      const int used = (int)w.result[2];
      if (rc == OGR_OK && fin != OGR_OK && used < pa.fallback_quota) {
        const ogr_net_args a = ogr_pass_net_args(t, pa, nf, 1);
        search_net<L>(sh, g, st, a, w, t.store_path + (int64_t)nf * t.slot_cap, t.slot_cap, stats);
        fin = sh.status;
        len = sh.len;
        flags |= 2;
        if (tid == 0) w.result[2] = used + 1;
        if (fin < 0) rc = fin;
      }
      __syncthreads();
      if (rc == OGR_OK && fin == OGR_OK) {
        rc = apply_path_dev(g, st, t.store_path + (int64_t)nf * t.slot_cap, len, t.net_id[nf], +1, pa.pres_fac,
                            pa.live, t.store_arcs + (int64_t)nf * 2 * t.slot_cap, s_via, s_flags);
        if (tid == 0 && rc == OGR_OK) t.store_len[nf] = len;
      } else {
        flags |= 1;
      }
      if (tid == 0) {
        pa.net_status[kf] = flags;
        if (rc != OGR_OK) atomicExch(&c->error, rc);
      }
      }
    }
    if (!win_barrier(c, target, &s_bar)) break;
    if (*(volatile int32_t*)&c->error) break;
  }
  if (b == 0 && tid == 0) {
    if (*(volatile int32_t*)&c->bar_err) w.result[0] = OGR_ERR_TIMEOUT;
    else if (*(volatile int32_t*)&c->error) w.result[0] = *(volatile int32_t*)&c->error;
  }
}

__global__ void window_ws_init_kernel(char* base, int32_t slots, size_t slot_bytes, int32_t N, int32_t rmax) {
  for (int32_t sidx = 0; sidx < slots; ++sidx) {
    Ws t;
    ws_slot_layout(N, rmax, base + (size_t)sidx * slot_bytes, &t);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
      t.g2r[i] = -1;
  }
}

// Long nets of a pass run as three launches each: this rip-up, the
// whole-lattice search on every SM (fullgraph.cu), then pass_full_tail_kernel.
__global__ void __launch_bounds__(kThreads, 1)
pass_ripup_kernel(ogr_graph g, ogr_state st, ogr_net_table t, ogr_pass_args pa, int32_t k, Ws w) {
  __shared__ int32_t s_via[kMaxViaNodes];
  __shared__ int s_flags[2];
  if (w.result[0] < 0) return;
  const int32_t n = pa.order[k];
  const int32_t old_len = t.store_len[n];
  if (old_len >= 2) {
    const int rc = apply_path_dev(g, st, t.store_path + (int64_t)n * t.slot_cap, old_len, t.net_id[n], -1,
                                  pa.pres_fac, pa.live, nullptr, s_via, s_flags);
    if (rc != OGR_OK) {
      if (threadIdx.x == 0) w.result[0] = rc;
      return;
    }
  }
  if (threadIdx.x == 0) t.store_len[n] = 0;
}

// After the whole-lattice search of net order[k]: the fallback ROI search if
// it failed and the pass has fallbacks left, then the commit.
template <int L>
__global__ void __launch_bounds__(kThreads, 1)
pass_full_tail_kernel(ogr_graph g, ogr_state st, ogr_net_table t, ogr_pass_args pa, int32_t k, Ws w,
                      const int32_t* full_res) {
  __shared__ Shared sh;
  __shared__ int32_t s_via[kMaxViaNodes];
  __shared__ int s_flags[2];
  if (w.result[0] < 0) return;
  const int32_t n = pa.order[k];
  int32_t* slot = t.store_path + (int64_t)n * t.slot_cap;
  int32_t* arcs = t.store_arcs + (int64_t)n * 2 * t.slot_cap;
  int fin = full_res[0];
  int len = full_res[1];
  if (fin < 0) {
    if (threadIdx.x == 0) w.result[0] = fin;
    return;
  }
  int flags = 0;
  const int used = (int)w.result[2];
  if (fin != OGR_OK && used < pa.fallback_quota) {
    const ogr_net_args a = ogr_pass_net_args(t, pa, n, 1);
    search_net<L>(sh, g, st, a, w, slot, t.slot_cap, reinterpret_cast<unsigned long long*>(pa.stats));
    fin = sh.status;
    len = sh.len;
    if (fin < 0) {
      if (threadIdx.x == 0) w.result[0] = fin;
      return;
    }
    flags |= 2;
    if (threadIdx.x == 0) w.result[2] = used + 1;
  }
  __syncthreads();
  if (fin == OGR_OK) {
    const int rc = apply_path_dev(g, st, slot, len, t.net_id[n], +1, pa.pres_fac, pa.live, arcs, s_via, s_flags);
    if (rc != OGR_OK) {
      if (threadIdx.x == 0) w.result[0] = rc;
      return;
    }
    if (threadIdx.x == 0) t.store_len[n] = len;
  } else {
    flags |= 1;
  }
  if (threadIdx.x == 0) pa.net_status[k] = flags;
}

}  // namespace

extern "C" size_t ogr_route_workspace_bytes(int32_t num_nodes) { return ws_layout(num_nodes, nullptr, nullptr); }

extern "C" size_t ogr_bfs_workspace_bytes(int32_t num_nodes, int64_t qcap, int32_t slots) {
  return bfs_slot_bytes(num_nodes, qcap) * (size_t)slots;
}

extern "C" int ogr_bfs_workspace_init(void* ws, int32_t num_nodes, int64_t qcap, int32_t slots, void* stream) {
  if (!ws || slots < 1 || qcap < 1) return OGR_ERR_ARG;
  bfs_init_kernel<<<ogr_blocks(num_nodes, 256), 256, 0, ogr_stream(stream)>>>(
      (char*)ws, slots, bfs_slot_bytes(num_nodes, qcap), num_nodes, qcap);
  OGR_LAUNCH_CHECK();
  return OGR_OK;
}

extern "C" size_t ogr_window_workspace_bytes(int32_t num_nodes, int32_t max_roi_nodes, int32_t slots) {
  const int32_t r = max_roi_nodes < num_nodes ? max_roi_nodes : num_nodes;
  return ws_slot_layout(num_nodes, r, nullptr, nullptr) * (size_t)(slots > 0 ? slots : 0);
}

extern "C" int ogr_window_workspace_init(void* ws, int32_t num_nodes, int32_t max_roi_nodes, int32_t slots,
                                         void* stream) {
  if (!ws || slots < 1 || num_nodes < 1 || max_roi_nodes < 1) return OGR_ERR_ARG;
  const int32_t r = max_roi_nodes < num_nodes ? max_roi_nodes : num_nodes;
  window_ws_init_kernel<<<ogr_blocks(num_nodes, 256), 256, 0, ogr_stream(stream)>>>(
      (char*)ws, slots, ws_slot_layout(num_nodes, r, nullptr, nullptr), num_nodes, r);
  OGR_LAUNCH_CHECK();
  return OGR_OK;
}

extern "C" size_t ogr_window_ctl_bytes(int32_t slots) { return win_ctl_layout(slots, nullptr, nullptr, nullptr); }

extern "C" int ogr_window_lookahead(int32_t nets, int32_t* current) {
  if (nets < -1 || nets > kMaxSkip) return OGR_ERR_ARG;
  if (nets >= 0) g_window_look = nets;
  if (current) *current = g_window_look;
  return OGR_OK;
}

extern "C" int ogr_search_lanes(int32_t lanes, int32_t* current) {
  if (lanes != 0 && lanes != 2 && lanes != 4 && lanes != 8 && lanes != 16) return OGR_ERR_ARG;
  if (lanes != 0) g_search_lanes = lanes;
  if (current) *current = g_search_lanes;
  return OGR_OK;
}

extern "C" int ogr_search_profile(int64_t* out16, int32_t reset) {
  if (!out16) return OGR_ERR_ARG;
  OGR_CUDA_TRY(cudaMemcpyFromSymbol(out16, g_stage, sizeof(unsigned long long) * 16));
  if (reset) {
    unsigned long long z[16] = {};
    OGR_CUDA_TRY(cudaMemcpyToSymbol(g_stage, z, sizeof(z)));
  }
  return OGR_OK;
}

extern "C" int ogr_route_workspace_init(void* ws, size_t bytes, int32_t N, void* stream) {
  if (!ws || bytes < ogr_route_workspace_bytes(N)) return OGR_ERR_CAPACITY;
  Ws w;
  ws_layout(N, (char*)ws, &w);
  ws_init_kernel<<<ogr_blocks(N, 256), 256, 0, ogr_stream(stream)>>>(w, N);
  OGR_LAUNCH_CHECK();
  return OGR_OK;
}

extern "C" int ogr_find_path(const ogr_graph* g, const ogr_state* st, const ogr_net_args* net, void* ws,
                             size_t bytes, int32_t* path_out, int32_t path_cap, int32_t* path_len_out,
                             int64_t* stats, void* stream) {
  if (!g || !st || !net || !ws || !path_out || !path_len_out) return OGR_ERR_ARG;
  if (bytes < ogr_route_workspace_bytes(g->num_nodes)) return OGR_ERR_CAPACITY;
  if (net->src < 0 || net->dst < 0 || net->src >= g->num_nodes || net->dst >= g->num_nodes) return OGR_ERR_ARG;
  Ws w;
  ws_layout(g->num_nodes, (char*)ws, &w);
  cudaStream_t s = ogr_stream(stream);
  OGR_WITH_LANES(L, find_path_kernel<L><<<1, kThreads, 0, s>>>(*g, *st, *net, w, path_out, path_cap, stats));
  OGR_LAUNCH_CHECK();
  int64_t res[2];
  OGR_CUDA_TRY(cudaMemcpyAsync(res, w.result, sizeof(res), cudaMemcpyDeviceToHost, s));
  OGR_CUDA_TRY(cudaStreamSynchronize(s));
  *path_len_out = (res[0] == OGR_OK) ? (int32_t)res[1] : 0;
  return (int)res[0];
}

extern "C" int ogr_find_path_roi(const ogr_graph* g, const float* costs, const int32_t* roi_nodes, int32_t n_roi,
                                 const float* roi_penalty, int32_t src, int32_t dst, void* ws, size_t bytes,
                                 int32_t* path_out, int32_t path_cap, int32_t* path_len_out, int64_t* stats,
                                 void* stream) {
  if (!g || !costs || !roi_nodes || !ws || !path_out || !path_len_out || n_roi < 0 || n_roi > g->num_nodes)
    return OGR_ERR_ARG;
  if (bytes < ogr_route_workspace_bytes(g->num_nodes)) return OGR_ERR_CAPACITY;
  if (src < 0 || dst < 0 || src >= g->num_nodes || dst >= g->num_nodes) return OGR_ERR_ARG;
  *path_len_out = 0;
  if (n_roi == 0) return OGR_NO_PATH;
  Ws w;
  ws_layout(g->num_nodes, (char*)ws, &w);
  ogr_state st{};
  st.total_cost = const_cast<float*>(costs);
  ogr_net_args a{};
  a.net_id = -1;
  a.src = src;
  a.dst = dst;
  a.full_graph = 0;
  a.penalty_enabled = 0;
  cudaStream_t s = ogr_stream(stream);
  OGR_WITH_LANES(L, find_path_given_roi_kernel<L><<<1, kThreads, 0, s>>>(*g, st, a, w, roi_nodes, n_roi, roi_penalty,
                                                                          path_out, path_cap, stats));
  OGR_LAUNCH_CHECK();
  int64_t res[2];
  OGR_CUDA_TRY(cudaMemcpyAsync(res, w.result, sizeof(res), cudaMemcpyDeviceToHost, s));
  OGR_CUDA_TRY(cudaStreamSynchronize(s));
  *path_len_out = (res[0] == OGR_OK) ? (int32_t)res[1] : 0;
  return (int)res[0];
}

extern "C" size_t ogr_multi_workspace_bytes(int32_t num_nodes) {
  return ogr_route_workspace_bytes(num_nodes) + 2 * round256(8 * (size_t)(num_nodes > 0 ? num_nodes : 0));
}

extern "C" int ogr_find_path_multi(const ogr_graph* g, const float* costs, const int32_t* roi_nodes, int32_t n_roi,
                                   const float* roi_penalty, const int32_t* seeds, const double* seed_cost,
                                   int32_t n_seeds, const int32_t* targets, const double* target_cost,
                                   int32_t n_targets, void* ws, size_t bytes, int32_t* path_out, int32_t path_cap,
                                   int32_t* path_len_out, int64_t* stats, void* stream) {
  if (!g || !costs || !roi_nodes || !ws || !path_out || !path_len_out || n_roi < 0 || n_roi > g->num_nodes ||
      n_seeds < 0 || n_targets < 0 || (n_seeds > 0 && (!seeds || !seed_cost)) ||
      (n_targets > 0 && (!targets || !target_cost)))
    return OGR_ERR_ARG;
  if (bytes < ogr_multi_workspace_bytes(g->num_nodes)) return OGR_ERR_CAPACITY;
  *path_len_out = 0;
  if (n_roi == 0 || n_seeds == 0 || n_targets == 0) return OGR_NO_PATH;
  Ws w;
  const size_t base = ws_layout(g->num_nodes, (char*)ws, &w);
  MultiSeeds ms{};
  ms.seeds = seeds;
  ms.seed_cost = seed_cost;
  ms.nseeds = n_seeds;
  ms.targets = targets;
  ms.target_cost = target_cost;
  ms.ntargets = n_targets;
  ms.init = (double*)((char*)ws + base);
  ms.tcost = (double*)((char*)ws + base + round256(8 * (size_t)g->num_nodes));
  ogr_state st{};
  st.total_cost = const_cast<float*>(costs);
  ogr_net_args a{};
  a.net_id = -1;
  a.src = -1;
  a.dst = -1;
  a.full_graph = 0;
  a.penalty_enabled = 0;
  cudaStream_t s = ogr_stream(stream);
  OGR_WITH_LANES(L, find_path_multi_kernel<L><<<1, kThreads, 0, s>>>(*g, st, a, w, roi_nodes, n_roi, roi_penalty, ms,
                                                                      path_out, path_cap, stats));
  OGR_LAUNCH_CHECK();
  int64_t res[2];
  OGR_CUDA_TRY(cudaMemcpyAsync(res, w.result, sizeof(res), cudaMemcpyDeviceToHost, s));
  OGR_CUDA_TRY(cudaStreamSynchronize(s));
  *path_len_out = (res[0] == OGR_OK) ? (int32_t)res[1] : 0;
  return (int)res[0];
}

extern "C" int ogr_extract_roi(const ogr_graph* g, const ogr_net_args* net, void* ws, size_t bytes,
                               int32_t* roi_out, int32_t roi_cap, int32_t* roi_len_out, void* stream) {
  if (!g || !net || !ws || !roi_out || !roi_len_out) return OGR_ERR_ARG;
  if (bytes < ogr_route_workspace_bytes(g->num_nodes)) return OGR_ERR_CAPACITY;
  if (!net->full_graph && roi_cap < (net->max_roi_nodes < g->num_nodes ? net->max_roi_nodes : g->num_nodes))
    return OGR_ERR_ARG;
  Ws w;
  ws_layout(g->num_nodes, (char*)ws, &w);
  cudaStream_t s = ogr_stream(stream);
  roi_kernel<<<1, kThreads, 0, s>>>(*g, *net, w, roi_out, roi_cap);
  OGR_LAUNCH_CHECK();
  int64_t res[2];
  OGR_CUDA_TRY(cudaMemcpyAsync(res, w.result, sizeof(res), cudaMemcpyDeviceToHost, s));
  OGR_CUDA_TRY(cudaStreamSynchronize(s));
  *roi_len_out = (int32_t)res[1];
  return (int)res[0];
}

extern "C" int ogr_paths_commit(const ogr_graph* g, const ogr_state* st, const int32_t* nodes, const int32_t* offsets,
                                const int32_t* net_ids, int32_t n_paths, int32_t* arcs_out, int32_t* store_path,
                                int32_t* store_len, int32_t* store_arcs, const int32_t* store_slot, int32_t slot_cap,
                                int32_t* status_dev, void* stream) {
  if (!g || !st || n_paths < 0 || !status_dev) return OGR_ERR_ARG;
  if (n_paths == 0) return OGR_OK;
  if (!nodes || !offsets || !net_ids || !arcs_out ||
      ((store_path || store_len || store_arcs) && (!store_slot || slot_cap < 2)))
    return OGR_ERR_ARG;
  cudaStream_t s = ogr_stream(stream);
  OGR_CUDA_TRY(cudaMemsetAsync(status_dev, 0, sizeof(int32_t), s));
  const int grid = n_paths < 152 * 8 ? n_paths : 152 * 8;
  paths_commit_kernel<<<grid, kApplyThreads, 0, s>>>(*g, *st, nodes, offsets, net_ids, n_paths, arcs_out, store_path,
                                                      store_len, store_arcs, store_slot, slot_cap, status_dev);
  OGR_LAUNCH_CHECK();
  return OGR_OK;
}

extern "C" int ogr_path_apply(const ogr_graph* g, const ogr_state* st, const int32_t* path, int32_t len,
                              int32_t net_id, int32_t sign, float pres_fac_f32, int32_t live, int32_t* arcs_out,
                              int32_t* status_dev, void* stream) {
  if (!g || !st || !path || !status_dev || len < 2 || (sign != 1 && sign != -1)) return OGR_ERR_ARG;
  path_apply_kernel<<<1, kApplyThreads, 0, ogr_stream(stream)>>>(*g, *st, path, len, net_id, sign, pres_fac_f32,
                                                                   live, arcs_out, status_dev);
  OGR_LAUNCH_CHECK();
  return OGR_OK;
}

// Window-pass grid size: one 1024-thread CTA per SM, at most `slots`.
template <int L>
static int window_grid_for(int slots) {
  static int per_dev[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
  if (per_dev[dev] == 0) {
    int sms = 0, per_sm = 0, coop = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, window_pass_kernel<L>, kThreads, 0) != cudaSuccess)
      return 0;
    per_dev[dev] = sms * per_sm;
  }
  return slots < per_dev[dev] ? slots : per_dev[dev];
}

static int window_grid(int slots) {
  int grid = 0;
  OGR_WITH_LANES(L, grid = window_grid_for<L>(slots));
  return grid;
}

extern "C" int ogr_route_pass(const ogr_graph* g, const ogr_state* st, const ogr_net_table* t,
                              const ogr_pass_args* pa, const ogr_roi_batch* rb, void* ws, size_t bytes,
                              const uint8_t* order_full, void* full_ws, size_t full_bytes,
                              const ogr_window_args* win, int32_t* status_out, void* stream) {
  if (!g || !st || !t || !pa || !ws || !status_out) return OGR_ERR_ARG;
  if (bytes < ogr_route_workspace_bytes(g->num_nodes)) return OGR_ERR_CAPACITY;
  if (pa->count < 0 || t->slot_cap < 2) return OGR_ERR_ARG;
  if (pa->count == 0) {
    *status_out = OGR_OK;
    return OGR_OK;
  }
  if (!pa->order || !pa->net_status || !pa->stats) return OGR_ERR_ARG;
  const bool batch = rb != nullptr && rb->slots > 0;
  const int32_t need_cap = pa->max_roi_nodes < g->num_nodes ? pa->max_roi_nodes : g->num_nodes;
  if (batch && (!rb->bfs_ws || !rb->roi_pool || !rb->roi_len || !rb->next || rb->roi_cap < need_cap))
    return OGR_ERR_ARG;
  bool any_full = false;
  if (order_full)
    for (int32_t k = 0; k < pa->count; ++k) any_full = any_full || order_full[k] != 0;
  if (any_full && (!full_ws || full_bytes < ogr_full::workspace_bytes(g->num_nodes, g->num_edges)))
    return OGR_ERR_CAPACITY;
  Ws w;
  ws_layout(g->num_nodes, (char*)ws, &w);
  cudaStream_t s = ogr_stream(stream);
  // result[0] = first error of the pass, result[2] = fallbacks used so far
  OGR_CUDA_TRY(cudaMemsetAsync(w.result, 0, 64, s));
  ogr_roi_batch rbv{};
  if (batch) {
    rbv = *rb;
    OGR_CUDA_TRY(cudaMemsetAsync(rbv.next, 0, sizeof(int32_t), s));
    roi_batch_kernel<<<rbv.slots, kThreads, 0, s>>>(*g, *t, *pa, rbv);
    OGR_LAUNCH_CHECK();
  }
  const bool windows = win != nullptr && win->slots > 0 && batch && rbv.roi_box != nullptr;
  int grid = 0;
  if (windows) {
    if (!win->ws || !win->scratch || !win->ctl ||
        win->slot_bytes < ogr_window_workspace_bytes(g->num_nodes, pa->max_roi_nodes, 1))
      return OGR_ERR_ARG;
    grid = window_grid(win->slots);
    if (grid < 1) return OGR_ERR_CUDA;
  }
  // one run of ROI nets: batched windows, or the single-CTA sequential pass
  auto roi_segment = [&](const ogr_pass_args& seg) -> int {
    if (!windows) {
      OGR_WITH_LANES(L, route_pass_kernel<L><<<1, kThreads, 0, s>>>(*g, *st, *t, seg, rbv, batch ? 1 : 0, w));
      OGR_LAUNCH_CHECK();
      return OGR_OK;
    }
    OGR_CUDA_TRY(cudaMemsetAsync(win->ctl, 0, ogr_window_ctl_bytes(grid), s));
    // every net of the segment starts pending (-1); the window pass sets its status when done
    OGR_CUDA_TRY(cudaMemsetAsync(seg.net_status, 0xff, sizeof(int32_t) * (size_t)seg.count, s));
    int32_t lookv = g_window_look < 0 ? 0 : (g_window_look > kMaxSkip ? kMaxSkip : g_window_look);
    ogr_graph gv = *g;
    ogr_state sv = *st;
    ogr_net_table tv = *t;
    ogr_pass_args pv = seg;
    char* slot_base = (char*)win->ws;
    size_t slot_bytes = win->slot_bytes;
    int32_t rmax = pa->max_roi_nodes < g->num_nodes ? pa->max_roi_nodes : g->num_nodes;
    int32_t* scratch = win->scratch;
    char* ctl = (char*)win->ctl;
    Ws wv = w;
    unsigned long long* discarded = reinterpret_cast<unsigned long long*>(win->discarded);
    void* args[] = {&gv, &sv, &tv, &pv, &rbv, &slot_base, &slot_bytes, &rmax, &scratch, &ctl, &wv, &lookv,
                    &discarded};
    const void* wk = nullptr;
    OGR_WITH_LANES(L, wk = (const void*)window_pass_kernel<L>);
    OGR_CUDA_TRY(cudaLaunchCooperativeKernel(wk, dim3(grid), dim3(kThreads), args, 0,
                                             s));
    return OGR_OK;
  };
  if (!any_full) {
    const int rc = roi_segment(*pa);
    if (rc != OGR_OK) return rc;
  } else {
    // Runs of ROI nets go through one single-CTA launch each; every long net
    // gets the whole GPU for its search.  Same order, same state updates.
    int32_t* full_res = ogr_full::result_words(full_ws, g->num_nodes, g->num_edges);
    int32_t k = 0;
    while (k < pa->count) {
      if (order_full[k]) {
        pass_ripup_kernel<<<1, kThreads, 0, s>>>(*g, *st, *t, *pa, k, w);
        OGR_LAUNCH_CHECK();
        ogr_full::Job job{};
        job.from_pass = 1;
        job.t = *t;
        job.pa = *pa;
        job.k = k;
        job.pass_result = w.result;
        job.stats = reinterpret_cast<unsigned long long*>(pa->stats);
        const int rc = ogr_full::launch(*g, *st, job, full_ws, s);
        if (rc != OGR_OK) return rc;
        OGR_WITH_LANES(L, pass_full_tail_kernel<L><<<1, kThreads, 0, s>>>(*g, *st, *t, *pa, k, w, full_res));
        OGR_LAUNCH_CHECK();
        ++k;
      } else {
        int32_t k1 = k;
        while (k1 < pa->count && !order_full[k1]) ++k1;
        ogr_pass_args seg = *pa;
        seg.order = pa->order + k;
        seg.count = k1 - k;
        seg.net_status = pa->net_status + k;
        const int rc = roi_segment(seg);
        if (rc != OGR_OK) return rc;
        k = k1;
      }
    }
  }
  int64_t res;
  OGR_CUDA_TRY(cudaMemcpyAsync(&res, w.result, sizeof(res), cudaMemcpyDeviceToHost, s));
  OGR_CUDA_TRY(cudaStreamSynchronize(s));
  *status_out = (int32_t)res;
  return res < 0 ? (int)res : OGR_OK;
}

// ---- allocation-free search ----------------------------------------------------
// Some hosts cannot hand this library a workspace: a plugin loaded into an
// application that owns the device allocator, or a serving process that
// reserves its whole memory budget at start-up and forbids allocations on the
// request path.  ogr_find_path_noalloc runs the same search as ogr_find_path
// with its scratch in a fixed device array that lives in this library's image
// (resident on every GPU that loads the library until the process exits).
//
// Limits and rules:
//  - at most OGR_NOALLOC_MAX_NODES lattice nodes; larger graphs are rejected
//    with OGR_ERR_CAPACITY before anything is launched;
//  - the first call on a device looks up the array's device address for that
//    device (cudaGetSymbolAddress); make that first call before any stream
//    capture;
//  - all calls share the one array: each call re-initialises the parts the
//    search needs cleared, and calls that overlap on the GPU (another stream,
//    another host thread) race on it — serialise them.
namespace {

constexpr size_t noalloc_ws_bytes() { return ws_bytes_for((size_t)OGR_NOALLOC_MAX_NODES); }

static __device__ __align__(256) unsigned char g_noalloc_ws[noalloc_ws_bytes()];

constexpr int kMaxDevices = 64;
// Device address of the array per device, looked up on the first call there
// (atomic: concurrent first calls from several host threads store the same
// value).  A device reset invalidates it; the process does not reset here.
std::atomic<void*> g_noalloc_ptr[kMaxDevices] = {};

}  // namespace

extern "C" int ogr_find_path_noalloc(const ogr_graph* g, const ogr_state* st, const ogr_net_args* net,
                                     int32_t* path_out, int32_t path_cap, int32_t* path_len_out, int64_t* stats,
                                     void* stream) {
  if (!g || !st || !net || !path_out || !path_len_out) return OGR_ERR_ARG;
  if (g->num_nodes < 1 || g->num_nodes > OGR_NOALLOC_MAX_NODES) return OGR_ERR_CAPACITY;
  if (net->src < 0 || net->dst < 0 || net->src >= g->num_nodes || net->dst >= g->num_nodes) return OGR_ERR_ARG;
  int dev = 0;
  OGR_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return OGR_ERR_ARG;
  void* base = g_noalloc_ptr[dev].load(std::memory_order_acquire);
  if (base == nullptr) {
    OGR_CUDA_TRY(cudaGetSymbolAddress(&base, g_noalloc_ws));
    g_noalloc_ptr[dev].store(base, std::memory_order_release);
  }
  const size_t need = ws_layout(g->num_nodes, nullptr, nullptr);
  if (need > noalloc_ws_bytes()) return OGR_ERR_CAPACITY;
  Ws w;
  ws_layout(g->num_nodes, (char*)base, &w);
  cudaStream_t s = ogr_stream(stream);
  // The array keeps whatever the previous call left: clear seen[] / g2r[].
  ws_init_kernel<<<ogr_blocks(g->num_nodes, 256), 256, 0, s>>>(w, g->num_nodes);
  OGR_WITH_LANES(L, find_path_kernel<L><<<1, kThreads, 0, s>>>(*g, *st, *net, w, path_out, path_cap, stats));
  OGR_LAUNCH_CHECK();
  int64_t res[2];
  OGR_CUDA_TRY(cudaMemcpyAsync(res, w.result, sizeof(res), cudaMemcpyDeviceToHost, s));
  OGR_CUDA_TRY(cudaStreamSynchronize(s));
  *path_len_out = (res[0] == OGR_OK) ? (int32_t)res[1] : 0;
  return (int)res[0];
}
