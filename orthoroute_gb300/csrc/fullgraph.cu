// A7 for long nets: the exact search over the whole lattice on every SM.
//
// The reference searches nets whose Manhattan length is 125 steps or more on
// the full graph (_route_all, unified_pathfinder.py:8219-8262: roi_nodes =
// arange(N)), so its heap Dijkstra (find_path_roi, :2451-2548) settles every
// node cheaper than dst — most of a 600x400x12 lattice.  This kernel computes
// the same result as the per-CTA search in route.cu (each node takes the
// lexicographic minimum of (float32(alt), L(u), u) over its settled
// in-neighbours; nodes are settled in phases by the IN-criterion) with the
// node states in global memory and all SMs working on each phase.
//
// One phase = two grid-wide steps:
//   E  every node settled last phase claims its unsettled out-neighbours
//      (atomicMax on a per-node stamp: one claimer per node and phase) and
//      the claimer's 16-lane group recomputes the claimed node from all its
//      settled in-neighbours; newly reached nodes join the frontier;
//   S  with T = the smallest frontier label, frontier nodes with label == T
//      or float32 key < float32((T + cin) + pen) are settled.
// T is the minimum of the labels written in E and of the labels carried over
// in the previous S.  Recomputing a node can move its FP64 label within the
// same float32 value in either direction, so T may lie below the true
// minimum; both settling tests only get stricter then (no label equals such
// a T, and the IN bound is monotone in T), the phase settles a subset of what
// it would have, and the next phase's T is exact again.  The result is a
// function of the settled set alone, independent of thread scheduling.
//
// The kernel is launched cooperatively with one grid of fully resident CTAs
// (occupancy API), and its grid barrier gives up after a bounded wait and
// reports OGR_ERR_TIMEOUT.  List appends are staged per CTA in shared memory
// and published with one global atomic per CTA and list.
#include <cooperative_groups.h>

#include "fullgraph.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int kThreads = 512;
constexpr int kSub = 8;                    // lanes per recomputed node
constexpr int kGroups = kThreads / kSub;   // groups per CTA
constexpr int32_t ST_FRONT = 1, ST_DONE = 2;   // state 0 (or another epoch): unreached
constexpr int kStage = 1536;               // staged list entries per CTA and list
constexpr int kClaim = 3072;               // claimed nodes per CTA and phase held in shared memory
constexpr unsigned kBarSpin = 1u << 22;
constexpr int32_t kMaxEpoch = (1 << 29) - 1;

// Node state.  `st` = (epoch << 2) | state: a node whose epoch is not the
// current search's is unreached, so a search clears no per-node memory.
// `stamp` = global phase number of the last claim (monotone across searches).
struct __align__(32) FNode {
  double lab;
  float m32;
  float pen;
  float cin;
  int32_t par;
  int32_t st;
  int32_t stamp;
};
static_assert(sizeof(FNode) == 32, "FNode must fill one 32-byte sector");

struct FCtl {
  alignas(128) unsigned long long bar_count;   // monotone arrival counter
  alignas(128) int32_t bar_err;
  alignas(128) unsigned long long tbits[2];
  alignas(128) int32_t nfront[2];
  alignas(128) int32_t nlog;                   // settled-log length
  alignas(128) int32_t res[4];
  int32_t epoch;                               // persistent across searches
  int32_t gbase;
};

struct FWs {
  FNode* node;
  float* rcost;   // rcost[e] = cost of the arc opposite to e, i.e. into the row's node
  int32_t* fr[2];
  int32_t* log;   // settled nodes in settle order
  FCtl* ctl;
};

constexpr size_t r256(size_t v) { return (v + 255) & ~(size_t)255; }

size_t fws_layout(int32_t N, int64_t E, char* base, FWs* w) {
  size_t off = 0;
  auto take = [&](size_t b) -> char* {
    char* p = base ? base + off : nullptr;
    off += r256(b);
    return p;
  };
  const size_t n = (size_t)N;
  FWs t{};
  t.ctl = (FCtl*)take(sizeof(FCtl));
  t.node = (FNode*)take(32 * n);
  t.rcost = (float*)take(4 * (size_t)E);
  t.fr[0] = (int32_t*)take(4 * n);
  t.fr[1] = (int32_t*)take(4 * n);
  t.log = (int32_t*)take(4 * n);
  if (w) *w = t;
  return off;
}

struct Smem {
  int32_t buf[2][kStage];
  int32_t claim[kClaim];
  int32_t nclaim;
  int32_t cnt[2];
  int32_t base[2];
  unsigned long long tmin;
  int flag;
};

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ int ld_volatile(const int32_t* p) { return *(const volatile int32_t*)p; }

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Tracing counters of the whole-lattice search (read with ogr_full_profile):
// [0] searches, [1] phases, [2] kernel ns, [3] init ns (CTA 0), [4] work ns
// of the E steps and [5] of the S steps (largest CTA total), [6] barrier
// wait ns (CTA 0), [7] statistics + backtrace ns (CTA 0).
__device__ unsigned long long g_full_prof[8];

// Per-CTA timing kept by thread 0.
struct Clock {
  unsigned long long mark, init, e, s, wait;
};

// Grid barrier on a monotone arrival counter: the k-th barrier of a launch
// is passed when the counter reaches k * gridDim.x.  The wait is bounded;
// false when any CTA gave up.  Thread 0 adds the time since the previous
// barrier to *work and the wait to clk.wait.
__device__ bool grid_barrier(FCtl* c, unsigned long long& target, Smem& sm, Clock& clk, unsigned long long* work) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned long long t0 = gtimer();
    *work += t0 - clk.mark;
    target += gridDim.x;
    int ok = 1;
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
    asm volatile("red.relaxed.gpu.global.add.u64 [%0], 1;" ::"l"(&c->bar_count) : "memory");
    unsigned it = 0;
    while (ld_acquire_u64(&c->bar_count) < target) {
      if (++it > kBarSpin || ld_volatile(&c->bar_err)) {
        atomicExch(&c->bar_err, 1);
        ok = 0;
        break;
      }
      if (it > 64) __nanosleep(32);
    }
    sm.flag = ok;
    clk.mark = gtimer();
    clk.wait += clk.mark - t0;
  }
  __syncthreads();
  return sm.flag != 0;
}

__device__ __forceinline__ void stage_push(Smem& sm, int k, int32_t v, int32_t* gl, int32_t* gcnt) {
  const int i = atomicAdd(&sm.cnt[k], 1);
  if (i < kStage)
    sm.buf[k][i] = v;
  else
    gl[atomicAdd(gcnt, 1)] = v;
}

// Publishes lists 0..nl-1 of this CTA (call after __syncthreads, from all
// threads): one global reservation per list, then a coalesced copy.
__device__ __forceinline__ void stage_flush(Smem& sm, int nl, int32_t* gl0, int32_t* gc0, int32_t* gl1,
                                            int32_t* gc1) {
  if (threadIdx.x == 0) {
    for (int k = 0; k < nl; ++k) {
      const int n = min(sm.cnt[k], kStage);
      sm.base[k] = n ? atomicAdd(k == 0 ? gc0 : gc1, n) : 0;
      sm.cnt[k] = n;
    }
  }
  __syncthreads();
  for (int k = 0; k < nl; ++k) {
    const int n = sm.cnt[k], b = sm.base[k];
    int32_t* gl = k == 0 ? gl0 : gl1;
    for (int i = threadIdx.x; i < n; i += kThreads) gl[b + i] = sm.buf[k][i];
  }
}

__device__ __forceinline__ void stage_reset(Smem& sm) {
  if (threadIdx.x == 0) {
    sm.cnt[0] = 0;
    sm.cnt[1] = 0;
    sm.nclaim = 0;
    sm.tmin = ~0ull;
  }
  __syncthreads();
}

// Recomputes node yy from all its settled in-neighbours with W lanes (lane
// `sl` of the tile; W = 1 runs on one thread without shuffles).  A node
// reached for the first time gets its penalty and joins the frontier list.
template <int W, typename Tile>
__device__ __forceinline__ void recompute(Tile& tile, int sl, int32_t yy, int32_t ep2, const ogr_graph& g,
                                          const ogr_state& st, const ogr_net_args& a, const FWs& w, Smem& sm,
                                          int32_t* fr, int32_t* nfront) {
  const float kInf = __int_as_float(0x7f800000);
  const int32_t* __restrict__ indptr = g.indptr;
  const int32_t* __restrict__ indices = g.indices;
  FNode* __restrict__ node = w.node;
  FNode* ny = &node[yy];
  const bool fresh = (__ldcg(&ny->st) & ~3) != ep2;
  const float p = fresh ? ogr_node_penalty(st, a, yy) : __ldcg(&ny->pen);
  const double pd = (double)p;
  float ba = kInf, bc = kInf, cin = kInf;
  double bl = 0.0;
  int32_t bu = 0x7fffffff;
  const int32_t f1 = indptr[yy + 1];
  for (int32_t f = indptr[yy] + sl; f < f1; f += W) {
    const int32_t u = indices[f];
    const float c = w.rcost[f];
    const int32_t su = __ldcg(&node[u].st);
    const double lu = __ldcg(&node[u].lab);
    if (su != (ep2 | ST_DONE)) {
      cin = fminf(cin, c);
      continue;
    }
    const float a32 = __double2float_rn((lu + (double)c) + pd);
    if (!(a32 < kInf)) continue;
    if (ogr_key_lt(a32, lu, u, ba, bl, bu)) { ba = a32; bl = lu; bu = u; bc = c; }
  }
#pragma unroll
  for (int o = W / 2; o > 0; o >>= 1) {
    const float oa = tile.shfl_xor(ba, o);
    const double ol = tile.shfl_xor(bl, o);
    const int32_t ou = tile.shfl_xor(bu, o);
    const float oc = tile.shfl_xor(bc, o);
    if (ogr_key_lt(oa, ol, ou, ba, bl, bu)) { ba = oa; bl = ol; bu = ou; bc = oc; }
    cin = fminf(cin, tile.shfl_xor(cin, o));
  }
  if (sl == 0) {
    if (fresh) ny->pen = p;
    ny->cin = cin;
    if (ba < kInf) {
      const double lab = (bl + (double)bc) + pd;
      ny->m32 = ba;
      ny->lab = lab;
      ny->par = bu;
      atomicMin(&sm.tmin, ogr_dbits(lab));
      if (fresh) {
        ny->st = ep2 | ST_FRONT;
        stage_push(sm, 0, yy, fr, nfront);
      }
    }
  }
}

__global__ void __launch_bounds__(kThreads, 2)
full_sssp_kernel(ogr_graph g, ogr_state st, ogr_full::Job job, FWs w) {
  __shared__ Smem sm;
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int sl = tid & (kSub - 1);
  const int gi = tid / kSub;
  const int64_t gthreads = (int64_t)gridDim.x * kThreads;
  const int64_t gtid = (int64_t)blockIdx.x * kThreads + tid;
  const bool leader = gtid == 0;
  const unsigned nblocks = gridDim.x;
  FCtl* ctl = w.ctl;

  if (job.from_pass && job.pass_result[0] < 0) return;  // uniform: written by an earlier launch
  ogr_net_args a = job.a;
  int32_t* path_out = job.path_out;
  int32_t path_cap = job.path_cap;
  if (job.from_pass) {
    const int32_t n = job.pa.order[job.k];
    a = ogr_pass_net_args(job.t, job.pa, n, 0);
    path_out = job.t.store_path + (int64_t)n * job.t.slot_cap;
    path_cap = job.t.slot_cap;
  }
  const int32_t N = g.num_nodes;
  const int64_t E = g.num_edges;
  const int32_t src = a.src, dst = a.dst;
  if (src == dst) {
    if (leader) {
      ctl->res[0] = OGR_NO_PATH;
      ctl->res[1] = 0;
      ctl->res[2] = 0;
    }
    return;
  }
  const int32_t* __restrict__ indptr = g.indptr;
  const int32_t* __restrict__ indices = g.indices;
  FNode* __restrict__ node = w.node;
  const float kInf = __int_as_float(0x7f800000);
  auto tile = cg::tiled_partition<kSub>(cg::this_thread_block());
  Clock clk{};
  unsigned long long t_start = 0;
  if (tid == 0) {
    t_start = gtimer();
    clk.mark = t_start;
  }
  unsigned long long bar_target = 0;

  // Epoch and phase numbering; when either would run out of range every node
  // is reset (all CTAs read the same persistent words, so all decide alike).
  int32_t ep = __ldcg(&ctl->epoch) + 1;
  int32_t gbase = __ldcg(&ctl->gbase);
  const int max_phase = 2 * N + 4;
  if (ep < 1 || ep > kMaxEpoch || gbase < 1 || gbase > 0x7fffffff - (max_phase + 8)) {
    for (int64_t r = gtid; r < N; r += gthreads)
      if (r != src) *reinterpret_cast<int2*>(&node[r].st) = make_int2(0, 0);   // src is written below
    ep = 1;
    gbase = 1;
  }
  const int32_t ep2 = ep << 2;
  {
    const int32_t* __restrict__ rev = g.rev;
    const float* __restrict__ tc = st.total_cost;
    float* __restrict__ rc = w.rcost;
#pragma unroll 4
    for (int64_t e = gtid; e < E; e += gthreads) rc[e] = tc[rev[e]];
  }
  if (leader) {
    FNode s0;
    s0.lab = 0.0;
    s0.m32 = 0.0f;
    s0.pen = 0.0f;
    s0.cin = kInf;
    s0.par = -1;
    s0.st = ep2 | ST_DONE;
    s0.stamp = gbase;
    node[src] = s0;
    ctl->nfront[0] = 0;
    ctl->nfront[1] = 0;
    ctl->nlog = 1;
    ctl->tbits[0] = ~0ull;
    ctl->tbits[1] = ~0ull;
    w.log[0] = src;
  }
  bool alive = grid_barrier(ctl, bar_target, sm, clk, &clk.init);
  int status = OGR_OK;
  bool found = false;
  // With statistics requested the search goes on after dst is settled until
  // every node with a label <= L(dst) is settled (T > L(dst)): the IN bound
  // can settle dst before cheaper nodes, which the heap pops earlier.
  const bool want_stats = job.stats != nullptr;
  bool dst_done = false;
  double ld = 0.0;
  int32_t lo = 0, hi = 1;   // log range settled in the previous phase
  int phase = 0;
  while (alive) {
    const int q = phase & 1;
    const int32_t gp = gbase + 1 + phase;
    stage_reset(sm);
    if (leader) {
      ctl->nfront[q ^ 1] = 0;
      ctl->tbits[q ^ 1] = ~0ull;
    }
    // E: the nodes settled last phase, dealt round-robin over the CTAs,
    // claim their unsettled out-neighbours; then the CTA's groups recompute
    // the claimed nodes from the shared-memory list.
    {
      for (int64_t i = lo + blockIdx.x + (int64_t)gi * nblocks; i < hi; i += (int64_t)nblocks * kGroups) {
        const int32_t x = __ldcg(&w.log[i]);
        const int32_t e1 = indptr[x + 1];
        for (int32_t e = indptr[x] + sl; e < e1; e += kSub) {
          const int32_t y = indices[e];
          const int32_t sy = __ldcg(&node[y].st);
          if (atomicMax(&node[y].stamp, gp) < gp && sy != (ep2 | ST_DONE)) {
            const int j = atomicAdd(&sm.nclaim, 1);
            if (j < kClaim)
              sm.claim[j] = y;
            else
              recompute<1>(tile, 0, y, ep2, g, st, a, w, sm, w.fr[q], &ctl->nfront[q]);
          }
        }
      }
      __syncthreads();
      const int nc = min(sm.nclaim, kClaim);
      for (int j = gi; j < nc; j += kGroups)
        recompute<kSub>(tile, sl, sm.claim[j], ep2, g, st, a, w, sm, w.fr[q], &ctl->nfront[q]);
      __syncthreads();
      stage_flush(sm, 1, w.fr[q], &ctl->nfront[q], nullptr, nullptr);
      if (tid == 0 && sm.tmin != ~0ull) atomicMin(&ctl->tbits[q], sm.tmin);
    }
    alive = grid_barrier(ctl, bar_target, sm, clk, &clk.e);
    if (!alive) break;
    const int nf = __ldcg(&ctl->nfront[q]);
    if (nf == 0) {
      if (dst_done)
        found = true;
      else
        status = OGR_NO_PATH;
      break;
    }
    const double T = __longlong_as_double((long long)__ldcg(&ctl->tbits[q]));
    if (dst_done && T > ld) {
      found = true;
      break;
    }
    // S: settle every frontier node whose state can no longer change
    {
      stage_reset(sm);
      const int32_t* fr = w.fr[q];
      for (int64_t i = blockIdx.x + (int64_t)tid * nblocks; i < nf; i += gthreads) {
        const int32_t x = __ldcg(&fr[i]);
        FNode* nx = &node[x];
        const double lab = __ldcg(&nx->lab);
        const float m32 = __ldcg(&nx->m32);
        const float cin = __ldcg(&nx->cin);
        const float pen = __ldcg(&nx->pen);
        const bool settle = (lab == T) || m32 < __double2float_rn((T + (double)cin) + (double)pen);
        if (settle) {
          nx->st = ep2 | ST_DONE;
          stage_push(sm, 1, x, w.log, &ctl->nlog);
        } else {
          stage_push(sm, 0, x, w.fr[q ^ 1], &ctl->nfront[q ^ 1]);
          atomicMin(&sm.tmin, ogr_dbits(lab));
        }
      }
      __syncthreads();
      stage_flush(sm, 2, w.fr[q ^ 1], &ctl->nfront[q ^ 1], w.log, &ctl->nlog);
      if (tid == 0 && sm.tmin != ~0ull) atomicMin(&ctl->tbits[q ^ 1], sm.tmin);
    }
    alive = grid_barrier(ctl, bar_target, sm, clk, &clk.s);
    if (!alive) break;
    lo = hi;
    hi = __ldcg(&ctl->nlog);
    if (!dst_done && __ldcg(&node[dst].st) == (ep2 | ST_DONE)) {
      dst_done = true;
      ld = __ldcg(&node[dst].lab);
      if (!want_stats) {
        found = true;
        break;
      }
    }
    if (++phase > max_phase) {
      status = OGR_ERR_ITER_CAP;
      break;
    }
  }
  if (!alive) status = OGR_ERR_TIMEOUT;
  // statistics: the rows of every node the sequential search pops before dst
  // (all of them are in the settled log)
  if (found && want_stats) {
    unsigned long long arcs = 0, pops = 0;
    for (int64_t i = gtid; i < hi; i += gthreads) {
      const int32_t r = __ldcg(&w.log[i]);
      const double lr = __ldcg(&node[r].lab);
      if (lr < ld || (lr == ld && r < dst)) {
        arcs += (unsigned long long)(indptr[r + 1] - indptr[r]);
        ++pops;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      arcs += __shfl_xor_sync(0xffffffffu, arcs, o);
      pops += __shfl_xor_sync(0xffffffffu, pops, o);
    }
    if (lane == 0 && pops) {
      atomicAdd(&job.stats[0], arcs);
      atomicAdd(&job.stats[1], pops);
    }
    if (leader) {
      atomicAdd(&job.stats[1], 1ull);
      atomicAdd(&job.stats[2], (unsigned long long)N);
      atomicAdd(&job.stats[3], (unsigned long long)(phase + 1));
    }
  }
  if (tid == 0) {
    atomicMax(&g_full_prof[4], clk.e);
    atomicMax(&g_full_prof[5], clk.s);
  }
  if (blockIdx.x != 0) return;
  // backtrace dst -> src in one walk (reversed into path_out), then CTA 0
  // turns it around
  if (tid == 0) {
    int len = 0;
    if (found) {
      const int limit = min(path_cap, N);
      int32_t c = dst;
      while (c != -1 && len < limit) {
        path_out[len++] = c;
        c = __ldcg(&node[c].par);
      }
      if (c != -1) status = len >= N ? OGR_ERR_ITER_CAP : OGR_ERR_CAPACITY;
      else if (len < 2) status = OGR_NO_PATH;
    }
    if (ld_volatile(&ctl->bar_err)) status = OGR_ERR_TIMEOUT;
    sm.base[0] = status;
    sm.base[1] = (found && status == OGR_OK) ? len : 0;
  }
  __syncthreads();
  const int len = sm.base[1];
  for (int i = tid; i < len / 2; i += kThreads) {
    const int32_t t = path_out[i];
    path_out[i] = path_out[len - 1 - i];
    path_out[len - 1 - i] = t;
  }
  if (tid != 0) return;
  status = sm.base[0];
  ctl->res[0] = status;
  ctl->res[1] = len;
  ctl->res[2] = phase + 1;
  ctl->epoch = ep;
  ctl->gbase = gbase + phase + 2;
  const unsigned long long t_end = gtimer();
  atomicAdd(&g_full_prof[0], 1ull);
  atomicAdd(&g_full_prof[1], (unsigned long long)(phase + 1));
  atomicAdd(&g_full_prof[2], t_end - t_start);
  atomicAdd(&g_full_prof[3], clk.init);
  atomicAdd(&g_full_prof[6], clk.wait);
  atomicAdd(&g_full_prof[7], t_end - clk.mark);
}

constexpr int kMaxDevices = 64;
int g_grid_blocks[kMaxDevices] = {};

}  // namespace

namespace ogr_full {

size_t workspace_bytes(int32_t num_nodes, int64_t num_edges) {
  return fws_layout(num_nodes, num_edges, nullptr, nullptr);
}

int32_t* result_words(void* ws, int32_t num_nodes, int64_t num_edges) {
  FWs w;
  fws_layout(num_nodes, num_edges, (char*)ws, &w);
  return w.ctl->res;
}

int launch(const ogr_graph& g, const ogr_state& st, const Job& job, void* ws, cudaStream_t s) {
  int dev = 0;
  OGR_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return OGR_ERR_ARG;
  if (g_grid_blocks[dev] == 0) {
    int sms = 0, per_sm = 0, coop = 0;
    OGR_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    OGR_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    OGR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, full_sssp_kernel, kThreads, 0));
    if (!coop || per_sm < 1) return OGR_ERR_CUDA;
    g_grid_blocks[dev] = sms * per_sm;
  }
  FWs w;
  fws_layout(g.num_nodes, g.num_edges, (char*)ws, &w);
  // bar_count, bar_gen and bar_err start at zero on every launch
  OGR_CUDA_TRY(cudaMemsetAsync(w.ctl, 0, offsetof(FCtl, tbits), s));
  ogr_graph gv = g;
  ogr_state sv = st;
  ogr_full::Job jv = job;
  void* args[] = {&gv, &sv, &jv, &w};
  OGR_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)full_sssp_kernel, dim3(g_grid_blocks[dev]), dim3(kThreads),
                                           args, 0, s));
  return OGR_OK;
}

}  // namespace ogr_full

extern "C" size_t ogr_full_workspace_bytes(int32_t num_nodes, int64_t num_edges) {
  return ogr_full::workspace_bytes(num_nodes, num_edges);
}

extern "C" int ogr_full_workspace_init(void* ws, size_t bytes, int32_t num_nodes, int64_t num_edges,
                                       void* stream) {
  if (!ws || num_nodes < 1 || num_edges < 0) return OGR_ERR_ARG;
  if (bytes < ogr_full::workspace_bytes(num_nodes, num_edges)) return OGR_ERR_CAPACITY;
  FWs w;
  fws_layout(num_nodes, num_edges, (char*)ws, &w);
  // epoch 0 / phase base 0: the first search resets every node
  OGR_CUDA_TRY(cudaMemsetAsync(w.ctl, 0, sizeof(FCtl), ogr_stream(stream)));
  return OGR_OK;
}

extern "C" int ogr_full_profile(int64_t* out8, int32_t reset) {
  if (!out8) return OGR_ERR_ARG;
  OGR_CUDA_TRY(cudaMemcpyFromSymbol(out8, g_full_prof, sizeof(unsigned long long) * 8));
  if (reset) {
    unsigned long long z[8] = {};
    OGR_CUDA_TRY(cudaMemcpyToSymbol(g_full_prof, z, sizeof(z)));
  }
  return OGR_OK;
}

extern "C" int ogr_find_path_full(const ogr_graph* g, const ogr_state* st, const ogr_net_args* net, void* ws,
                                  size_t bytes, int32_t* path_out, int32_t path_cap, int32_t* path_len_out,
                                  int64_t* stats, void* stream) {
  if (!g || !st || !net || !ws || !path_out || !path_len_out || path_cap < 2) return OGR_ERR_ARG;
  if (bytes < ogr_full::workspace_bytes(g->num_nodes, g->num_edges)) return OGR_ERR_CAPACITY;
  if (net->src < 0 || net->dst < 0 || net->src >= g->num_nodes || net->dst >= g->num_nodes) return OGR_ERR_ARG;
  ogr_full::Job job{};
  job.a = *net;
  job.path_out = path_out;
  job.path_cap = path_cap;
  job.from_pass = 0;
  job.stats = reinterpret_cast<unsigned long long*>(stats);
  cudaStream_t s = ogr_stream(stream);
  const int rc = ogr_full::launch(*g, *st, job, ws, s);
  if (rc != OGR_OK) return rc;
  int32_t res[4];
  OGR_CUDA_TRY(cudaMemcpyAsync(res, ogr_full::result_words(ws, g->num_nodes, g->num_edges), sizeof(res),
                               cudaMemcpyDeviceToHost, s));
  OGR_CUDA_TRY(cudaStreamSynchronize(s));
  *path_len_out = res[0] == OGR_OK ? res[1] : 0;
  return res[0];
}
