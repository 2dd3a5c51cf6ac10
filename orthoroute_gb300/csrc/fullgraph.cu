// A7 for long nets: the exact search over the whole lattice on every SM.
//
// The reference searches nets whose Manhattan length is 125 steps or more on
// the full graph (_route_all, unified_pathfinder.py:8219-8262: roi_nodes =
// arange(N)), so its heap Dijkstra (find_path_roi, :2451-2548) settles every
// node cheaper than dst — most of a 600x400x12 lattice.  The result here is
// the same as the heap's: every node takes the lexicographic minimum of
// (float32(alt), L(u), u) over its in-neighbours u, alt = (L(u) + c) + pen.
//
// Phases, one grid step each.  Every frontier node v pulls its key, label
// and parent from the in-neighbours settled before this phase (settle-phase
// stamps make that set a snapshot) and cin(v), its cheapest in-arc from any
// other node.  With T = a lower bound of the frontier's labels, v is final
// when L(v) == T or key(v) < float32((T + cin) + pen) — the IN criterion.  A
// node that settles marks its unreached out-neighbours as reached (they join
// the next frontier) and offers its candidate labels to the next T.  Every
// decision of a phase depends only on the set settled before it, so the
// result does not depend on thread timing.  T for the next phase is the
// minimum of the labels carried over and of the settling nodes' candidate
// labels; a label recomputed from a new winner can move within one float32
// value in either direction, so T may lie below the true minimum, which only
// makes both tests stricter.
//
// The kernel is launched cooperatively with one grid of fully resident CTAs
// (occupancy API); its grid barrier gives up after a bounded wait and reports
// OGR_ERR_TIMEOUT.  Per-node words carry the search's phase numbers (reach
// stamp, settle stamp), which keep increasing across searches, so no search
// clears per-node memory.  List appends are staged per CTA in shared memory.
#include <cooperative_groups.h>

#include <atomic>

#include "fullgraph.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int kThreads = 512;
// The tuning knobs below are per host thread: each job of a server routes in
// its own thread and keeps its own settings.
// Lanes per examined frontier node: 4, 8 or 16 (one instantiation each,
// chosen at launch by ogr_full_lanes; results do not depend on it).  Narrow
// groups keep more nodes in flight when rows are short and fronts are wide.
thread_local int g_full_lanes = 16;
// Reuse of clean carried nodes' last pull (ogr_full_reuse): it saves the
// pulls of wide fronts of waiting nodes and costs a stamp load per entry and
// state stores per carried node; which wins depends on the lattice.
thread_local int g_full_reuse = 0;
constexpr int kStage = 2048;               // staged list entries per CTA and list
constexpr unsigned kBarSpin = 1u << 22;
// Limits for tests of failure handling (ogr_debug_limits): the grid
// barrier's spin bound and a cap on settle phases; the defaults are
// kBarSpin and 2N + 4 (no search needs more).
thread_local unsigned g_dbg_spin = kBarSpin;
thread_local int g_dbg_phases = 0;


struct FCtl {
  alignas(128) unsigned long long bar_count;   // monotone arrival counter
  alignas(128) int32_t bar_err;
  alignas(128) unsigned long long tbits[3];
  alignas(128) int32_t nfront[3];
  alignas(128) int32_t nlog;                   // settled-log length
  alignas(128) int32_t res[4];
  int32_t gbase;                               // persistent across searches
  int32_t tile_gate;                           // 1: the tile engine handed this net over
  int32_t merr;                                // multi-source: a bad or repeated seed / target
  unsigned long long mk[3];                    // multi-source: the chosen target's keys
};

// Multi-source searches mark seeds and targets in per-node doubles that hold
// this NaN pattern otherwise (written by the workspace init, restored by
// every search).
constexpr unsigned long long kNoTerm = 0x7ff8deadbeef0001ull;

// Per-node search record: label, settle stamp, reach stamp in one 16-byte
// load.  A reader uses lab only where sp says the node settled in an earlier
// phase (written before the barrier), so a record torn by a concurrent settle
// of this phase is never misread.
struct __align__(16) NodeRec {
  double lab;        // label, valid once settled in this search
  int32_t sp;        // phase number of the settle (this search: > gbase)
  int32_t reach;     // == gbase: reached in this search
};

// Frontier entry: node, its CSR row [f0, f1) and its penalty bits, filled in
// by whoever appends it, so the examination starts with the row.
using FEntry = int4;

struct FWs {
  NodeRec* rec;
  int32_t* par;              // winning in-neighbour (tentative while carried, final once settled)
  int32_t* dirty;            // phase in which the node must pull again (an in-neighbour settled)
  float* tcin;               // cin of a carried node's last pull
  int32_t reuse;             // 1: carried nodes with no newly settled in-neighbour skip the pull
  unsigned bar_spin;         // grid barrier spin bound
  int32_t max_phases;        // > 0: cap on settle phases (else 2N + 4)
  float* rcost;              // reverse-arc cost gather when the state carries none
  FEntry* fr[3];             // frontier lists: read, write, and the one being cleared
  int32_t* log;              // settled nodes in settle order
  FCtl* ctl;
  char* tile;                // scratch of the tile-window engine
  double* mseed;             // multi-source: seed cost per node (kNoTerm bits otherwise)
  double* mtgt;              // multi-source: target cost per node (kNoTerm bits otherwise)
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
  t.rec = (NodeRec*)take(16 * n);
  t.par = (int32_t*)take(4 * n);
  t.dirty = (int32_t*)take(4 * n);
  t.tcin = (float*)take(4 * n);
  t.rcost = (float*)take(4 * (size_t)E);
  for (int i = 0; i < 3; ++i) t.fr[i] = (FEntry*)take(16 * n);
  t.log = (int32_t*)take(4 * n);
  t.tile = take(ogr_tile::workspace_bytes(N));
  t.mseed = (double*)take(8 * n);
  t.mtgt = (double*)take(8 * n);
  if (w) *w = t;
  return off;
}

struct Smem {
  FEntry fbuf[kStage];
  int32_t lbuf[kStage];
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
// [0] searches, [1] phases, [2] kernel ns, [3] init ns (CTA 0), [4] phase
// work ns (largest CTA total), [5] frontier entries examined, [6] barrier
// wait ns (CTA 0), [7] statistics + backtrace ns (CTA 0).
__device__ unsigned long long g_full_prof[8];

// Per-CTA timing kept by thread 0.
struct Clock {
  unsigned long long mark, init, e, wait;
};

// Grid barrier on a monotone arrival counter: the k-th barrier of a launch
// is passed when the counter reaches k * gridDim.x.  The wait is bounded;
// false when any CTA gave up.  Thread 0 adds the time since the previous
// barrier to *work and the wait to clk.wait.
__device__ bool grid_barrier(FCtl* c, unsigned long long& target, Smem& sm, Clock& clk, unsigned long long* work,
                             unsigned spin) {
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
      if (++it > spin || ld_volatile(&c->bar_err)) {
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

// Appends x to the staged frontier list (k = 0) or the settled log (k = 1)
// from the lanes of `tile` whose `want` is set: one shared-memory
// reservation per tile; past the staging capacity the entry goes straight to
// the global list.
template <typename Tile, typename T>
__device__ __forceinline__ void stage_push_tile(Tile& tile, Smem& sm, int k, bool want, const T& x, T* gl,
                                                int32_t* gcnt) {
  const unsigned m = tile.ballot(want);
  if (m == 0) return;
  const int lead = __ffs(m) - 1;
  int base = 0;
  if ((int)tile.thread_rank() == lead) base = atomicAdd(&sm.cnt[k], __popc(m));
  base = tile.shfl(base, lead);
  if (want) {
    const int i = base + __popc(m & ((1u << tile.thread_rank()) - 1u));
    if (i < kStage) {
      if constexpr (sizeof(T) == sizeof(FEntry))
        sm.fbuf[i] = x;
      else
        sm.lbuf[i] = x;
    } else {
      gl[atomicAdd(gcnt, 1)] = x;
    }
  }
}

// Publishes both staged lists of this CTA (call after __syncthreads, from all
// threads): one global reservation per list, issued together, then a
// coalesced copy.
__device__ __forceinline__ void stage_flush(Smem& sm, FEntry* gf, int32_t* gfc, int32_t* gl, int32_t* glc) {
  if (threadIdx.x == 0) {
    const int n0 = min(sm.cnt[0], kStage), n1 = min(sm.cnt[1], kStage);
    const int b0 = n0 ? atomicAdd(gfc, n0) : 0;
    const int b1 = n1 ? atomicAdd(glc, n1) : 0;
    sm.cnt[0] = n0;
    sm.cnt[1] = n1;
    sm.base[0] = b0;
    sm.base[1] = b1;
  }
  __syncthreads();
  const int n0 = sm.cnt[0], b0 = sm.base[0], n1 = sm.cnt[1], b1 = sm.base[1];
  for (int i = threadIdx.x; i < n0; i += kThreads) gf[b0 + i] = sm.fbuf[i];
  for (int i = threadIdx.x; i < n1; i += kThreads) gl[b1 + i] = sm.lbuf[i];
}

__device__ __forceinline__ void stage_reset(Smem& sm) {
  if (threadIdx.x == 0) {
    sm.cnt[0] = 0;
    sm.cnt[1] = 0;
    sm.tmin = ~0ull;
  }
  __syncthreads();
}

// Multi-source: whether node u is marked in a seed / target array.
__device__ __forceinline__ bool is_term(const double* arr, int32_t u) {
  return (unsigned long long)__double_as_longlong(__ldcg(&arr[u])) != kNoTerm;
}

__device__ __forceinline__ NodeRec ld_rec(const NodeRec* p) {
  const int4 q = __ldcg(reinterpret_cast<const int4*>(p));
  NodeRec r;
  r.lab = __hiloint2double(q.y, q.x);
  r.sp = q.z;
  r.reach = q.w;
  return r;
}

template <int S>
__global__ void __launch_bounds__(kThreads, 2)
full_sssp_kernel(ogr_graph g, ogr_state st, ogr_full::Job job, FWs w) {
  constexpr int kSub = S;                    // lanes per examined node
  constexpr int kGroups = kThreads / kSub;   // groups per CTA
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
  if (job.gated && __ldcg(&ctl->tile_gate) == 0) return;  // uniform: the tile engine found the result
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
  const bool multi = job.multi != 0;
  const int32_t src = multi ? -1 : a.src, dst = multi ? -1 : a.dst;
  if (!multi && src == dst) {
    if (leader) {
      ctl->res[0] = OGR_NO_PATH;
      ctl->res[1] = 0;
      ctl->res[2] = 0;
    }
    return;
  }
  const int32_t* __restrict__ indptr = g.indptr;
  const int32_t* __restrict__ indices = g.indices;
  const float* __restrict__ fcost = st.total_cost;
  NodeRec* __restrict__ rec = w.rec;
  const float kInf = __int_as_float(0x7f800000);
  auto tile = cg::tiled_partition<kSub>(cg::this_thread_block());
  Clock clk{};
  unsigned long long t_start = 0;
  if (tid == 0) {
    t_start = gtimer();
    clk.mark = t_start;
  }
  unsigned long long bar_target = 0;
  unsigned long long examined = 0;

  // Phase numbers continue across searches, so the stamps of older searches
  // (<= gbase) read as unreached / unsettled; when they would run out of range
  // the stamps are cleared (all CTAs read the same persistent word).
  int32_t gbase = __ldcg(&ctl->gbase);
  const int max_phase_natural = 2 * N + 4;
  const int max_phase = w.max_phases > 0 ? min(w.max_phases, max_phase_natural) : max_phase_natural;
  bool cleared = false;
  if (gbase < 1 || gbase > 0x7fffffff - (max_phase_natural + 8)) {
    for (int64_t r = gtid; r < N; r += gthreads) {
      w.dirty[r] = 0;
      if (r != src) {
        rec[r].sp = 0;
        rec[r].reach = 0;
      }
    }
    gbase = 1;
    cleared = true;
  }
  bool alive = true;
  // the seeds' records are written below by one thread: the clearing must be over
  if (multi && cleared) alive = grid_barrier(ctl, bar_target, sm, clk, &clk.init, w.bar_spin);
  const float* rc = st.rcost;
  if (rc == nullptr) {
    const int32_t* __restrict__ rev = g.rev;
    float* __restrict__ out = w.rcost;
#pragma unroll 4
    for (int64_t e = gtid; e < E; e += gthreads) out[e] = fcost[rev[e]];
    rc = w.rcost;
  }
  if (leader && !multi) {
    rec[src].reach = gbase;
    rec[src].sp = 0;
    w.fr[0][0] = make_int4(src, indptr[src], indptr[src + 1], __float_as_int(0.0f));
    for (int i = 0; i < 3; ++i) {
      ctl->nfront[i] = i == 0 ? 1 : 0;
      ctl->tbits[i] = i == 0 ? 0ull : ~0ull;   // T of phase 0 = L(src) = 0
    }
    ctl->nlog = 0;
  } else if (leader) {
    // Multi-source: mark the targets, then put every seed in the first
    // frontier with its label seed cost + penalty (T of phase 0 = the least).
    int bad = 0, nf0 = 0;
    unsigned long long t0 = ~0ull;
    for (int i = 0; i < job.n_targets && !bad; ++i) {
      const int32_t t = job.targets[i];
      const double tc = job.target_cost[i];
      if (t < 0 || t >= N || tc != tc) { bad = 1; break; }
      unsigned long long* p = reinterpret_cast<unsigned long long*>(&w.mtgt[t]);
      if (*p != kNoTerm) { bad = 1; break; }   // repeated target
      *p = (unsigned long long)__double_as_longlong(tc);
    }
    for (int i = 0; i < job.n_seeds && !bad; ++i) {
      const int32_t s0 = job.seeds[i];
      const double sc = job.seed_cost[i];
      if (s0 < 0 || s0 >= N || !(sc >= 0.0)) { bad = 1; break; }
      unsigned long long* p = reinterpret_cast<unsigned long long*>(&w.mseed[s0]);
      if (*p != kNoTerm) { bad = 1; break; }   // repeated seed
      *p = (unsigned long long)__double_as_longlong(sc);
      const float pen = ogr_node_penalty(st, a, s0);
      rec[s0].reach = gbase;
      rec[s0].sp = 0;
      w.fr[0][nf0++] = make_int4(s0, indptr[s0], indptr[s0 + 1], __float_as_int(pen));
      const unsigned long long lb = ogr_dbits(sc + (double)pen);
      t0 = lb < t0 ? lb : t0;
    }
    for (int i = 0; i < 3; ++i) {
      ctl->nfront[i] = (i == 0 && !bad) ? nf0 : 0;
      ctl->tbits[i] = i == 0 ? t0 : ~0ull;
      ctl->mk[i] = ~0ull;
    }
    ctl->nlog = 0;
    ctl->merr = bad;
  }
  if (alive) alive = grid_barrier(ctl, bar_target, sm, clk, &clk.init, w.bar_spin);
  int status = OGR_OK;
  if (multi && __ldcg(&ctl->merr)) status = OGR_ERR_ARG;
  bool found = false;
  // With statistics requested the search goes on after dst is settled until
  // every node with a label <= L(dst) is settled (T > L(dst)): the IN bound
  // can settle dst before cheaper nodes, which the heap pops earlier.
  const bool want_stats = job.stats != nullptr;
  bool dst_done = false;
  double ld = 0.0;
  int phase = 0;
  while (alive && status == OGR_OK) {
    const int b = phase % 3, bn = (phase + 1) % 3, bz = (phase + 2) % 3;
    const int32_t gp = gbase + 1 + phase;
    // the frontier length, T and (until it settles) dst's record, issued as
    // one batch of loads after the barrier
    const int nf = __ldcg(&ctl->nfront[b]);
    const unsigned long long tb = __ldcg(&ctl->tbits[b]);
    if (!multi && !dst_done && phase > 0) {
      const NodeRec rd = ld_rec(&rec[dst]);
      if (rd.sp > gbase) {
        dst_done = true;
        ld = rd.lab;
        if (!want_stats) {
          found = true;
          --phase;             // no work of this phase was done
          break;
        }
      }
    }
    if (nf == 0) {
      if (dst_done || multi)
        found = true;            // multi-source: the target is chosen below
      else
        status = OGR_NO_PATH;
      break;
    }
    const double T = __longlong_as_double((long long)tb);
    if (dst_done && T > ld) {
      found = true;
      break;
    }
    stage_reset(sm);
    if (leader) {
      ctl->nfront[bz] = 0;
      ctl->tbits[bz] = ~0ull;
    }
    const FEntry* fr = w.fr[b];
    FEntry* frn = w.fr[bn];
    for (int64_t i = blockIdx.x + (int64_t)gi * nblocks; i < nf; i += (int64_t)nblocks * kGroups) {
      const FEntry ent = __ldcg(&fr[i]);
      const int32_t v = ent.x, f0 = ent.y, f1 = ent.z;
      const float pv = __int_as_float(ent.w);
      const double pd = (double)pv;
      const bool is_src = v == src;
      // A carried node none of whose in-neighbours settled since its last
      // pull keeps that pull's state (label in rec, parent, cin): a pull is a
      // function of the in-neighbours settled before the phase.  A settle in
      // phase q writes dirty = q + 1 (values only grow; a settle of this very
      // phase may already show as gp + 1, which only adds a harmless pull).
      // (seeds are never marked dirty: a multi-source search always pulls)
      const bool pull = multi || !w.reuse || is_src || __ldcg(&w.dirty[v]) >= gp;
      const bool one_pass = pull && f1 - f0 <= kSub;
      // pull: the lexicographic minimum of the candidates of the in-neighbours
      // settled before this phase; cin from the others.  One-pass rows keep
      // each lane's neighbour data (stamps, penalty, CSR row) for the marking.
      float ba = kInf, bc = kInf, cin = kInf;
      double bl = 0.0;
      int32_t bu = 0x7fffffff;
      int32_t u0 = -1, s0 = 0, r0 = 0, i0 = 0, i1 = 0;
      float cout0 = kInf, p0 = 0.0f;
      for (int32_t f = f0 + sl; pull && f < f1; f += kSub) {
        const int32_t u = indices[f];
        const float c = rc[f];
        const NodeRec ru = ld_rec(&rec[u]);
        if (one_pass) {
          u0 = u;
          s0 = ru.sp;
          r0 = ru.reach;
          cout0 = fcost[f];
          p0 = ogr_node_penalty(st, a, u);
          i0 = indptr[u];
          i1 = indptr[u + 1];
        }
        // multi-source: a target never relaxes anything, settled or not
        const bool u_term = multi && is_term(w.mtgt, u);
        if (!(ru.sp > gbase && ru.sp < gp)) {
          if (!u_term) cin = fminf(cin, c);
          continue;
        }
        if (u_term) continue;
        const float a32 = __double2float_rn((ru.lab + (double)c) + pd);
        if (!(a32 < kInf)) continue;
        if (ogr_key_lt(a32, ru.lab, u, ba, bl, bu)) { ba = a32; bl = ru.lab; bu = u; bc = c; }
      }
#pragma unroll
      for (int o = kSub / 2; o > 0; o >>= 1) {
        const float oa = tile.shfl_xor(ba, o);
        const double ol = tile.shfl_xor(bl, o);
        const int32_t ou = tile.shfl_xor(bu, o);
        const float oc = tile.shfl_xor(bc, o);
        if (ogr_key_lt(oa, ol, ou, ba, bl, bu)) { ba = oa; bl = ol; bu = ou; bc = oc; }
        cin = fminf(cin, tile.shfl_xor(cin, o));
      }
      double lv;
      float m32;
      if (pull) {
        lv = is_src ? 0.0 : (bl + (double)bc) + pd;
        m32 = is_src ? 0.0f : ba;   // == float32(lv): the same expression
        if (multi) {
          // a seed's own candidate comes before every relaxation: it loses
          // only to a strictly smaller float32 value
          const double sc = __ldcg(&w.mseed[v]);
          if ((unsigned long long)__double_as_longlong(sc) != kNoTerm) {
            const double sl = sc + pd;
            const float s32 = __double2float_rn(sl);
            if (!(ba < s32)) {
              lv = sl;
              m32 = s32;
              bu = -1;
            }
          }
        }
      } else {
        lv = __ldcg(&rec[v].lab);
        m32 = __double2float_rn(lv);
        cin = __ldcg(&w.tcin[v]);
        bu = __ldcg(&w.par[v]);
      }
      const bool settle = (lv == T) || m32 < __double2float_rn((T + (double)cin) + pd);
      examined += (sl == 0);
      if (!settle) {
        stage_push_tile(tile, sm, 0, sl == 0, ent, frn, &ctl->nfront[bn]);
        if (sl == 0) {
          atomicMin(&sm.tmin, ogr_dbits(lv));
          if (pull && w.reuse) {   // keep the pulled state; rec[v].lab is read by others only once settled
            rec[v].lab = lv;
            w.tcin[v] = cin;
            w.par[v] = bu;
          }
        }
        continue;
      }
      if (sl == 0) {
        rec[v].lab = lv;
        rec[v].sp = gp;
        w.par[v] = is_src ? -1 : bu;
      }
      stage_push_tile(tile, sm, 1, sl == 0, v, w.log, &ctl->nlog);
      if (multi && is_term(w.mtgt, v)) continue;   // a settled target is never expanded
      // mark the unreached out-neighbours and offer the candidate labels
      unsigned long long tl = ~0ull;
      for (int32_t fb = f0; fb < f1; fb += kSub) {   // same trip count on every lane (ballots inside)
        const int32_t f = fb + sl;
        const bool act = f < f1;
        int32_t y = -1, sy = 0;
        if (act) {
          y = one_pass ? u0 : indices[f];
          sy = one_pass ? s0 : __ldcg(&rec[y].sp);
        }
        bool fresh = false;
        FEntry ny = make_int4(0, 0, 0, 0);
        if (w.reuse && act && !(sy > gbase)) w.dirty[y] = gp + 1;   // v settled: y pulls next phase
        if (act && !(sy > gbase)) {   // settled nodes cannot improve
          const float c = one_pass ? cout0 : fcost[f];
          const float py = one_pass ? p0 : ogr_node_penalty(st, a, y);
          const double ly = (lv + (double)c) + (double)py;
          if (__double2float_rn(ly) < kInf) {
            const unsigned long long bits = ogr_dbits(ly);
            tl = bits < tl ? bits : tl;
            const int32_t ry = one_pass ? r0 : __ldcg(&rec[y].reach);
            fresh = ry != gbase && atomicExch(&rec[y].reach, gbase) != gbase;
            if (fresh) ny = make_int4(y, one_pass ? i0 : indptr[y], one_pass ? i1 : indptr[y + 1], __float_as_int(py));
          }
        }
        stage_push_tile(tile, sm, 0, fresh, ny, frn, &ctl->nfront[bn]);
      }
#pragma unroll
      for (int o = kSub / 2; o > 0; o >>= 1) {
        const unsigned long long ot = tile.shfl_xor(tl, o);
        tl = ot < tl ? ot : tl;
      }
      if (sl == 0 && tl != ~0ull) atomicMin(&sm.tmin, tl);
    }
    __syncthreads();
    stage_flush(sm, frn, &ctl->nfront[bn], w.log, &ctl->nlog);
    if (tid == 0 && sm.tmin != ~0ull) atomicMin(&ctl->tbits[bn], sm.tmin);
    alive = grid_barrier(ctl, bar_target, sm, clk, &clk.e, w.bar_spin);
    if (!alive) break;
    if (++phase > max_phase) {
      status = OGR_ERR_ITER_CAP;
      break;
    }
  }
  if (!alive) status = OGR_ERR_TIMEOUT;
  const int nlog = __ldcg(&ctl->nlog);
  // Multi-source: the settled target with the least (label + target cost,
  // label, id) -- the first strict improvement in the heap's pop order.
  int32_t tgt = dst;
  if (multi && found) {
    const double dinf = __longlong_as_double(0x7ff0000000000000ll);
    unsigned long long k1 = ~0ull, k2 = ~0ull;
    for (int pass = 0; pass < 3 && alive; ++pass) {
      unsigned long long k = ~0ull;
      for (int64_t i = gtid; i < nlog; i += gthreads) {
        const int32_t r = __ldcg(&w.log[i]);
        const double tc = __ldcg(&w.mtgt[r]);
        if ((unsigned long long)__double_as_longlong(tc) == kNoTerm) continue;
        const double lr = __ldcg(&rec[r].lab);
        const double tot = lr + tc;
        if (!(tot < dinf)) continue;
        const unsigned long long kt = ogr_order_bits(tot), kl = ogr_order_bits(lr);
        const unsigned long long x = pass == 0 ? kt : pass == 1 ? (kt == k1 ? kl : ~0ull)
                                                               : (kt == k1 && kl == k2 ? (unsigned long long)r : ~0ull);
        k = x < k ? x : k;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long ok = __shfl_xor_sync(0xffffffffu, k, o);
        k = ok < k ? ok : k;
      }
      if (lane == 0 && k != ~0ull) atomicMin(&ctl->mk[pass], k);
      alive = grid_barrier(ctl, bar_target, sm, clk, &clk.e, w.bar_spin);
      if (pass == 0) k1 = __ldcg(&ctl->mk[0]);
      if (pass == 1) k2 = __ldcg(&ctl->mk[1]);
      if (k1 == ~0ull) break;   // uniform: no target reached
    }
    if (!alive) {
      status = OGR_ERR_TIMEOUT;
      found = false;
    } else if (k1 == ~0ull) {
      status = OGR_NO_PATH;
      found = false;
    } else {
      tgt = (int32_t)__ldcg(&ctl->mk[2]);
    }
  }
  // statistics: the rows of every node the sequential search pops before dst
  // (all of them are in the settled log)
  // A search that cannot reach dst pops every node it reaches (all of them in
  // the log once the frontier is empty) and scans each one's row.
  const bool exhausted = !multi && alive && status == OGR_NO_PATH;
  if ((found || exhausted) && want_stats) {
    unsigned long long arcs = 0, pops = 0;
    for (int64_t i = gtid; i < nlog; i += gthreads) {
      const int32_t r = __ldcg(&w.log[i]);
      if (multi) {   // the heap runs empty: every settled node popped, the non-targets expanded
        ++pops;
        if (!is_term(w.mtgt, r)) arcs += (unsigned long long)(indptr[r + 1] - indptr[r]);
        continue;
      }
      const double lr = __ldcg(&rec[r].lab);
      if (exhausted || lr < ld || (lr == ld && r < dst)) {
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
      if (found && !multi) atomicAdd(&job.stats[1], 1ull);   // dst's own pop
      atomicAdd(&job.stats[2], (unsigned long long)N);
      atomicAdd(&job.stats[3], (unsigned long long)(phase + 1));
    }
  }
  if (tid == 0) atomicMax(&g_full_prof[4], clk.e);
  examined = __reduce_add_sync(0xffffffffu, (unsigned)examined);
  if (lane == 0 && examined) atomicAdd(&g_full_prof[5], examined);
  if (multi) {
    // every CTA is past its reads of the marks: restore them for the next search
    grid_barrier(ctl, bar_target, sm, clk, &clk.e, w.bar_spin);
    const unsigned long long none = kNoTerm;
    for (int64_t i = gtid; i < job.n_seeds; i += gthreads) {
      const int32_t x = job.seeds[i];
      if (x >= 0 && x < N) w.mseed[x] = __longlong_as_double((long long)none);
    }
    for (int64_t i = gtid; i < job.n_targets; i += gthreads) {
      const int32_t x = job.targets[i];
      if (x >= 0 && x < N) w.mtgt[x] = __longlong_as_double((long long)none);
    }
  }
  if (blockIdx.x != 0) return;
  // backtrace dst -> src in one walk (reversed into path_out), then CTA 0
  // turns it around
  if (tid == 0) {
    int len = 0;
    if (found) {
      const int limit = min(path_cap, N);
      int32_t c = tgt;
      while (c != -1 && len < limit) {
        path_out[len++] = c;
        c = __ldcg(&w.par[c]);
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
  ctl->gbase = gbase + phase + 2;
  const unsigned long long t_end = gtimer();
  atomicAdd(&g_full_prof[0], 1ull);
  atomicAdd(&g_full_prof[1], (unsigned long long)(phase + 1));
  atomicAdd(&g_full_prof[2], t_end - t_start);
  atomicAdd(&g_full_prof[3], clk.init);
  atomicAdd(&g_full_prof[6], clk.wait);
  atomicAdd(&g_full_prof[7], t_end - clk.mark);
}

__global__ void fill_u64_kernel(unsigned long long* p, int64_t n, unsigned long long v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

constexpr int kMaxDevices = 64;
thread_local int g_grid_blocks[kMaxDevices] = {};   // grid of the cooperative launch (0: not sized yet)
std::atomic<int> g_grid_limit[kMaxDevices] = {};    // SMs x resident CTAs per SM (a device property)

int size_grid(int dev) {
  if (g_grid_limit[dev] == 0) {
    int sms = 0, per_sm = 0, coop = 0;
    OGR_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    OGR_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    // every lane width must fit the same cooperative grid
    int p4 = 0, p8 = 0, p16 = 0;
    OGR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p4, full_sssp_kernel<4>, kThreads, 0));
    OGR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p8, full_sssp_kernel<8>, kThreads, 0));
    OGR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p16, full_sssp_kernel<16>, kThreads, 0));
    per_sm = min(p4, min(p8, p16));
    if (!coop || per_sm < 1) return OGR_ERR_CUDA;
    g_grid_limit[dev] = sms * per_sm;
  }
  if (g_grid_blocks[dev] == 0) g_grid_blocks[dev] = g_grid_limit[dev];
  return OGR_OK;
}

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
  const int rc = size_grid(dev);
  if (rc != OGR_OK) return rc;
  FWs w;
  fws_layout(g.num_nodes, g.num_edges, (char*)ws, &w);
  w.reuse = g_full_reuse;
  w.bar_spin = g_dbg_spin;
  w.max_phases = g_dbg_phases;
  ogr_full::Job jv = job;
  jv.gated = 0;
  if (ogr_tile::enabled() && !job.multi) {
    const int trc = ogr_tile::launch(g, st, job, w.tile, w.ctl->res, &w.ctl->tile_gate, s);
    if (trc == OGR_OK)
      jv.gated = 1;              // the phase engine runs only if the net was handed over
    else if (trc != OGR_ERR_CAPACITY)
      return trc;                // (capacity: this lattice does not tile; phase engine alone)
  }
  // bar_count, bar_gen and bar_err start at zero on every launch
  OGR_CUDA_TRY(cudaMemsetAsync(w.ctl, 0, offsetof(FCtl, tbits), s));
  ogr_graph gv = g;
  ogr_state sv = st;
  void* args[] = {&gv, &sv, &jv, &w};
  const void* fn = g_full_lanes == 4   ? (const void*)full_sssp_kernel<4>
                   : g_full_lanes == 8 ? (const void*)full_sssp_kernel<8>
                                       : (const void*)full_sssp_kernel<16>;
  OGR_CUDA_TRY(cudaLaunchCooperativeKernel(fn, dim3(g_grid_blocks[dev]), dim3(kThreads), args, 0, s));
  return OGR_OK;
}

}  // namespace ogr_full

extern "C" int ogr_debug_limits(int32_t barrier_spin, int32_t max_phases, int32_t* cur_spin,
                                int32_t* cur_phases) {
  if (barrier_spin < -1 || max_phases < -1) return OGR_ERR_ARG;
  if (barrier_spin >= 0) g_dbg_spin = barrier_spin == 0 ? kBarSpin : (unsigned)barrier_spin - 1u;
  if (max_phases >= 0) g_dbg_phases = max_phases;
  if (cur_spin) *cur_spin = (int32_t)(g_dbg_spin == kBarSpin ? 0 : g_dbg_spin + 1u);
  if (cur_phases) *cur_phases = g_dbg_phases;
  return OGR_OK;
}

extern "C" int ogr_full_lanes(int32_t lanes, int32_t* current) {
  if (lanes != 0 && lanes != 4 && lanes != 8 && lanes != 16) return OGR_ERR_ARG;
  if (lanes != 0) g_full_lanes = lanes;
  if (current) *current = g_full_lanes;
  return OGR_OK;
}

extern "C" int ogr_full_reuse(int32_t mode, int32_t* current) {
  if (mode < -1 || mode > 1) return OGR_ERR_ARG;
  if (mode >= 0) g_full_reuse = mode;
  if (current) *current = g_full_reuse;
  return OGR_OK;
}

extern "C" int ogr_full_grid(int32_t ctas, int32_t* current, int32_t* limit) {
  int dev = 0;
  OGR_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return OGR_ERR_ARG;
  const int rc = size_grid(dev);
  if (rc != OGR_OK) return rc;
  if (ctas < 0 || ctas > g_grid_limit[dev]) return OGR_ERR_ARG;
  if (ctas > 0) g_grid_blocks[dev] = ctas;
  if (current) *current = g_grid_blocks[dev];
  if (limit) *limit = g_grid_limit[dev];
  return OGR_OK;
}

extern "C" size_t ogr_full_workspace_bytes(int32_t num_nodes, int64_t num_edges) {
  return ogr_full::workspace_bytes(num_nodes, num_edges);
}

extern "C" int ogr_full_workspace_init(void* ws, size_t bytes, int32_t num_nodes, int64_t num_edges,
                                       void* stream) {
  if (!ws || num_nodes < 1 || num_edges < 0) return OGR_ERR_ARG;
  if (bytes < ogr_full::workspace_bytes(num_nodes, num_edges)) return OGR_ERR_CAPACITY;
  FWs w;
  fws_layout(num_nodes, num_edges, (char*)ws, &w);
  // phase base 0: the first search clears the settle stamps; tile stamp 0:
  // the first tile search clears its node words
  cudaStream_t s = ogr_stream(stream);
  OGR_CUDA_TRY(cudaMemsetAsync(w.ctl, 0, sizeof(FCtl), s));
  OGR_CUDA_TRY(cudaMemsetAsync(w.tile, 0, ogr_tile::ctl_bytes(), s));
  // no node is a multi-source seed or target until a search marks it
  const int blocks = (int)std::min<int64_t>((num_nodes + 255) / 256, 152 * 8);
  fill_u64_kernel<<<blocks, 256, 0, s>>>(reinterpret_cast<unsigned long long*>(w.mseed), num_nodes, kNoTerm);
  OGR_LAUNCH_CHECK();
  fill_u64_kernel<<<blocks, 256, 0, s>>>(reinterpret_cast<unsigned long long*>(w.mtgt), num_nodes, kNoTerm);
  OGR_LAUNCH_CHECK();
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

extern "C" int ogr_find_path_full_multi(const ogr_graph* g, const ogr_state* st, const ogr_net_args* net,
                                        const int32_t* seeds, const double* seed_cost, int32_t n_seeds,
                                        const int32_t* targets, const double* target_cost, int32_t n_targets,
                                        void* ws, size_t bytes, int32_t* path_out, int32_t path_cap,
                                        int32_t* path_len_out, int64_t* stats, void* stream) {
  if (!g || !st || !net || !ws || !path_out || !path_len_out || path_cap < 2) return OGR_ERR_ARG;
  if (n_seeds < 0 || n_targets < 0 || (n_seeds > 0 && (!seeds || !seed_cost)) ||
      (n_targets > 0 && (!targets || !target_cost)))
    return OGR_ERR_ARG;
  if (bytes < ogr_full::workspace_bytes(g->num_nodes, g->num_edges)) return OGR_ERR_CAPACITY;
  *path_len_out = 0;
  if (n_seeds == 0 || n_targets == 0) return OGR_NO_PATH;
  ogr_full::Job job{};
  job.a = *net;
  job.path_out = path_out;
  job.path_cap = path_cap;
  job.stats = reinterpret_cast<unsigned long long*>(stats);
  job.multi = 1;
  job.seeds = seeds;
  job.seed_cost = seed_cost;
  job.n_seeds = n_seeds;
  job.targets = targets;
  job.target_cost = target_cost;
  job.n_targets = n_targets;
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
