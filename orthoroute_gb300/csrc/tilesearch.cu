// A7 for long nets, second engine: label windows over lattice tiles.
//
// The heap search of the reference (find_path_roi, unified_pathfinder.py:
// 2451-2548) gives every node v the lexicographic minimum of
// (float32(alt), L(u), u) over its in-neighbours u, alt = (L(u) + c) + pen(v)
// in float64.  With positive costs that rule has exactly one fixed point, so
// any procedure that stops at a fixed point returns the heap's labels and
// parents.  The phase-settled engine (fullgraph.cu) proves one hop final per
// grid step; this one propagates many hops per grid step and then checks
// that nothing moves any more:
//
//   * window: with T = the least unsettled label, the nodes whose labels
//     fall below B = T + delta are computed together; only nodes with a
//     label below B are sources.  When no label changes, every node below B
//     is final (each window's fixed point is the global one restricted to
//     it, and no unsettled node can end below B);
//   * tiles: the lattice is cut into columns of TX x TY cells over all
//     layers (vias never leave a column).  A CTA loads a tile into shared
//     memory (its CSR rows, in-arc costs, node penalties, the labels of the
//     tile and of the ring of cells around it) and iterates the rule on a
//     worklist until the tile is stable, so a label crosses a tile in one
//     grid step.  A tile whose boundary labels changed marks the tiles
//     beside it for the next grid step; a window ends after a grid step in
//     which nothing was marked.
//
// Arithmetic: every finite cost and node penalty of at least 2^-7 is a
// multiple of 2^-30 (float32), so while labels stay below 2^23 the float64
// sums of the reference are exact and equal the int64 sums of labels in
// units of 2^-30 ("ticks"); float32(alt) is the int64 -> float32 rounding
// scaled by 2^-30.  A search that meets a smaller cost or penalty, a larger
// label, a tile over the shared-memory capacity or an iteration cap stops
// and hands the net to the phase-settled engine (tile_gate = 1), so every
// result is the heap's.
//
// Per-node state: one 64-bit word per node (search stamp in the top 11 bits,
// ticks below) read and written whole, so no reader sees half an update;
// the winner is kept in a separate array read only by its tile's owner and
// the backtrace.  Every tile is always processed by the same CTA (tile id
// modulo the grid), the only writer of its words.  Per tile: the least
// unsettled label and, per side, the least label of its boundary cells at or
// above the window bound.
#include <cooperative_groups.h>

#include <atomic>

#include "fullgraph.cuh"

namespace ogr_tile {
// Tracing counters (ogr_tile_profile): [0] searches, [1] grid rounds,
// [2] windows, [3] kernel ns, [4] searches handed to the phase engine,
// [5] bit set of the reasons for handing over (1 << kWhy*), [6] local
// iterations, [7] tile processings; per-stage globaltimer ns summed over the
// CTAs: [8] structure loads, [9] label loads, [10] local iterations,
// [11] write-back, [12] barrier waits; [13] structure loads, [14] most
// tiles one CTA processed in a round, [15] node evaluations, [16] ns of
// first sweeps.
__device__ unsigned long long g_tile_prof[24];
}  // namespace ogr_tile

namespace {

constexpr int kT = 1024;                         // threads per CTA
constexpr int kMaxNodes = 2048;                  // nodes of a tile
constexpr int kMaxArcs = 18432;                  // arcs of a tile's rows
constexpr int kMaxHalo = 1024;                   // ring cells around a tile (all layers)
constexpr int kMaxTiles = 65536;                 // tiles of a lattice (else: phase engine)
constexpr int kMaxOwn = 512;                     // tiles of one CTA listed in a round
constexpr long long kInf = (1LL << 53) - 1;      // "no label"
constexpr unsigned long long kTickMask = (1ULL << 53) - 1;
constexpr int kStampMax = 2047;                  // 11-bit search stamp, 0 = never valid
constexpr unsigned kBarSpin = 1u << 22;

// Knobs of the engine (ogr_full_tile), per host thread: tile size in cells
// and the window width delta in label units; enable = 0 keeps the phase
// engine.
thread_local int g_tile_enable = 0;
thread_local int g_tile_tx = 0, g_tile_ty = 0;    // 0: chosen from the lattice
thread_local double g_tile_delta = 0.0;

struct TCtl {
  alignas(128) unsigned long long bar_count;     // monotone arrival counter (zeroed per launch)
  alignas(128) int32_t bar_err;
  alignas(128) int32_t err;                      // a precondition or cap failed: hand over (reason)
  alignas(128) int32_t nlist[3];                 // lengths of the three rotating tile lists
  alignas(128) int32_t stamp;                    // persistent: stamp of the last search
  uint32_t round_base;                           // persistent: global round numbering
};

struct TWs {
  TCtl* ctl;
  unsigned long long* word;   // [N] stamp << 53 | ticks
  int32_t* par;               // [N] winner (valid where word carries the stamp)
  // Per-tile minima, double-buffered by window parity: window k reads buffer
  // k & 1 (complete after the previous window) and writes the other, into
  // which each CTA first copies its own tiles, so no CTA reads a value that
  // another is rewriting.
  unsigned long long* minf[2];   // [kMaxTiles] least unsettled label of each tile
  unsigned long long* side[2];   // [4 * kMaxTiles] least boundary label >= B per side (W, E, S, N)
  uint32_t* mark;                // [kMaxTiles] round in which the tile was last listed
  int32_t* list[3];              // [kMaxTiles] tiles to process in a round
};

constexpr size_t r256(size_t v) { return (v + 255) & ~(size_t)255; }

size_t tws_layout(int32_t N, char* base, TWs* w) {
  const size_t tiles = kMaxTiles;
  size_t off = 0;
  auto take = [&](size_t b) -> char* {
    char* p = base ? base + off : nullptr;
    off += r256(b);
    return p;
  };
  TWs t{};
  t.ctl = (TCtl*)take(sizeof(TCtl));
  t.word = (unsigned long long*)take(8 * (size_t)N);
  t.par = (int32_t*)take(4 * (size_t)N);
  for (int i = 0; i < 2; ++i) {
    t.minf[i] = (unsigned long long*)take(8 * tiles);
    t.side[i] = (unsigned long long*)take(32 * tiles);
  }
  t.mark = (uint32_t*)take(4 * tiles);
  for (int i = 0; i < 3; ++i) t.list[i] = (int32_t*)take(4 * tiles);
  if (w) *w = t;
  return off;
}

// Geometry of the tiling, the same on every CTA.
struct Geo {
  int nx, ny, nz, tx, ty, tm, ntx, nty;
  int64_t plane;
  int ntiles;
  float inv_plane;           // 1 / plane: the layer step of a via arc, checked exactly
};

// Shared memory of a CTA (dynamic; one tile resident at a time).
struct Sm {
  long long lab[kMaxNodes + kMaxHalo];   // ticks of the tile's nodes, then of the ring
  int32_t par[kMaxNodes];
  long long pen[kMaxNodes];              // node penalty in ticks
  uint16_t rs[kMaxNodes + 1];            // tile-local row starts
  uint16_t anb[kMaxArcs];                // slot of each in-neighbour
  float acost[kMaxArcs];                 // cost of the arc in-neighbour -> node
  int32_t hgid[kMaxHalo];                // global id of each ring slot (-1: off the lattice)
  int32_t gid[kMaxNodes];                // global id of each tile node
  int32_t f0[kMaxNodes];                 // global CSR row start of each tile node
  uint32_t rmask[kMaxNodes / 8];         // 4 bits per node: ring sides (W, E, S, N) its arcs reach
  uint32_t wl[3][kMaxNodes / 32];        // activation bitmaps of three consecutive iterations
  uint32_t chg[kMaxNodes / 32];          // label or winner changed since the load
  uint32_t lchg[kMaxNodes / 32];         // label changed since the load
  int32_t scan[kT / 32 + 1];
  unsigned long long red[kT / 32];
  unsigned long long sred[4][kT / 32];
  int32_t own[kMaxOwn];                  // this CTA's tiles of the current round
  int32_t nown;
  int32_t cached;                        // tile whose structure is resident (-1: none)
  int32_t nt, narcs, x0, y0, tw, th, srcl;
  int flag;
  int sidemark[4];
};

static_assert(sizeof(Sm) <= 200 * 1024, "a tile must leave room in the 227 KB of shared memory");

__device__ __forceinline__ unsigned long long ld_word(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_word(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

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

// Label of a node word under the search stamp (kInf when not labelled).
__device__ __forceinline__ long long word_ticks(unsigned long long w, unsigned stamp) {
  return (unsigned)(w >> 53) == stamp ? (long long)(w & kTickMask) : kInf;
}

// float32 value -> ticks; false when the value is not a multiple of 2^-30
// below 2^23 that the int64 sums can carry exactly (zero -> 0).
__device__ __forceinline__ bool f32_ticks(float v, long long& t) {
  const unsigned b = __float_as_uint(v);
  if (b == 0u) {
    t = 0;
    return true;
  }
  const int e = (int)((b >> 23) & 0xffu) - 127;
  if ((b >> 31) || e < -7 || e > 22) return false;
  t = (long long)((b & 0x7fffffu) | 0x800000u) << (e + 7);
  return true;
}

// The largest tick count whose float32 rounding (x 2^-30, to nearest, ties
// to even; 30 - 23 = 7 is not needed here, only the mantissa spacing) equals
// that of t, from integer operations.  t >= 1.
__device__ __forceinline__ long long round_hi(long long t) {
  const unsigned long long u = (unsigned long long)t;
  const int nb = 64 - __clzll(u);
  if (nb <= 24) return t;                    // exact: no other integer rounds to it
  const int sh = nb - 24;
  unsigned long long m = u >> sh;
  const unsigned long long rem = u & ((1ull << sh) - 1ull);
  const unsigned long long half = 1ull << (sh - 1);
  if (rem > half || (rem == half && (m & 1ull))) ++m;
  int e = sh;
  if (m == (1ull << 24)) {
    m >>= 1;
    ++e;
  }
  return (long long)((m << e) + (1ull << (e - 1)) - (m & 1ull));
}

// Grid barrier on a monotone arrival counter (bounded wait; false when any
// CTA gave up).
__device__ bool tbarrier(TCtl* c, unsigned long long& target, Sm& sm) {
  __syncthreads();
  if (threadIdx.x == 0) {
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
  }
  __syncthreads();
  return sm.flag != 0;
}

// Why a search was handed over (the first reason is kept; the profile
// counters record each reason's bit).
enum : int32_t {
  kWhyTileNodes = 1, kWhyTileArcs = 2, kWhyRing = 3, kWhyPenalty = 4, kWhyLocalCap = 5, kWhyArcCost = 6,
  kWhyOwn = 7, kWhyWindows = 8, kWhyRounds = 9, kWhyTotal = 10
};

__device__ __forceinline__ void fail(TCtl* c, int32_t why) { atomicCAS(&c->err, 0, why); }

// Global id of tile slot s (s < nt: a tile node; else a ring slot).
__device__ __forceinline__ int32_t slot_gid(const Sm& sm, int s) {
  return s >= sm.nt ? sm.hgid[s - sm.nt] : sm.gid[s];
}

// Block-wide exclusive scan of one value per thread (returns the total).
__device__ int block_scan(Sm& sm, int v, int& excl) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm.scan[wid] = x;
  __syncthreads();
  if (wid == 0) {
    const int w = lane < kT / 32 ? sm.scan[lane] : 0;
    int s = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < kT / 32) sm.scan[lane] = s - w;
    if (lane == 31) sm.scan[kT / 32] = s;
  }
  __syncthreads();
  excl = sm.scan[wid] + x - v;
  const int total = sm.scan[kT / 32];
  __syncthreads();
  return total;
}

// Loads the rows, in-arc costs, penalties and ring ids of tile t (the part
// that does not change during a search).  Tile node i sits in row chunk
// c = i / tw = z * th + ly (tw nodes of consecutive global ids), whose CSR
// rows are contiguous, so one warp copies a chunk's arcs with coalesced
// loads.  False (and err set) when the tile exceeds the shared-memory
// capacity, an arc is not a lattice step inside the tile or to its ring, or
// a penalty is off the exact grid.
__device__ bool load_structure(Sm& sm, const Geo& G, int t, int32_t src, const ogr_graph& g,
                               const ogr_state& st, const ogr_net_args& a, TCtl* ctl) {
  const int tid = threadIdx.x;
  if (tid == 0) {
    const int tyi = t / G.ntx, txi = t - tyi * G.ntx;
    sm.x0 = txi * G.tx;
    sm.y0 = tyi * G.ty;
    sm.tw = min(G.tx, G.nx - sm.x0);
    sm.th = min(G.ty, G.ny - sm.y0);
    sm.nt = sm.tw * sm.th * G.nz;
    sm.cached = -1;
    const int sz = (int)(src / G.plane);
    const int sr = (int)(src - (int64_t)sz * G.plane);
    const int sy = sr / G.nx, sx = sr - sy * G.nx;
    sm.srcl = (sx >= sm.x0 && sx < sm.x0 + sm.tw && sy >= sm.y0 && sy < sm.y0 + sm.th)
                  ? (sz * sm.th + (sy - sm.y0)) * sm.tw + (sx - sm.x0)
                  : -1;
  }
  __syncthreads();
  const int nt = sm.nt, tw = sm.tw, th = sm.th, x0 = sm.x0, y0 = sm.y0;
  if (nt > kMaxNodes) {
    if (tid == 0) fail(ctl, kWhyTileNodes);
    return false;
  }
  // node ids, row lengths and penalties: two consecutive nodes per thread
  int deg[2] = {0, 0};
  bool badpen = false;
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int i = 2 * tid + k;
    if (i < nt) {
      const int c = i / tw, lx = i - c * tw;
      const int z = c / th, ly = c - z * th;
      const int32_t gid = (int32_t)((int64_t)z * G.plane + (int64_t)(y0 + ly) * G.nx + x0 + lx);
      sm.gid[i] = gid;
      const int32_t r0 = g.indptr[gid];
      sm.f0[i] = r0;
      deg[k] = g.indptr[gid + 1] - r0;
      long long pt;
      if (!f32_ticks(ogr_node_penalty(st, a, gid), pt)) badpen = true;
      sm.pen[i] = pt;
    }
  }
  int excl = 0;
  const int total = block_scan(sm, deg[0] + deg[1], excl);
  if (total > kMaxArcs) {
    if (tid == 0) fail(ctl, kWhyTileArcs);
    return false;
  }
  if (2 * tid < nt) sm.rs[2 * tid] = (uint16_t)excl;
  if (2 * tid + 1 < nt) sm.rs[2 * tid + 1] = (uint16_t)(excl + deg[0]);
  if (tid == 0) sm.rs[nt] = (uint16_t)total;
  for (int k = tid; k < kMaxNodes / 8; k += kT) sm.rmask[k] = 0u;
  const int nh = 4 * G.nz * G.tm;
  for (int h = tid; h < nh; h += kT) {
    const int sd = h / (G.nz * G.tm);
    const int rem = h - sd * G.nz * G.tm;
    const int z = rem / G.tm;
    const int off = rem - z * G.tm;
    int ux, uy;
    bool ok;
    if (sd < 2) {
      ux = sd == 0 ? x0 - 1 : x0 + tw;
      uy = y0 + off;
      ok = off < th && ux >= 0 && ux < G.nx;
    } else {
      uy = sd == 2 ? y0 - 1 : y0 + th;
      ux = x0 + off;
      ok = off < tw && uy >= 0 && uy < G.ny;
    }
    sm.hgid[h] = ok ? (int32_t)((int64_t)z * G.plane + (int64_t)uy * G.nx + ux) : -1;
  }
  __syncthreads();
  // arcs, one warp per row chunk
  const int lane = tid & 31, wid = tid >> 5;
  bool bad = false;
  const int nchunks = th * G.nz;
  for (int c = wid; c < nchunks; c += kT / 32) {
    const int i0 = c * tw;
    const int z = c / th, ly = c - z * th;
    const int l0 = sm.rs[i0], l1 = sm.rs[i0 + tw];
    const int64_t gf0 = sm.f0[i0];
    for (int e = l0 + lane; e < l1; e += 32) {
      const int64_t f = gf0 + (e - l0);
      const int32_t u = g.indices[f];
      const float cst = st.rcost ? st.rcost[f] : st.total_cost[g.rev[f]];
      int lo = i0, hi = i0 + tw;                 // rs[lo] <= e < rs[hi]
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if ((int)sm.rs[mid] <= e) lo = mid;
        else hi = mid;
      }
      const int i = lo, lx = i - i0;
      const int d = u - sm.gid[i];
      int slot = -1, side = -1;
      if (G.nx > 1 && (d == 1 || d == -1)) {
        const int nlx = lx + d;
        if (nlx >= 0 && nlx < tw) {
          slot = i + d;
        } else {
          side = d < 0 ? 0 : 1;
          slot = nt + (side * G.nz + z) * G.tm + ly;
        }
      } else if (G.ny > 1 && (d == G.nx || d == -G.nx)) {
        const int nly = ly + (d > 0 ? 1 : -1);
        if (nly >= 0 && nly < th) {
          slot = i + (d > 0 ? tw : -tw);
        } else {
          side = d < 0 ? 2 : 3;
          slot = nt + (side * G.nz + z) * G.tm + lx;
        }
      } else {
        const int dz = __float2int_rn((float)d * G.inv_plane);
        if ((int64_t)dz * G.plane == (int64_t)d && z + dz >= 0 && z + dz < G.nz) slot = i + dz * tw * th;
      }
      if (slot < 0 || slot_gid(sm, slot) != u) {   // not a lattice step of this tile or its ring
        bad = true;
        slot = 0;
      }
      if (side >= 0) atomicOr(&sm.rmask[i >> 3], 1u << (4 * (i & 7) + side));
      sm.anb[e] = (uint16_t)slot;
      sm.acost[e] = cst;
    }
  }
  const bool anybad = __syncthreads_or(bad) != 0;
  const bool anypen = __syncthreads_or(badpen) != 0;
  if (anybad || anypen) {
    if (tid == 0) fail(ctl, anybad ? kWhyRing : kWhyPenalty);
    return false;
  }
  if (tid == 0) {
    sm.narcs = total;
    sm.cached = t;
  }
  __syncthreads();
  return true;
}

template <typename F>
__device__ __forceinline__ void for_my_nodes(int nt, F f) {
  for (int i = threadIdx.x; i < nt; i += kT) f(i);
}

// Processes tile t for the window [wstart, B): loads the labels of the tile
// and its ring, iterates the rule on a worklist until no label of the tile
// changes, writes back what changed, lists the tiles beside changed boundary
// cells for round `rnext` (global round id gnext), and stores the tile's
// least unsettled label and per-side boundary minima into buffer wb.  False
// on a failure (err set).
__device__ bool process_tile(Sm& sm, const Geo& G, int t, const ogr_graph& g, const ogr_state& st,
                             const ogr_net_args& a, const TWs& w, unsigned stamp, int32_t src, long long wstart,
                             long long B, int rnext, uint32_t gnext, int wb) {
  const int tid = threadIdx.x;
  unsigned long long tm0 = tid == 0 ? gtimer() : 0;
  if (sm.cached != t) {
    if (!load_structure(sm, G, t, src, g, st, a, w.ctl)) return false;
    if (tid == 0) {
      const unsigned long long t1 = gtimer();
      atomicAdd(&ogr_tile::g_tile_prof[8], t1 - tm0);
      atomicAdd(&ogr_tile::g_tile_prof[13], 1ull);
      tm0 = t1;
    }
  }
  const int nt = sm.nt;
  const int nh = 4 * G.nz * G.tm;
  const int nwords = (nt + 31) >> 5;
  // labels of the tile (with winners) and of the ring
  for_my_nodes(nt, [&](int i) {
    const int32_t gid = sm.gid[i];
    const long long lt = word_ticks(ld_word(&w.word[gid]), stamp);
    sm.lab[i] = lt;
    sm.par[i] = lt < kInf ? __ldcg(&w.par[gid]) : -1;
  });
  for (int h = tid; h < nh; h += kT) {
    const int32_t gid = sm.hgid[h];
    sm.lab[nt + h] = gid >= 0 ? word_ticks(ld_word(&w.word[gid]), stamp) : kInf;
  }
  for (int k = tid; k < nwords; k += kT) {
    sm.wl[0][k] = 0u;
    sm.wl[1][k] = 0u;
    sm.wl[2][k] = 0u;
    sm.chg[k] = 0u;
    sm.lchg[k] = 0u;
  }
  if (tid < 4) sm.sidemark[tid] = 0;
  if (tid == 0) sm.flag = 1;
  __syncthreads();
  if (tid == 0) {
    const unsigned long long t1 = gtimer();
    atomicAdd(&ogr_tile::g_tile_prof[9], t1 - tm0);
    tm0 = t1;
  }
  // Iteration 0 evaluates every node; iteration k evaluates the nodes with
  // an in-tile in-neighbour whose label changed in iteration k - 1.  A node
  // whose label changes marks its in-tile neighbours in the next
  // iteration's bitmap (lattice arcs come in pairs, so its in-neighbours are
  // the nodes it feeds): a node's activity is one bit, not a walk over its
  // in-neighbours.  Bitmaps rotate over three buffers: iteration k reads
  // wl[k % 3], marks wl[(k + 1) % 3] and clears wl[(k + 2) % 3], whose last
  // reader finished at the previous barrier.  Node i = base + tid: a warp
  // owns one 32-bit word of chg / lchg and writes it from a ballot.  One
  // barrier per iteration.
  const int lane = tid & 31, wid = tid >> 5;
  unsigned nev_all = 0;
  const int cap = 4 * nt + 64;
  int it = 0;
  for (;; ++it) {
    if (it >= cap) {
      if (tid == 0) fail(w.ctl, kWhyLocalCap);
      return false;
    }
    const int rd = it % 3, mk = (it + 1) % 3, clr = (it + 2) % 3;
    for (int k = tid; k < nwords; k += kT) sm.wl[clr][k] = 0u;
    bool changed = false, bad = false;
    unsigned nev = 0;
    for (int base = 0; base < nt; base += kT) {
      const int i = base + tid;
      bool ch = false, lch = false;
      if (i < nt) {
        const long long li = sm.lab[i];
        bool act = li >= wstart && i != sm.srcl;    // settled nodes and the source never change
        const int r0 = sm.rs[i], r1 = sm.rs[i + 1];
        if (act && it > 0) act = (sm.wl[rd][i >> 5] >> (i & 31)) & 1u;
        if (act) {
          ++nev;
          const long long pt = sm.pen[i];
          // pass 1: the least alt (ticks); float32 rounding is monotone, so
          // the winners of (float32(alt), L(u), u) are the candidates whose
          // alt rounds like it: alt <= hi, the largest such tick count
          long long amin = kInf;
          for (int k = r0; k < r1; ++k) {
            const long long lu = sm.lab[sm.anb[k]];
            if (lu >= B) continue;                      // not a source of this window (or none)
            const float c = sm.acost[k];
            if (!(c < __int_as_float(0x7f800000))) continue;   // blocked arc
            long long ct;
            if (!f32_ticks(c, ct)) {
              bad = true;
              continue;
            }
            const long long alt = lu + ct + pt;
            if (alt >= kInf) {
              bad = true;
              continue;
            }
            amin = alt < amin ? alt : amin;
          }
          long long nl = kInf;
          int32_t np = -1;
          if (amin < kInf) {
            const long long hi = round_hi(amin);
            // pass 2: the least (L(u), u) among them
            long long bl = kInf;
            int bs = -1;
            int32_t bg = -1;   // global id of the best source, computed only on a tie of L(u)
            for (int k = r0; k < r1; ++k) {
              const int s = sm.anb[k];
              const long long lu = sm.lab[s];
              if (lu >= B || lu > bl) continue;
              const float c = sm.acost[k];
              if (!(c < __int_as_float(0x7f800000))) continue;
              long long ct;
              f32_ticks(c, ct);
              const long long alt = lu + ct + pt;
              if (alt > hi) continue;
              if (lu < bl) {
                bl = lu;
                bs = s;
                nl = alt;
                bg = -1;
              } else {                                  // same L(u): the lower node id
                const int32_t ug = slot_gid(sm, s);
                if (bg < 0) bg = slot_gid(sm, bs);
                if (ug < bg) {
                  bs = s;
                  nl = alt;
                  bg = ug;
                }
              }
            }
            np = bg >= 0 ? bg : slot_gid(sm, bs);
          }
          if (nl != li || np != sm.par[i]) {
            ch = true;
            sm.par[i] = np;
            if (nl != li) {
              sm.lab[i] = nl;
              lch = true;
              for (int k = r0; k < r1; ++k) {   // wake the in-tile nodes this one feeds
                const int s2 = sm.anb[k];
                if (s2 < nt) atomicOr(&sm.wl[mk][s2 >> 5], 1u << (s2 & 31));
              }
            }
          }
        }
      }
      const unsigned bl_ = __ballot_sync(0xffffffffu, lch);
      const unsigned bc_ = __ballot_sync(0xffffffffu, ch);
      const int word = (base >> 5) + wid;
      if (lane == 0 && word < nwords) {
        sm.chg[word] |= bc_;
        sm.lchg[word] |= bl_;
      }
      changed |= lch;
    }
    if (bad) sm.flag = 0;
    nev_all += nev;
    // sm.flag is 1 here unless a thread met an arc off the exact grid
    const bool any = __syncthreads_or(changed || bad) != 0;
    if (it == 0 && tid == 0) atomicAdd(&ogr_tile::g_tile_prof[16], gtimer() - tm0);
    if (any && sm.flag == 0) {
      if (tid == 0) fail(w.ctl, kWhyArcCost);
      return false;
    }
    if (!any) break;
  }
  nev_all = __reduce_add_sync(0xffffffffu, nev_all);
  if (lane == 0 && nev_all) atomicAdd(&ogr_tile::g_tile_prof[15], (unsigned long long)nev_all);
  if (tid == 0) {
    atomicAdd(&ogr_tile::g_tile_prof[6], (unsigned long long)(it + 1));
    atomicAdd(&ogr_tile::g_tile_prof[7], 1ull);
    const unsigned long long t1 = gtimer();
    atomicAdd(&ogr_tile::g_tile_prof[10], t1 - tm0);
    tm0 = t1;
  }
  // write back; list the tiles beside changed boundary cells; minima
  unsigned long long mn = ~0ull, smn[4] = {~0ull, ~0ull, ~0ull, ~0ull};
  for_my_nodes(nt, [&](int i) {
    const long long li = sm.lab[i];
    const bool ch = (sm.chg[i >> 5] >> (i & 31)) & 1u;
    const bool lch = (sm.lchg[i >> 5] >> (i & 31)) & 1u;
    if (ch) {
      const int32_t gid = sm.gid[i];
      w.par[gid] = sm.par[i];
      st_word(&w.word[gid], ((unsigned long long)stamp << 53) | (unsigned long long)li);
    }
    const unsigned sides = (sm.rmask[i >> 3] >> (4 * (i & 7))) & 0xfu;
#pragma unroll
    for (int sd = 0; sd < 4; ++sd) {
      if (!((sides >> sd) & 1u)) continue;
      if (lch) sm.sidemark[sd] = 1;
      if (li >= B && li < kInf) smn[sd] = min(smn[sd], (unsigned long long)li);
    }
    if (li >= B && li < kInf) mn = min(mn, (unsigned long long)li);
  });
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
#pragma unroll
    for (int d = 0; d < 4; ++d) smn[d] = min(smn[d], __shfl_xor_sync(0xffffffffu, smn[d], o));
  }
  if (lane == 0) {
    sm.red[wid] = mn;
#pragma unroll
    for (int d = 0; d < 4; ++d) sm.sred[d][wid] = smn[d];
  }
  __syncthreads();
  if (tid < 5) {
    unsigned long long m = ~0ull;
    for (int k = 0; k < kT / 32; ++k) m = min(m, tid == 0 ? sm.red[k] : sm.sred[tid - 1][k]);
    const unsigned long long v = m == ~0ull ? (unsigned long long)kInf : m;
    if (tid == 0) w.minf[wb][t] = v;
    else w.side[wb][4 * (int64_t)t + tid - 1] = v;
  }
  if (tid < 4 && sm.sidemark[tid]) {
    const int tyi = t / G.ntx, txi = t - tyi * G.ntx;
    int nb = -1;
    if (tid == 0 && txi > 0) nb = t - 1;
    if (tid == 1 && txi + 1 < G.ntx) nb = t + 1;
    if (tid == 2 && tyi > 0) nb = t - G.ntx;
    if (tid == 3 && tyi + 1 < G.nty) nb = t + G.ntx;
    if (nb >= 0 && atomicExch(&w.mark[nb], gnext) != gnext) {
      const int idx = atomicAdd(&w.ctl->nlist[rnext], 1);
      w.list[rnext][idx] = nb;
    }
  }
  __syncthreads();
  if (tid == 0) atomicAdd(&ogr_tile::g_tile_prof[11], gtimer() - tm0);
  return true;
}

__global__ void __launch_bounds__(kT, 1)
tile_sssp_kernel(ogr_graph g, ogr_state st, ogr_full::Job job, TWs w, Geo G, long long delta,
                 int32_t* res, int32_t* gate) {
  extern __shared__ __align__(16) unsigned char smraw[];
  Sm& sm = *reinterpret_cast<Sm*>(smraw);
  uint32_t* abits = reinterpret_cast<uint32_t*>(smraw + ((sizeof(Sm) + 15) & ~(size_t)15));
  const int tid = threadIdx.x;
  const unsigned cta = blockIdx.x, ncta = gridDim.x;
  const int64_t gtid = (int64_t)cta * kT + tid;
  const int64_t gthreads = (int64_t)ncta * kT;
  const bool leader = gtid == 0;
  TCtl* ctl = w.ctl;

  if (job.from_pass && job.pass_result[0] < 0) return;   // uniform: written by an earlier launch
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
  const int32_t src = a.src, dst = a.dst;
  if (src == dst) {
    if (leader) {
      res[0] = OGR_NO_PATH;
      res[1] = 0;
      res[2] = 0;
      *gate = 0;
    }
    return;
  }
  const unsigned long long t_start = gtimer();
  if (tid == 0) sm.cached = -1;
  // the search stamp; on wrap-around (and on first use) every node word and
  // tile mark is cleared
  const int prev = __ldcg(&ctl->stamp);
  const uint32_t rbase = __ldcg(&ctl->round_base);
  const bool fresh = prev < 1 || prev >= kStampMax;
  const unsigned stamp = fresh ? 1u : (unsigned)prev + 1u;
  if (fresh) {
    for (int64_t i = gtid; i < N; i += gthreads) w.word[i] = 0ull;
    for (int64_t i = gtid; i < G.ntiles; i += gthreads) w.mark[i] = 0u;
  }
  uint32_t gr = fresh ? 1u : rbase;                 // global id of the current round
  for (int64_t i = gtid; i < G.ntiles; i += gthreads) {
    w.minf[0][i] = (unsigned long long)kInf;
#pragma unroll
    for (int d = 0; d < 4; ++d) w.side[0][4 * i + d] = (unsigned long long)kInf;
  }
  const int64_t sr = src % G.plane;
  const int src_tile = (int)((sr % G.nx) / G.tx) + (int)((sr / G.nx) / G.ty) * G.ntx;
  unsigned long long bar_target = 0;
  if (leader) {
    ctl->err = 0;
    for (int i = 0; i < 3; ++i) ctl->nlist[i] = 0;
  }
  bool alive = tbarrier(ctl, bar_target, sm);
  if (leader) {
    st_word(&w.word[src], (unsigned long long)stamp << 53);
    w.par[src] = -1;
    w.minf[0][src_tile] = 0ull;
  }
  alive = alive && tbarrier(ctl, bar_target, sm);

  long long wstart = -1;      // labels below it are final
  int status = OGR_OK;
  bool found = false, failed = false;
  int32_t why = 0;
  int rounds = 0, windows = 0;
  long long ld = kInf;
  const int nab = (G.ntiles + 31) >> 5;
  const int max_windows = 4 * N + 16;
  const int max_rounds = 4 * G.ntiles + 64;          // per window
  const int max_total = 64 * G.ntiles + 16384;       // per search
  int rb = 0;                  // per-tile minima of the finished windows: buffer rb
  while (alive) {
    if (__ldcg(&ctl->err)) {
      failed = true;
      break;
    }
    const int wb = rb ^ 1;
    // least unsettled label over all tiles, and the destination's label (a
    // settled label never changes and an unsettled one never falls below
    // wstart, so every CTA reaches the same decision)
    unsigned long long m = ~0ull;
    for (int t = tid; t < G.ntiles; t += kT) m = min(m, __ldcg(&w.minf[rb][t]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((tid & 31) == 0) sm.red[tid >> 5] = m;
    __syncthreads();
    if (tid == 0) {
      unsigned long long x = ~0ull;
      for (int k = 0; k < kT / 32; ++k) x = min(x, sm.red[k]);
      sm.red[0] = x;
    }
    __syncthreads();
    const long long T = (long long)sm.red[0];
    ld = word_ticks(ld_word(&w.word[dst]), stamp);
    __syncthreads();
    if (ld < wstart) {          // dst final, and with it every cheaper node
      found = true;
      break;
    }
    if (T >= kInf) {
      status = OGR_NO_PATH;
      break;
    }
    if (++windows > max_windows) {
      failed = true;
      why = kWhyWindows;
      break;
    }
    const long long B = (T > kInf - delta) ? kInf : T + delta;
    // the window's first grid step: tiles with an unsettled label below B,
    // and the tiles beside a side whose boundary holds a label that becomes
    // a source now
    for (int k = tid; k < nab; k += kT) abits[k] = 0u;
    __syncthreads();
    for (int t = tid; t < G.ntiles; t += kT) {
      if ((long long)__ldcg(&w.minf[rb][t]) < B) atomicOr(&abits[t >> 5], 1u << (t & 31));
      const int tyi = t / G.ntx, txi = t - tyi * G.ntx;
#pragma unroll
      for (int d = 0; d < 4; ++d) {
        if ((long long)__ldcg(&w.side[rb][4 * (int64_t)t + d]) >= B) continue;
        int nb = -1;
        if (d == 0 && txi > 0) nb = t - 1;
        if (d == 1 && txi + 1 < G.ntx) nb = t + 1;
        if (d == 2 && tyi > 0) nb = t - G.ntx;
        if (d == 3 && tyi + 1 < G.nty) nb = t + G.ntx;
        if (nb >= 0) atomicOr(&abits[nb >> 5], 1u << (nb & 31));
      }
    }
    // this CTA's tiles carry their minima into the buffer the window writes
    for (int t = (int)cta + (int)ncta * (tid / 8); t < G.ntiles; t += (int)ncta * (kT / 8)) {
      const int d = tid & 7;
      if (d == 0) w.minf[wb][t] = __ldcg(&w.minf[rb][t]);
      else if (d < 5) w.side[wb][4 * (int64_t)t + d - 1] = __ldcg(&w.side[rb][4 * (int64_t)t + d - 1]);
    }
    __syncthreads();
    int nlist = -1;   // -1: the window's first grid step reads the bitmap
    int wrounds = 0;
    while (true) {
      if (++wrounds > max_rounds || rounds >= max_total) {
        failed = true;
        why = wrounds > max_rounds ? kWhyRounds : kWhyTotal;
        break;
      }
      // list rotation over all rounds of the search: round r reads list r%3
      // (rounds after the first of a window), appends to (r+1)%3 and clears
      // (r+2)%3, which round r-1 read
      const int rcur = rounds % 3, rnext = (rounds + 1) % 3, rclear = (rounds + 2) % 3;
      if (leader) ctl->nlist[rclear] = 0;
      const uint32_t gnext = gr + 1;
      int nproc = 0;
      if (nlist < 0) {
        for (int t = (int)cta; t < G.ntiles; t += (int)ncta) {
          if (!((abits[t >> 5] >> (t & 31)) & 1u)) continue;
          ++nproc;
          if (!process_tile(sm, G, t, g, st, a, w, stamp, src, wstart, B, rnext, gnext, wb)) break;
        }
      } else {
        // every tile is always processed by the same CTA (t mod grid), which
        // keeps its structure resident and makes it the only writer of the
        // tile's words
        if (tid == 0) sm.nown = 0;
        __syncthreads();
        for (int k = tid; k < nlist; k += kT) {
          const int t = __ldcg(&w.list[rcur][k]);
          if (t % (int)ncta != (int)cta) continue;
          const int j = atomicAdd(&sm.nown, 1);
          if (j < kMaxOwn) sm.own[j] = t;
        }
        __syncthreads();
        const int nown = sm.nown;
        if (nown > kMaxOwn) {
          if (tid == 0) fail(ctl, kWhyOwn);
        } else {
          nproc = nown;
          for (int j = 0; j < nown; ++j)
            if (!process_tile(sm, G, sm.own[j], g, st, a, w, stamp, src, wstart, B, rnext, gnext, wb)) break;
        }
      }
      const unsigned long long tb0 = tid == 0 ? gtimer() : 0;
      alive = tbarrier(ctl, bar_target, sm);
      if (tid == 0) {
        atomicAdd(&ogr_tile::g_tile_prof[12], gtimer() - tb0);
        atomicMax(&ogr_tile::g_tile_prof[14], (unsigned long long)nproc);
      }
      ++gr;
      if (!alive) break;
      if (__ldcg(&ctl->err)) {
        failed = true;
        break;
      }
      nlist = __ldcg(&ctl->nlist[rnext]);
      ++rounds;
      if (nlist == 0) break;
    }
    if (!alive || failed) break;
    wstart = B;
    rb = wb;
  }
  if (!alive) status = OGR_ERR_TIMEOUT;
  if (failed) status = OGR_ERR_ITER_CAP;
  // statistics: the nodes the sequential heap pops before dst, and their rows;
  // a search that cannot reach dst pops every node it reaches (every finite
  // label is final once no label below the infinity is left)
  const bool exhausted = status == OGR_NO_PATH;
  if ((found || exhausted) && job.stats) {
    unsigned long long arcs = 0, pops = 0;
    for (int64_t i = gtid; i < N; i += gthreads) {
      const long long li = word_ticks(ld_word(&w.word[i]), stamp);
      if (exhausted ? li < kInf : (li < ld || (li == ld && i < dst))) {
        arcs += (unsigned long long)(g.indptr[i + 1] - g.indptr[i]);
        ++pops;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      arcs += __shfl_xor_sync(0xffffffffu, arcs, o);
      pops += __shfl_xor_sync(0xffffffffu, pops, o);
    }
    if ((tid & 31) == 0 && pops) {
      atomicAdd(&job.stats[0], arcs);
      atomicAdd(&job.stats[1], pops);
    }
    if (leader) {
      if (found) atomicAdd(&job.stats[1], 1ull);   // dst's own pop
      atomicAdd(&job.stats[2], (unsigned long long)N);
      atomicAdd(&job.stats[3], (unsigned long long)rounds);
    }
  }
  if (cta != 0 || tid != 0) return;
  int len = 0;
  if (found) {
    const int limit = min(path_cap, N);
    int32_t c = dst;
    while (c != -1 && len < limit) {
      path_out[len++] = c;
      c = __ldcg(&w.par[c]);
    }
    if (c != -1) status = len >= N ? OGR_ERR_ITER_CAP : OGR_ERR_CAPACITY;
    else if (len < 2) status = OGR_NO_PATH;
    for (int i = 0; i < len / 2; ++i) {
      const int32_t x = path_out[i];
      path_out[i] = path_out[len - 1 - i];
      path_out[len - 1 - i] = x;
    }
  }
  if (ld_volatile(&ctl->bar_err)) status = OGR_ERR_TIMEOUT;
  const int32_t err_why = ld_volatile(&ctl->err);
  const bool handover = status != OGR_ERR_TIMEOUT && (failed || err_why != 0);
  *gate = handover ? 1 : 0;
  res[0] = handover ? OGR_ERR_ITER_CAP : status;
  res[1] = (found && status == OGR_OK && !handover) ? len : 0;
  res[2] = rounds;
  ctl->stamp = (int32_t)stamp;
  ctl->round_base = gr + 1;
  atomicAdd(&ogr_tile::g_tile_prof[0], 1ull);
  atomicAdd(&ogr_tile::g_tile_prof[1], (unsigned long long)rounds);
  atomicAdd(&ogr_tile::g_tile_prof[2], (unsigned long long)windows);
  atomicAdd(&ogr_tile::g_tile_prof[3], gtimer() - t_start);
  if (handover) {
    atomicAdd(&ogr_tile::g_tile_prof[4], 1ull);
    atomicOr(&ogr_tile::g_tile_prof[5], 1ull << (err_why ? err_why : why));
  }
}

constexpr int kMaxDevices = 64;
std::atomic<int> g_tile_grid[kMaxDevices] = {};       // device properties, set once
std::atomic<size_t> g_tile_smem[kMaxDevices] = {};

Geo make_geo(const ogr_graph& g) {
  Geo G{};
  G.nx = g.nx;
  G.ny = g.ny;
  G.nz = g.nz;
  G.plane = (int64_t)g.nx * g.ny;
  // arcs per column (interior columns have slightly more than the mean)
  const double apc = (double)g.num_edges / (double)G.plane * 1.1;
  int side = 1;
  while ((side + 1) * (side + 1) * g.nz <= kMaxNodes && 4 * g.nz * (side + 1) <= kMaxHalo &&
         (side + 1) * (side + 1) * apc <= kMaxArcs)
    ++side;
  G.tx = g_tile_tx > 0 ? g_tile_tx : side;
  G.ty = g_tile_ty > 0 ? g_tile_ty : side;
  G.tx = G.tx < g.nx ? G.tx : g.nx;
  G.ty = G.ty < g.ny ? G.ty : g.ny;
  G.tm = G.tx > G.ty ? G.tx : G.ty;
  G.ntx = (g.nx + G.tx - 1) / G.tx;
  G.nty = (g.ny + G.ty - 1) / G.ty;
  G.ntiles = G.ntx * G.nty;
  G.inv_plane = (float)(1.0 / (double)G.plane);
  return G;
}

}  // namespace

namespace ogr_tile {

bool enabled() { return g_tile_enable != 0; }

size_t workspace_bytes(int32_t num_nodes) { return tws_layout(num_nodes, nullptr, nullptr); }

size_t ctl_bytes() { return sizeof(TCtl); }

int launch(const ogr_graph& g, const ogr_state& st, const ogr_full::Job& job, void* tws, int32_t* res,
           int32_t* gate, cudaStream_t s) {
  int dev = 0;
  OGR_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return OGR_ERR_ARG;
  const Geo G = make_geo(g);
  if (G.tx * G.ty * G.nz > kMaxNodes || 4 * G.nz * G.tm > kMaxHalo || G.ntiles > kMaxTiles) return OGR_ERR_CAPACITY;
  const size_t smem = ((sizeof(Sm) + 15) & ~(size_t)15) + 4 * (size_t)((G.ntiles + 31) / 32);
  if (g_tile_smem[dev] < smem) {
    int optin = 0;
    OGR_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if ((size_t)optin < smem) return OGR_ERR_CAPACITY;
    OGR_CUDA_TRY(cudaFuncSetAttribute(tile_sssp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0, sms = 0, coop = 0;
    OGR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tile_sssp_kernel, kT, smem));
    OGR_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    OGR_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop || per_sm < 1) return OGR_ERR_CUDA;
    g_tile_grid[dev] = sms * per_sm;
    g_tile_smem[dev] = smem;
  }
  TWs w;
  tws_layout(g.num_nodes, (char*)tws, &w);
  OGR_CUDA_TRY(cudaMemsetAsync(w.ctl, 0, offsetof(TCtl, err), s));
  const double dt = g_tile_delta * 1073741824.0;
  long long delta = dt >= 9.0e15 ? kInf : (long long)dt;
  if (delta < 1) delta = 1;
  ogr_graph gv = g;
  ogr_state sv = st;
  ogr_full::Job jv = job;
  Geo gg = G;
  void* args[] = {&gv, &sv, &jv, &w, &gg, &delta, &res, &gate};
  OGR_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)tile_sssp_kernel, dim3(g_tile_grid[dev].load()), dim3(kT),
                                           args, g_tile_smem[dev].load(), s));
  return OGR_OK;
}

}  // namespace ogr_tile

extern "C" int ogr_full_tile(int32_t enable, double delta, int32_t tx, int32_t ty, int32_t* cur_enable,
                             double* cur_delta) {
  if (enable < -1 || enable > 1 || tx < 0 || ty < 0 || tx > 4096 || ty > 4096) return OGR_ERR_ARG;
  if (enable >= 0) {
    if (enable == 1 && !(delta > 0.0)) return OGR_ERR_ARG;
    g_tile_enable = enable;
    if (enable == 1) {
      g_tile_delta = delta;
      g_tile_tx = tx;
      g_tile_ty = ty;
    }
  }
  if (cur_enable) *cur_enable = g_tile_enable;
  if (cur_delta) *cur_delta = g_tile_delta;
  return OGR_OK;
}

extern "C" int ogr_tile_profile(int64_t* out24, int32_t reset) {
  int64_t* out8 = out24;
  if (!out8) return OGR_ERR_ARG;
  OGR_CUDA_TRY(cudaMemcpyFromSymbol(out8, ogr_tile::g_tile_prof, sizeof(unsigned long long) * 24));
  if (reset) {
    unsigned long long z[24] = {};
    OGR_CUDA_TRY(cudaMemcpyToSymbol(ogr_tile::g_tile_prof, z, sizeof(z)));
  }
  return OGR_OK;
}
