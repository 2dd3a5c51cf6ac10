// A6–A8: per-net ROI extraction, exact ROI shortest path, backtrace, and the
// commit / rip-up scatter.  One CTA (1024 threads) owns one net's search; the
// batched entry points run one CTA per independent net.
//
// ROI (extract_roi_bfs, unified_pathfinder.py:2257-2384): level-synchronous
// bidirectional BFS.  Within one wave step the reference's marks are a set
// function of the frontier (unseen -> wave mark, other wave -> 3 and
// "met"), so claiming nodes with atomicCAS yields the same seen[] array,
// meeting depth and early stop.  The ROI is then compacted in ascending
// global id order (np.where) by scanning the BFS bounding box, and truncated
// to max_roi_nodes with the reference's must-keep swap.
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
#include "common.cuh"

namespace {

constexpr int kThreads = 1024;
constexpr int kWarps = kThreads / 32;
constexpr uint8_t ST_NONE = 0, ST_FRONT = 1, ST_DONE = 2;

struct Ws {
  int32_t* seen;
  int32_t* g2r;
  int32_t* q[4];
  int32_t* roi;
  double* lab;
  float* m32;
  int32_t* par;
  float* pen;
  float* cin;
  int32_t* fr[2];
  int32_t* dl;
  int32_t* dstamp;
  int32_t* blist;
  uint8_t* st;
  int64_t* result;  // [0] status, [1] path len, [2..5] stats
};

__host__ __device__ inline size_t align_up(size_t v) { return (v + 255) & ~(size_t)255; }

__host__ inline size_t ws_layout(int32_t N, char* base, Ws* w) {
  size_t off = 0;
  auto take = [&](size_t bytes) -> char* {
    char* p = base ? base + off : nullptr;
    off = align_up(off + bytes);
    return p;
  };
  const size_t n = (size_t)N;
  Ws t{};
  t.seen = (int32_t*)take(4 * n);
  t.g2r = (int32_t*)take(4 * n);
  for (int i = 0; i < 4; ++i) t.q[i] = (int32_t*)take(4 * n);
  t.roi = (int32_t*)take(4 * n);
  t.lab = (double*)take(8 * n);
  t.m32 = (float*)take(4 * n);
  t.par = (int32_t*)take(4 * n);
  t.pen = (float*)take(4 * n);
  t.cin = (float*)take(4 * n);
  t.fr[0] = (int32_t*)take(4 * n);
  t.fr[1] = (int32_t*)take(4 * n);
  t.dl = (int32_t*)take(4 * n);
  t.dstamp = (int32_t*)take(4 * n);
  t.blist = (int32_t*)take(4 * n);
  t.st = (uint8_t*)take(n);
  t.result = (int64_t*)take(8 * 8);
  if (w) *w = t;
  return off;
}

// ---- block primitives ------------------------------------------------------
__device__ __forceinline__ int block_excl_scan(int v, int* s_warp, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = (lane < kWarps) ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kWarps) s_warp[lane] = w;  // inclusive
    if (lane == kWarps - 1) *total = w;
  }
  __syncthreads();
  const int before = (wid == 0) ? 0 : s_warp[wid - 1];
  const int res = before + x - v;
  __syncthreads();
  return res;
}

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

struct Key {  // lexicographic (float32 alt, L(u), roi idx of u)
  float a32;
  double lu;
  int32_t u;
  double alt;
};

__device__ __forceinline__ bool key_less(float a32, double lu, int32_t u, const Key& k) {
  if (a32 != k.a32) return a32 < k.a32;
  if (lu != k.lu) return lu < k.lu;
  return u < k.u;
}

__device__ __forceinline__ float node_penalty(const ogr_state& st, const ogr_net_args& a, int32_t gid) {
  if (!a.penalty_enabled) return 0.0f;
  const int32_t cnt = st.owner_count[gid];
  const int32_t owner = (cnt == 0) ? -1 : (cnt == 1 ? st.owner_xor[gid] : -2);
  const bool foreign = (owner != -1) && (owner != a.net_id);
  const bool occupied = st.path_node_use[gid] > 0;
  const float f = foreign ? a.owner_weight : 0.0f;
  const float o = occupied ? a.path_weight : 0.0f;
  return __fadd_rn(__fadd_rn(f, o), __fmul_rn(st.node_history[gid], a.history_weight));
}

// ---- the per-net search kernel -----------------------------------------------
struct Shared {
  int s_warp[kWarps];
  unsigned long long s_min[kWarps];
  int total;
  int nq[4];
  int seen_count;
  int met;
  int bx0, bx1, by0, by1;
  int R;
  int nfront, nnext, ndirty, nb;
  int status;
  int found;
};

__device__ void search_one(const ogr_graph& g, const ogr_state& st, const ogr_net_args& a, const Ws& w,
                           int32_t* path_out, int32_t path_cap, bool roi_only, int32_t* roi_out, int32_t roi_cap,
                           int64_t* stats_out) {
  __shared__ Shared sh;
  const int tid = threadIdx.x;
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const int64_t plane = (int64_t)nx * ny;
  const int32_t src = a.src, dst = a.dst;
  const bool full = a.full_graph != 0;
  const int32_t* indptr = g.indptr;
  const int32_t* indices = g.indices;

  if (tid == 0) {
    sh.status = OGR_OK;
    sh.found = 0;
  }
  // ------------------------------------------------------------------ ROI
  if (!full) {
    if (tid == 0) {
      w.seen[src] = 1;
      w.seen[dst] = 2;
      w.q[0][0] = src;
      w.q[2][0] = dst;
      sh.nq[0] = 1;
      sh.nq[2] = 1;
      sh.seen_count = (src != dst) ? 2 : 1;
      const int sy = (int)((src % plane) / nx), sx = (int)((src % plane) % nx);
      const int dy = (int)((dst % plane) / nx), dx = (int)((dst % plane) % nx);
      sh.bx0 = min(sx, dx); sh.bx1 = max(sx, dx);
      sh.by0 = min(sy, dy); sh.by1 = max(sy, dy);
      sh.met = 0;
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
        const int n = sh.nq[cur];
        const int32_t* qc = w.q[cur];
        int32_t* qn = w.q[nxt];
        int local_met = 0, local_new = 0;
        int lx0 = 1 << 30, lx1 = -1, ly0 = 1 << 30, ly1 = -1;
        for (int i = tid; i < n; i += kThreads) {
          const int32_t u = qc[i];
          const int32_t e1 = indptr[u + 1];
          for (int32_t e = indptr[u]; e < e1; ++e) {
            if (g.blocked != nullptr && g.blocked[e]) continue;
            const int32_t v = indices[e];
            const int32_t old = atomicCAS(&w.seen[v], 0, mark);
            if (old == 0) {
              const int pos = atomicAdd(&sh.nq[nxt], 1);
              qn[pos] = v;
              ++local_new;
              const int64_t r = v % plane;
              const int vy = (int)(r / nx), vx = (int)(r % nx);
              lx0 = min(lx0, vx); lx1 = max(lx1, vx);
              ly0 = min(ly0, vy); ly1 = max(ly1, vy);
            } else if (old != mark) {
              w.seen[v] = 3;
              local_met = 1;
            }
          }
        }
        if (local_met) sh.met = 1;
        if (local_new) {
          atomicAdd(&sh.seen_count, local_new);
          atomicMin(&sh.bx0, lx0); atomicMax(&sh.bx1, lx1);
          atomicMin(&sh.by0, ly0); atomicMax(&sh.by1, ly1);
        }
        __syncthreads();
        if (wave == 0) cur_s = nxt; else cur_d = nxt;
      }
      ++depth;
      if (sh.met && meet < 0) meet = depth;
      if (meet >= 0 && depth >= meet + a.bfs_halo) break;
      if ((double)sh.seen_count > a.bfs_stop_count) break;
    }
    __syncthreads();
    // Ordered compaction over the bounding box: ascending global id.
    const int W = sh.bx1 - sh.bx0 + 1, H = sh.by1 - sh.by0 + 1;
    const int64_t area = (int64_t)W * H;
    const int64_t V = area * nz;
    int base = 0;
    for (int64_t start = 0; start < V; start += kThreads) {
      const int64_t i = start + tid;
      int32_t gid = -1;
      int flag = 0;
      if (i < V) {
        const int z = (int)(i / area);
        const int64_t rem = i - (int64_t)z * area;
        const int y = sh.by0 + (int)(rem / W);
        const int x = sh.bx0 + (int)(rem % W);
        gid = (int32_t)(z * plane + (int64_t)y * nx + x);
        flag = w.seen[gid] != 0;
      }
      const int pos = block_excl_scan(flag, sh.s_warp, &sh.total);
      if (flag) w.roi[base + pos] = gid;
      base += sh.total;
      __syncthreads();
    }
    if (tid == 0) {
      int R = base;
      if (R > a.max_roi_nodes) {
        // Must-keep swap (extract_roi_bfs :2359-2379): positions of src/dst in
        // ascending order; each one beyond the cut swaps with slot 0 / 1.
        int kept[2];
        int nk = 0;
        for (int pass = 0; pass < 2; ++pass) {
          const int32_t target = pass == 0 ? min(src, dst) : max(src, dst);
          if (pass == 1 && src == dst) break;
          int lo = 0, hi = R - 1, found = -1;
          while (lo <= hi) {
            const int mid = (lo + hi) >> 1;
            const int32_t vmid = w.roi[mid];
            if (vmid == target) { found = mid; break; }
            if (vmid < target) lo = mid + 1; else hi = mid - 1;
          }
          if (found >= 0) kept[nk++] = found;
        }
        for (int k = 0; k < nk; ++k) {
          if (kept[k] >= a.max_roi_nodes) {
            const int32_t t = w.roi[kept[k]];
            w.roi[kept[k]] = w.roi[k];
            w.roi[k] = t;
          }
        }
        R = a.max_roi_nodes;
      }
      sh.R = R;
    }
    __syncthreads();
    for (int r = tid; r < sh.R; r += kThreads) w.g2r[w.roi[r]] = r;
    __syncthreads();
  } else {
    if (tid == 0) sh.R = g.num_nodes;
    __syncthreads();
  }
  const int R = sh.R;

  if (roi_only) {
    if (tid == 0 && R > roi_cap) sh.status = OGR_ERR_CAPACITY;
    __syncthreads();
    if (sh.status == OGR_OK)
      for (int r = tid; r < R; r += kThreads) roi_out[r] = full ? r : w.roi[r];
    if (tid == 0) w.result[1] = R;
  } else {
    // ---------------------------------------------------------------- SSSP
    const int32_t rs = full ? src : w.g2r[src];
    const int32_t rd = full ? dst : w.g2r[dst];
    for (int r = tid; r < R; r += kThreads) {
      w.st[r] = ST_NONE;
      w.dstamp[r] = -1;
    }
    if (tid == 0) {
      sh.nfront = 0;
      sh.nb = 0;
    }
    __syncthreads();
    bool run = true;
    if (rs < 0 || rd < 0 || rs == rd) {
      if (tid == 0) sh.status = OGR_NO_PATH;
      run = false;
    }
    __syncthreads();
    if (run) {
      if (tid == 0) {
        w.st[rs] = ST_DONE;
        w.lab[rs] = 0.0;
        w.m32[rs] = 0.0f;
        w.par[rs] = -1;
        w.blist[0] = rs;
        sh.nb = 1;
      }
      __syncthreads();
      int cur = 0;
      int phase = 0;
      const int max_phase = R + 2;
      while (true) {
        // 1. dirty = unsettled ROI neighbours of the newly settled set.
        if (tid == 0) sh.ndirty = 0;
        __syncthreads();
        const int nb = sh.nb;
        for (int i = tid; i < nb; i += kThreads) {
          const int32_t x = w.blist[i];
          const int32_t xg = full ? x : w.roi[x];
          for (int32_t e = indptr[xg]; e < indptr[xg + 1]; ++e) {
            const int32_t yg = indices[e];
            const int32_t y = full ? yg : w.g2r[yg];
            if (y < 0 || w.st[y] == ST_DONE) continue;
            if (atomicExch(&w.dstamp[y], phase) != phase) {
              const int p = atomicAdd(&sh.ndirty, 1);
              w.dl[p] = y;
            }
          }
        }
        __syncthreads();
        // 2. recompute each dirty node from all settled in-neighbours.
        const int nd = sh.ndirty;
        for (int i = tid; i < nd; i += kThreads) {
          const int32_t y = w.dl[i];
          const int32_t yg = full ? y : w.roi[y];
          const bool fresh = w.st[y] == ST_NONE;
          float p;
          if (fresh) {
            p = node_penalty(st, a, yg);
            w.pen[y] = p;
          } else {
            p = w.pen[y];
          }
          const double pd = (double)p;
          Key best{__int_as_float(0x7f800000), 0.0, 0x7fffffff, 0.0};
          bool have = false;
          float cin = __int_as_float(0x7f800000);
          for (int32_t e = indptr[yg]; e < indptr[yg + 1]; ++e) {
            const int32_t ug = indices[e];
            const int32_t u = full ? ug : w.g2r[ug];
            if (u < 0) continue;
            const float c = st.total_cost[g.rev[e]];
            if (w.st[u] != ST_DONE) {
              cin = fminf(cin, c);
              continue;
            }
            const double lu = w.lab[u];
            const double alt = (lu + (double)c) + pd;
            const float a32 = __double2float_rn(alt);
            if (!(a32 < __int_as_float(0x7f800000))) continue;
            if (!have || key_less(a32, lu, u, best)) {
              best.a32 = a32; best.lu = lu; best.u = u; best.alt = alt;
              have = true;
            }
          }
          w.cin[y] = cin;
          if (have) {
            w.m32[y] = best.a32;
            w.lab[y] = best.alt;
            w.par[y] = best.u;
            if (fresh) {
              w.st[y] = ST_FRONT;
              const int q = atomicAdd(&sh.nfront, 1);
              w.fr[cur][q] = y;
            }
          }
        }
        __syncthreads();
        const int nf = sh.nfront;
        if (nf == 0) {
          if (tid == 0) sh.status = OGR_NO_PATH;
          break;
        }
        // 3. T = smallest tentative label in the frontier.
        unsigned long long mn = ~0ull;
        for (int i = tid; i < nf; i += kThreads) {
          const unsigned long long b = ogr_dbits(w.lab[w.fr[cur][i]]);
          mn = b < mn ? b : mn;
        }
        mn = block_min_u64(mn, sh.s_min);
        const double T = __longlong_as_double((long long)mn);
        // 4. settle every node whose state can no longer change.
        if (tid == 0) { sh.nb = 0; sh.nnext = 0; }
        __syncthreads();
        for (int i = tid; i < nf; i += kThreads) {
          const int32_t x = w.fr[cur][i];
          const double lx = w.lab[x];
          bool settle = (lx == T);
          if (!settle) {
            const float bound = __double2float_rn((T + (double)w.cin[x]) + (double)w.pen[x]);
            settle = w.m32[x] < bound;
          }
          if (settle) {
            const int p = atomicAdd(&sh.nb, 1);
            w.blist[p] = x;
          } else {
            const int p = atomicAdd(&sh.nnext, 1);
            w.fr[cur ^ 1][p] = x;
          }
        }
        __syncthreads();
        for (int i = tid; i < sh.nb; i += kThreads) w.st[w.blist[i]] = ST_DONE;
        if (tid == 0) sh.nfront = sh.nnext;
        cur ^= 1;
        __syncthreads();
        if (w.st[rd] == ST_DONE) {
          if (tid == 0) sh.found = 1;
          break;
        }
        if (++phase > max_phase) {
          if (tid == 0) sh.status = OGR_ERR_ITER_CAP;
          break;
        }
      }
      __syncthreads();
      // Arcs the sequential search scans before popping dst: the rows of all
      // nodes popped before it, i.e. settled with (L, idx) < (L(dst), dst).
      if (sh.found && stats_out != nullptr) {
        if (tid == 0) { sh.total = 0; sh.nnext = 0; }
        __syncthreads();
        const double ld = w.lab[rd];
        int arcs = 0, pops = 0;
        for (int r = tid; r < R; r += kThreads) {
          if (w.st[r] != ST_DONE) continue;
          const double lr = w.lab[r];
          if (lr < ld || (lr == ld && r < rd)) {
            const int32_t rg = full ? r : w.roi[r];
            arcs += indptr[rg + 1] - indptr[rg];
            ++pops;
          }
        }
        atomicAdd(&sh.total, arcs);
        atomicAdd(&sh.nnext, pops);
        __syncthreads();
        if (tid == 0) {
          stats_out[0] = sh.total;
          stats_out[1] = sh.nnext + 1;
          stats_out[2] = R;
          stats_out[3] = phase + 1;
        }
      }
      // Backtrace dst -> src.
      if (tid == 0 && sh.found && sh.status == OGR_OK) {
        int len = 0;
        for (int32_t c = rd; c != -1 && len <= R; c = w.par[c]) ++len;
        if (len > R) {
          sh.status = OGR_ERR_ITER_CAP;  // parent chain longer than the ROI: a cycle
        } else if (len > path_cap) {
          sh.status = OGR_ERR_CAPACITY;
        } else {
          int i = len - 1;
          for (int32_t c = rd; c != -1; c = w.par[c]) path_out[i--] = full ? c : w.roi[c];
          w.result[1] = len;
          if (len < 2) sh.status = OGR_NO_PATH;
        }
      }
    }
  }
  __syncthreads();
  // ---------------------------------------------------------------- cleanup
  if (!full) {
    for (int r = tid; r < R; r += kThreads) w.g2r[w.roi[r]] = -1;
    const int W = sh.bx1 - sh.bx0 + 1, H = sh.by1 - sh.by0 + 1;
    const int64_t area = (int64_t)W * H;
    const int64_t V = area * nz;
    for (int64_t i = tid; i < V; i += kThreads) {
      const int z = (int)(i / area);
      const int64_t rem = i - (int64_t)z * area;
      const int y = sh.by0 + (int)(rem / W);
      const int x = sh.bx0 + (int)(rem % W);
      w.seen[z * plane + (int64_t)y * nx + x] = 0;
    }
  }
  if (tid == 0) w.result[0] = sh.status;
}

__global__ void __launch_bounds__(kThreads, 1)
find_path_kernel(ogr_graph g, ogr_state st, ogr_net_args a, Ws w, int32_t* path_out, int32_t path_cap,
                 int64_t* stats) {
  search_one(g, st, a, w, path_out, path_cap, false, nullptr, 0, stats);
}

__global__ void __launch_bounds__(kThreads, 1)
roi_kernel(ogr_graph g, ogr_net_args a, Ws w, int32_t* roi_out, int32_t roi_cap) {
  ogr_state st{};
  search_one(g, st, a, w, nullptr, 0, true, roi_out, roi_cap, nullptr);
}

__global__ void ws_init_kernel(Ws w, int64_t N) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    w.seen[i] = 0;
    w.g2r[i] = -1;
  }
}

// ---- commit / rip-up ---------------------------------------------------------
constexpr int kApplyThreads = 256;
constexpr int kMaxViaNodes = 4096;

__global__ void __launch_bounds__(kApplyThreads)
path_apply_kernel(ogr_graph g, ogr_state st, const int32_t* path, int32_t len, int32_t net_id, int32_t sign,
                  float pres_fac, int32_t live, int32_t* arcs_out, int32_t* status) {
  __shared__ int32_t s_via[kMaxViaNodes];
  __shared__ int s_nvia;
  __shared__ int s_bad;
  const int tid = threadIdx.x;
  if (tid == 0) { s_nvia = 0; s_bad = 0; }
  __syncthreads();
  const int hops = len - 1;
  const int64_t plane = (int64_t)g.nx * g.ny;
  // Arcs: forward hop i is path[i]->path[i+1]; the reversed path's hop j is
  // the opposite arc of forward hop hops-1-j (_path_to_edges order).
  for (int i = tid; i < hops; i += kApplyThreads) {
    const int32_t u = path[i], v = path[i + 1];
    int32_t f = -1;
    for (int32_t e = g.indptr[u]; e < g.indptr[u + 1]; ++e)
      if (g.indices[e] == v) { f = e; break; }
    if (f < 0) { s_bad = 1; continue; }
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
        st.total_cost[e] = __fadd_rn(st.live_static[e], __fmul_rn(scale, prosp));
      }
    }
  }
  // Path-node use (a simple path visits each node once).
  for (int i = tid; i < len; i += kApplyThreads) {
    const int32_t n = path[i];
    const int32_t u = st.path_node_use[n];
    st.path_node_use[n] = sign > 0 ? u + 1 : max(u - 1, 0);
  }
  __syncthreads();
  // Barrel ownership: union of the z-ranges of all via hops (deduplicated).
  if (tid == 0) {
    int nv = 0;
    for (int i = 0; i < hops && !s_bad; ++i) {
      const int32_t u = path[i], v = path[i + 1];
      const int64_t ru = u % plane, rv = v % plane;
      const int zu = (int)(u / plane), zv = (int)(v / plane);
      if (ru != rv || zu == zv) continue;
      for (int z = min(zu, zv); z <= max(zu, zv); ++z) {
        const int32_t node = (int32_t)(z * plane + ru);
        bool dup = false;
        for (int k = 0; k < nv; ++k)
          if (s_via[k] == node) { dup = true; break; }
        if (dup) continue;
        if (nv >= kMaxViaNodes) { s_bad = 2; break; }
        s_via[nv++] = node;
      }
    }
    s_nvia = nv;
  }
  __syncthreads();
  for (int k = tid; k < s_nvia; k += kApplyThreads) {
    const int32_t node = s_via[k];
    st.owner_count[node] += sign > 0 ? 1 : -1;
    st.owner_xor[node] ^= net_id;
  }
  if (tid == 0) *status = s_bad ? (s_bad == 1 ? OGR_ERR_ARG : OGR_ERR_CAPACITY) : OGR_OK;
}

}  // namespace

extern "C" size_t ogr_route_workspace_bytes(int32_t num_nodes) { return ws_layout(num_nodes, nullptr, nullptr); }

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
  find_path_kernel<<<1, kThreads, 0, s>>>(*g, *st, *net, w, path_out, path_cap, stats);
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

extern "C" int ogr_path_apply(const ogr_graph* g, const ogr_state* st, const int32_t* path, int32_t len,
                              int32_t net_id, int32_t sign, float pres_fac_f32, int32_t live, int32_t* arcs_out,
                              int32_t* status_dev, void* stream) {
  if (!g || !st || !path || !status_dev || len < 2 || (sign != 1 && sign != -1)) return OGR_ERR_ARG;
  path_apply_kernel<<<1, kApplyThreads, 0, ogr_stream(stream)>>>(*g, *st, path, len, net_id, sign, pres_fac_f32,
                                                                   live, arcs_out, status_dev);
  OGR_LAUNCH_CHECK();
  return OGR_OK;
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

constexpr size_t noalloc_round(size_t v) { return (v + 255) & ~(size_t)255; }

constexpr size_t noalloc_ws_bytes() {
  // The layout of ws_layout() for OGR_NOALLOC_MAX_NODES nodes: 16 int32 /
  // float arrays, one double array, one byte array, the 64-byte result block,
  // each rounded up to 256 bytes (about 19 MB).
  return 16 * noalloc_round((size_t)OGR_NOALLOC_MAX_NODES * 4) + noalloc_round((size_t)OGR_NOALLOC_MAX_NODES * 8) +
         noalloc_round((size_t)OGR_NOALLOC_MAX_NODES) + noalloc_round(64);
}

static __device__ __align__(256) unsigned char g_noalloc_ws[noalloc_ws_bytes()];

constexpr int kMaxDevices = 64;
void* g_noalloc_ptr[kMaxDevices] = {};

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
  if (g_noalloc_ptr[dev] == nullptr) {
    void* p = nullptr;
    OGR_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_ws));
    g_noalloc_ptr[dev] = p;
  }
  const size_t need = ws_layout(g->num_nodes, nullptr, nullptr);
  if (need > noalloc_ws_bytes()) return OGR_ERR_CAPACITY;
  Ws w;
  ws_layout(g->num_nodes, (char*)g_noalloc_ptr[dev], &w);
  cudaStream_t s = ogr_stream(stream);
  // The array keeps whatever the previous call left: clear seen[] / g2r[].
  ws_init_kernel<<<ogr_blocks(g->num_nodes, 256), 256, 0, s>>>(w, g->num_nodes);
  find_path_kernel<<<1, kThreads, 0, s>>>(*g, *st, *net, w, path_out, path_cap, stats);
  OGR_LAUNCH_CHECK();
  int64_t res[2];
  OGR_CUDA_TRY(cudaMemcpyAsync(res, w.result, sizeof(res), cudaMemcpyDeviceToHost, s));
  OGR_CUDA_TRY(cudaStreamSynchronize(s));
  *path_len_out = (res[0] == OGR_OK) ? (int32_t)res[1] : 0;
  return (int)res[0];
}
