// A2–A4: per-arc cost update, live-present rebase, present EMA, history;
// A9: overuse / node-use / per-layer tallies.
//
// All arithmetic is float32 with one rounding per operation in the order
// numpy evaluates the reference's expressions (explicit __f*_rn intrinsics,
// so no FMA contraction can merge two roundings).  These kernels stream
// 6–8 arrays of E entries once: HBM-bound, grid-stride over 152 SMs.
#include "common.cuh"

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float arc_bias(const float* layer_bias, unsigned char layer, unsigned char kind) {
  return (layer_bias != nullptr && kind == 0) ? layer_bias[layer] : 1.0f;
}

// float32(e) % 9973 * float32(1e-6): numpy's arange(E, float32) rounds e to
// nearest even like __int2float_rn; fmodf is exact.
__device__ __forceinline__ float jitter(int64_t e) {
  const float fe = __ll2float_rn((long long)e);
  return __fmul_rn(fmodf(fe, 9973.0f), 1e-6f);
}

__global__ void cost_kernel(ogr_cost_args a, float* __restrict__ total) {
  const bool have_bias = a.layer_bias != nullptr;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < a.num_edges;
       e += (int64_t)gridDim.x * blockDim.x) {
    const unsigned char lay = a.edge_layer[e], kind = a.edge_kind[e];
    const float over = fmaxf(0.0f, __fsub_rn(a.present_ema[e], a.capacity[e]));
    const float bias = arc_bias(a.layer_bias, lay, kind);
    // adjusted = ((base * vmult) * bw) * bias
    float adj = __fmul_rn(__fmul_rn(a.base_costs[e], a.via_cost_multiplier), a.base_cost_weight);
    if (have_bias) adj = __fmul_rn(adj, bias);
    // present = (pres_fac * bias) * over
    const float scale = have_bias ? __fmul_rn(a.pres_fac, bias) : a.pres_fac;
    const float pres = __fmul_rn(scale, over);
    float t = __fadd_rn(__fadd_rn(adj, pres), __fmul_rn(a.hist_weight, a.history[e]));
    if (a.blocked != nullptr && a.blocked[e]) t = __int_as_float(0x7f800000);
    if (a.add_jitter) t = __fadd_rn(t, jitter(e));
    total[e] = t;
  }
}

__global__ void live_kernel(ogr_cost_args a, const float* __restrict__ present, float* __restrict__ total,
                            float* __restrict__ live_static) {
  const bool have_bias = a.layer_bias != nullptr;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < a.num_edges;
       e += (int64_t)gridDim.x * blockDim.x) {
    const float bias = arc_bias(a.layer_bias, a.edge_layer[e], a.edge_kind[e]);
    const float scale = have_bias ? __fmul_rn(a.pres_fac, bias) : a.pres_fac;
    const float cap = a.capacity[e];
    const float it_over = fmaxf(0.0f, __fsub_rn(a.present_ema[e], cap));
    const float st = __fsub_rn(total[e], __fmul_rn(scale, it_over));
    const float prosp = fmaxf(0.0f, __fsub_rn(__fadd_rn(present[e], 1.0f), cap));
    live_static[e] = st;
    total[e] = __fadd_rn(st, __fmul_rn(scale, prosp));
  }
}

__global__ void ema_kernel(int64_t E, const float* __restrict__ present, float* __restrict__ ema, float beta,
                           float omb) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x)
    ema[e] = __fadd_rn(__fmul_rn(beta, present[e]), __fmul_rn(omb, ema[e]));
}

__global__ void history_kernel(int64_t E, float* __restrict__ hist, const float* __restrict__ src,
                               const float* __restrict__ cap, const float* __restrict__ base, float gain,
                               float cap_mult, float decay) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    float h = __fmul_rn(hist[e], decay);
    const float over = fmaxf(0.0f, __fsub_rn(src[e], cap[e]));
    float inc = __fmul_rn(gain, over);
    if (base != nullptr) inc = fminf(inc, __fmul_rn(cap_mult, base[e]));
    hist[e] = __fadd_rn(h, inc);
  }
}

// Exact integer tallies.  Per-layer EMA overuse is accumulated in units of
// 2^-23 (every max(0, ema-1) with ema >= 1 is a multiple of 2^-23, so the
// sum is exact and order independent, like numpy's float64 bincount).
constexpr int kMaxLayers = 64;

__global__ void tally_kernel(int64_t E, int32_t N, int32_t nz, const float* __restrict__ present,
                             const float* __restrict__ ema, const float* __restrict__ cap,
                             const int32_t* __restrict__ edge_src, const int32_t* __restrict__ indices,
                             const unsigned char* __restrict__ edge_layer, const int32_t* __restrict__ use,
                             int canonical_only, unsigned long long* out, unsigned long long* layer_units) {
  __shared__ unsigned long long s_layer[kMaxLayers];
  __shared__ unsigned long long s_out[5];
  for (int i = threadIdx.x; i < nz; i += blockDim.x) s_layer[i] = 0;
  if (threadIdx.x < 5) s_out[threadIdx.x] = 0;
  __syncthreads();
  unsigned long long over_sum = 0, over_cnt = 0, bad = 0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    const float c = cap[e];
    if (!canonical_only || edge_src[e] < indices[e]) {
      const float o = fmaxf(0.0f, __fsub_rn(present[e], c));
      if (o > 0.0f) {
        over_sum += (unsigned long long)o;
        over_cnt += 1;
      }
    }
    const float eo = fmaxf(0.0f, __fsub_rn(ema[e], c));
    if (eo > 0.0f) {
      const double units = (double)eo * 8388608.0;  // 2^23
      const unsigned long long u = (unsigned long long)units;
      if ((double)u != units) bad = 1;
      atomicAdd(&s_layer[edge_layer[e]], u);
    }
  }
  const int64_t plane = (int64_t)N / nz;
  unsigned long long nsum = 0, ncnt = 0;
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    const int32_t u = use[n];
    if (u > 1) {
      nsum += (unsigned long long)(u - 1);
      ncnt += 1;
      atomicAdd(&s_layer[(int)(n / plane)], (unsigned long long)(u - 1) << 23);
    }
  }
  atomicAdd(&s_out[0], over_sum);
  atomicAdd(&s_out[1], over_cnt);
  atomicAdd(&s_out[2], nsum);
  atomicAdd(&s_out[3], ncnt);
  if (bad) atomicOr(&s_out[4], 1ull);
  __syncthreads();
  if (threadIdx.x < 5) atomicAdd(&out[threadIdx.x], s_out[threadIdx.x]);
  for (int i = threadIdx.x; i < nz; i += blockDim.x) atomicAdd(&layer_units[i], s_layer[i]);
}

}  // namespace

__global__ void reverse_cost_kernel(int64_t E, const int32_t* __restrict__ rev, const float* __restrict__ total,
                                    float* __restrict__ rcost) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += stride) rcost[e] = total[rev[e]];
}

extern "C" int ogr_reverse_costs(int64_t E, const int32_t* rev, const float* total_cost, float* rcost,
                                 void* stream) {
  if (E < 0 || (E > 0 && (!rev || !total_cost || !rcost))) return OGR_ERR_ARG;
  if (E == 0) return OGR_OK;
  reverse_cost_kernel<<<ogr_blocks(E, 256), 256, 0, ogr_stream(stream)>>>(E, rev, total_cost, rcost);
  OGR_LAUNCH_CHECK();
  return OGR_OK;
}

extern "C" int ogr_costs_update(const ogr_cost_args* a, float* total_cost, void* stream) {
  if (!a || !total_cost || a->num_edges < 0) return OGR_ERR_ARG;
  cost_kernel<<<ogr_blocks(a->num_edges, kThreads, 152 * 32), kThreads, 0, ogr_stream(stream)>>>(*a, total_cost);
  OGR_LAUNCH_CHECK();
  return OGR_OK;
}

extern "C" int ogr_live_begin(const ogr_cost_args* a, const float* present, float* total_cost, float* live_static,
                              void* stream) {
  if (!a || !present || !total_cost || !live_static) return OGR_ERR_ARG;
  live_kernel<<<ogr_blocks(a->num_edges, kThreads, 152 * 32), kThreads, 0, ogr_stream(stream)>>>(
      *a, present, total_cost, live_static);
  OGR_LAUNCH_CHECK();
  return OGR_OK;
}

extern "C" int ogr_present_ema(int64_t E, const float* present, float* ema, float beta, float omb, void* stream) {
  if (!present || !ema) return OGR_ERR_ARG;
  ema_kernel<<<ogr_blocks(E, kThreads, 152 * 32), kThreads, 0, ogr_stream(stream)>>>(E, present, ema, beta, omb);
  OGR_LAUNCH_CHECK();
  return OGR_OK;
}

extern "C" int ogr_history_update(int64_t E, float* history, const float* present, const float* present_ema,
                                  const float* capacity, const float* base_costs, float gain, float cap_mult,
                                  float decay, int32_t use_raw_present, void* stream) {
  if (!history || !present || !present_ema || !capacity) return OGR_ERR_ARG;
  history_kernel<<<ogr_blocks(E, kThreads, 152 * 32), kThreads, 0, ogr_stream(stream)>>>(
      E, history, use_raw_present ? present : present_ema, capacity, base_costs, gain, cap_mult, decay);
  OGR_LAUNCH_CHECK();
  return OGR_OK;
}

extern "C" int ogr_tally(int64_t E, int32_t N, int32_t nz, const float* present, const float* present_ema,
                         const float* capacity, const int32_t* edge_src, const int32_t* indices,
                         const uint8_t* edge_layer, const int32_t* path_node_use, int32_t canonical_only,
                         int64_t* out, int64_t* layer_units, void* stream) {
  if (nz < 1 || nz > kMaxLayers || N % nz != 0) return OGR_ERR_ARG;
  cudaStream_t s = ogr_stream(stream);
  OGR_CUDA_TRY(cudaMemsetAsync(out, 0, 5 * sizeof(int64_t), s));
  OGR_CUDA_TRY(cudaMemsetAsync(layer_units, 0, nz * sizeof(int64_t), s));
  tally_kernel<<<ogr_blocks(E, kThreads, 152 * 8), kThreads, 0, s>>>(
      E, N, nz, present, present_ema, capacity, edge_src, indices, edge_layer, path_node_use, canonical_only,
      reinterpret_cast<unsigned long long*>(out), reinterpret_cast<unsigned long long*>(layer_units));
  OGR_LAUNCH_CHECK();
  return OGR_OK;
}

// ---------------------------------------------------------------- A5 ---------
// Via pool penalties (_apply_via_pooling_penalties CPU branch,
// unified_pathfinder.py:5884-5980) and the hard block of saturated via
// resources (_block_via_edges_with_collisions, :6094-6161), one thread per
// via arc.  Pools are [Nx][Ny] / [Nx][Ny][segZ] (x-major, like the reference).
// disc[z_lo*nz + z_hi] is the leave-hot-layer discount computed on the host
// with the reference's dtypes; the penalty is rounded to float32 after the
// product, which equals numpy's float32 multiply when the discount is float32.
namespace {

__global__ void via_pool_kernel(int64_t E, int32_t nx, int32_t ny, int32_t nz, const int32_t* __restrict__ edge_src,
                                const int32_t* __restrict__ indices, const uint8_t* __restrict__ kind,
                                const float* __restrict__ col_pres, const float* __restrict__ seg_prefix,
                                const int16_t* __restrict__ col_use, const int16_t* __restrict__ col_cap,
                                const int16_t* __restrict__ seg_use, const int8_t* __restrict__ seg_cap,
                                const double* __restrict__ disc, float col_w, float seg_w, float pres_fac,
                                int32_t apply_penalty, int32_t apply_block, float* __restrict__ total) {
  const int64_t plane = (int64_t)nx * ny;
  const int segZ = nz > 2 ? nz - 2 : 0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    if (!kind[e]) continue;
    const int32_t u = edge_src[e], v = indices[e];
    const int zu = (int)(u / plane), zv = (int)(v / plane);
    const int64_t r = u % plane;
    const int y = (int)(r / nx), x = (int)(r % nx);
    int zl = min(zu, zv), zh = max(zu, zv);
    zl = min(max(zl, 1), nz - 2);
    zh = min(max(zh, 1), nz - 2);
    const int64_t cxy = (int64_t)x * ny + y;
    if (apply_penalty) {
      float pen = 0.0f;
      pen = __fadd_rn(pen, __fmul_rn(col_w, col_pres[cxy]));
      if (segZ > 0) {
        const int hi = zh - 2, lo = zl - 2;
        const float ph = (hi >= 0 && hi < segZ) ? seg_prefix[cxy * segZ + hi] : 0.0f;
        const float pl = (lo >= 0 && lo < segZ) ? seg_prefix[cxy * segZ + lo] : 0.0f;
        const float sp = (zh > zl) ? __fsub_rn(ph, pl) : __fmul_rn(__fsub_rn(ph, pl), 0.0f);
        pen = __fadd_rn(pen, __fmul_rn(seg_w, sp));
      }
      if (disc != nullptr) pen = __double2float_rn((double)pen * disc[zl * nz + zh]);
      if (pen > 0.0f) total[e] = __fadd_rn(total[e], __fmul_rn(pres_fac, pen));
    }
    if (apply_block) {
      bool blocked = col_use[cxy] >= col_cap[cxy];
      if (segZ > 0) {
        for (int z = zl; z < zh && !blocked; ++z) {
          const int s = z - 1;
          if (s >= 0 && s < segZ && seg_use[cxy * segZ + s] >= seg_cap[cxy * segZ + s]) blocked = true;
        }
      }
      if (blocked) total[e] = __int_as_float(0x7f800000);
    }
  }
}

__global__ void overused_kernel(int64_t E, const float* __restrict__ present, const float* __restrict__ cap,
                                int32_t* __restrict__ out_idx, float* __restrict__ out_val, int32_t out_cap,
                                unsigned int* __restrict__ count) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    const float o = fmaxf(0.0f, __fsub_rn(present[e], cap[e]));
    if (o > 0.0f) {
      const unsigned int p = atomicAdd(count, 1u);
      if ((int32_t)p < out_cap) {
        out_idx[p] = (int32_t)e;
        out_val[p] = o;
      }
    }
  }
}

// Per net of a path store: the sum of max(0, present - capacity) over the
// arcs of its stored path (both directions of every hop) and whether any of
// them is overused; canonical_only counts only arcs with src < dst.  One warp
// per net.  The values are whole numbers held exactly in float32, so the
// double sum is exact in any order.
__global__ void nets_overuse_kernel(const int32_t* store_len, const int32_t* store_arcs, int32_t num_nets,
                                    int64_t arc_stride, const float* present, const float* cap,
                                    const int32_t* edge_src, const int32_t* indices, int32_t canonical_only,
                                    double* sums, uint8_t* hit) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t n = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; n < num_nets; n += warps) {
    const int32_t len = store_len[n];
    const int32_t na = len >= 2 ? 2 * (len - 1) : 0;
    const int32_t* arcs = store_arcs + n * arc_stride;
    double sum = 0.0;
    bool any = false;
    for (int32_t j = lane; j < na; j += 32) {
      const int32_t e = arcs[j];
      if (canonical_only && !(edge_src[e] < indices[e])) continue;
      const float o = __fsub_rn(present[e], cap[e]);
      if (o > 0.0f) {
        sum += (double)o;
        any = true;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    any = __any_sync(0xffffffffu, any);
    if (lane == 0) {
      sums[n] = sum;
      hit[n] = any ? 1 : 0;
    }
  }
}

// Via pool use of the stored paths (_rebuild_via_usage_from_committed,
// unified_pathfinder.py:4548-4615, per path _accumulate_via_usage_for_path
// :4470-4546): one thread walks one net's path; every maximal run of via hops
// in one column adds 1 to that column, and every segment z - 1 of the run's
// clamped z hull [lo, hi) (z in [1, nz-2]) adds 1 to that segment.  Counts go
// to int32 scratch ([nx][ny], [nx][ny][segZ], x-major).
__global__ void via_use_kernel(const int32_t* __restrict__ store_len, const int32_t* __restrict__ store_path,
                               int32_t num_nets, int64_t slot_cap, int32_t nx, int32_t ny, int32_t nz,
                               int32_t* col, int32_t* seg) {
  const int64_t plane = (int64_t)nx * ny;
  const int segZ = nz > 2 ? nz - 2 : 0;
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < num_nets;
       n += (int64_t)gridDim.x * blockDim.x) {
    const int32_t len = store_len[n];
    const int32_t* p = store_path + n * slot_cap;
    int64_t run_xy = -1;
    int lo = 0, hi = 0;
    auto close_run = [&]() {
      if (run_xy >= 0 && segZ > 0)
        for (int z = lo; z < hi; ++z) {
          const int sidx = z - 1;
          if (sidx >= 0 && sidx < segZ) atomicAdd(&seg[run_xy * segZ + sidx], 1);
        }
      run_xy = -1;
    };
    int32_t u = len > 0 ? p[0] : 0;
    for (int32_t k = 1; k < len; ++k) {
      const int32_t v = p[k];
      const int64_t ru = u % plane, rv = v % plane;
      const int zu = (int)(u / plane), zv = (int)(v / plane);
      if (ru == rv && zu != zv) {
        const int64_t xy = (ru % nx) * ny + ru / nx;
        int zl = min(zu, zv), zh = max(zu, zv);
        zl = min(max(zl, 1), nz - 2);
        zh = min(max(zh, 1), nz - 2);
        if (xy != run_xy) {
          close_run();
          atomicAdd(&col[xy], 1);
          run_xy = xy;
          lo = zl;
          hi = zh;
        } else {
          lo = min(lo, zl);
          hi = max(hi, zh);
        }
      } else {
        close_run();
      }
      u = v;
    }
    close_run();
  }
}

// Per column: the int16 use arrays the penalty / block kernel reads, the
// spatial overuse sum (Σ max(0, use - cap) over columns and segments) and the
// list of over-full pools as {kind (0 column, 1 segment), x, y, s, use}.
__global__ void via_use_finish_kernel(int32_t nx, int32_t ny, int32_t nz, const int32_t* col, const int32_t* seg,
                                      int16_t* col_use, int16_t* seg_use, const int16_t* col_cap,
                                      const int8_t* seg_cap, unsigned long long* spatial, int32_t* over,
                                      int32_t over_cap, int32_t* over_count) {
  const int64_t plane = (int64_t)nx * ny;
  const int segZ = nz > 2 ? nz - 2 : 0;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < plane; c += (int64_t)gridDim.x * blockDim.x) {
    unsigned long long o = 0;
    const int32_t cu = col[c];
    col_use[c] = (int16_t)min(cu, 32767);
    if (cu > col_cap[c]) {
      o += (unsigned long long)(cu - col_cap[c]);
      const int k = atomicAdd(over_count, 1);
      if (k < over_cap) {
        int32_t* e = over + 5 * (int64_t)k;
        e[0] = 0; e[1] = (int32_t)(c / ny); e[2] = (int32_t)(c % ny); e[3] = 0; e[4] = cu;
      }
    }
    for (int sidx = 0; sidx < segZ; ++sidx) {
      const int32_t su = seg[c * segZ + sidx];
      seg_use[c * segZ + sidx] = (int16_t)min(su, 32767);
      if (su > seg_cap[c * segZ + sidx]) {
        o += (unsigned long long)(su - seg_cap[c * segZ + sidx]);
        const int k = atomicAdd(over_count, 1);
        if (k < over_cap) {
          int32_t* e = over + 5 * (int64_t)k;
          e[0] = 1; e[1] = (int32_t)(c / ny); e[2] = (int32_t)(c % ny); e[3] = sidx; e[4] = su;
        }
      }
    }
    if (o) atomicAdd(spatial, o);
  }
}

// The via-present EMA and z prefix (:6279-6303): pres = 0.6 * over + 0.4 *
// prev in float32 (numpy's weak-scalar order), prefix = float32 cumulative
// sum over the column's segments.
__global__ void via_presence_kernel(int32_t nx, int32_t ny, int32_t nz, const int16_t* col_use,
                                    const int16_t* col_cap, const int16_t* seg_use, const int8_t* seg_cap,
                                    float* col_pres, float* seg_pres, float* seg_prefix) {
  const int64_t plane = (int64_t)nx * ny;
  const int segZ = nz > 2 ? nz - 2 : 0;
  const float a = 0.6f, b = 0.4f;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < plane; c += (int64_t)gridDim.x * blockDim.x) {
    const float oc = (float)max(0, (int)col_use[c] - (int)col_cap[c]);
    col_pres[c] = __fadd_rn(__fmul_rn(a, oc), __fmul_rn(b, col_pres[c]));
    float acc = 0.0f;
    for (int sidx = 0; sidx < segZ; ++sidx) {
      const int64_t i = c * segZ + sidx;
      const float os = (float)max(0, (int)seg_use[i] - (int)seg_cap[i]);
      const float v = __fadd_rn(__fmul_rn(a, os), __fmul_rn(b, seg_pres[i]));
      seg_pres[i] = v;
      acc = sidx == 0 ? v : __fadd_rn(acc, v);
      seg_prefix[i] = acc;
    }
  }
}

// Barrel owner of a node from the device ownership (count of distinct nets
// whose via hops span it, XOR of their ids): -1 none, the id, -2 several.
__device__ __forceinline__ int32_t barrel_owner(const int32_t* cnt, const int32_t* xr, int32_t n) {
  const int32_t c = cnt[n];
  return c == 0 ? -1 : (c == 1 ? xr[n] : -2);
}

// Reserve one slot of list k (counts[k]) and return it, or -1 past the cap
// (the count still grows, so the host learns the size it needs).
__device__ __forceinline__ long long list_slot(unsigned long long* counts, int k, long long cap) {
  const long long i = (long long)atomicAdd(&counts[k], 1ull);
  return i < cap ? i : -1;
}

// Exact barrel conflicts and shared path nodes of the stored paths
// (_detect_barrel_conflicts, unified_pathfinder.py:10778-11111;
// _detect_path_node_conflicts :10564-10606).  One warp per net, lanes over
// the path: hop (u, v) of net id en conflicts at an endpoint whose barrel
// owner is neither -1 nor en.  counts: {conflicting hops, endpoint
// occurrences, distinct conflict nodes, multi-owner members, shared-node
// occurrences}.
__global__ void barrel_hops_kernel(const int32_t* __restrict__ store_len, const int32_t* __restrict__ store_path,
                                   const int32_t* __restrict__ net_id, int32_t num_nets, int64_t slot_cap,
                                   const int32_t* __restrict__ owner_count, const int32_t* __restrict__ owner_xor,
                                   const int32_t* __restrict__ use, int32_t* mark, int32_t stamp, long long cap,
                                   int32_t* occ, int32_t* cnode, int32_t* shared, unsigned long long* counts) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t n = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; n < num_nets; n += warps) {
    const int32_t len = store_len[n];
    if (len < 2) continue;
    const int32_t* p = store_path + n * slot_cap;
    const int32_t en = net_id[n];
    unsigned hops = 0;
    for (int32_t j = lane; j < len; j += 32) {
      const int32_t u = p[j];
      if (use[u] > 1) {
        const long long i = list_slot(counts, 4, cap);
        if (i >= 0) { shared[2 * i] = u; shared[2 * i + 1] = (int32_t)n; }
      }
      if (j + 1 >= len) continue;
      const int32_t v = p[j + 1];
      const int32_t ou = barrel_owner(owner_count, owner_xor, u);
      const int32_t ov = barrel_owner(owner_count, owner_xor, v);
      const bool sc = ou != -1 && ou != en;
      const bool dc = ov != -1 && ov != en;
      if (!(sc || dc)) continue;
      ++hops;
      for (int k = 0; k < 2; ++k) {
        if (!(k == 0 ? sc : dc)) continue;
        const int32_t x = k == 0 ? u : v;
        const long long i = list_slot(counts, 1, cap);
        if (i >= 0) { occ[2 * i] = x; occ[2 * i + 1] = en; }
        if (atomicExch(&mark[x], stamp) != stamp) {
          const long long c = list_slot(counts, 2, cap);
          if (c >= 0) { cnode[3 * c] = x; cnode[3 * c + 1] = owner_count[x]; cnode[3 * c + 2] = owner_xor[x]; }
        }
      }
    }
    hops = __reduce_add_sync(0xffffffffu, hops);
    if (lane == 0 && hops) atomicAdd(&counts[0], (unsigned long long)hops);
  }
}

// The nets behind each conflict node that several nets own: every via hop
// (same column, different layers) spans the nodes of its z range; a spanned
// node marked in this call whose owner count is 2 or more gets (node, id).
// A net may list a node twice (two hops over it); the set is what counts.
__global__ void barrel_members_kernel(const int32_t* __restrict__ store_len, const int32_t* __restrict__ store_path,
                                      const int32_t* __restrict__ net_id, int32_t num_nets, int64_t slot_cap,
                                      int32_t plane, const int32_t* __restrict__ owner_count,
                                      const int32_t* __restrict__ mark, int32_t stamp, long long cap, int32_t* member,
                                      unsigned long long* counts) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t n = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; n < num_nets; n += warps) {
    const int32_t len = store_len[n];
    if (len < 2) continue;
    const int32_t* p = store_path + n * slot_cap;
    const int32_t en = net_id[n];
    for (int32_t j = lane; j + 1 < len; j += 32) {
      const int32_t u = p[j], v = p[j + 1];
      const int32_t ru = u % plane, rv = v % plane;
      const int zu = u / plane, zv = v / plane;
      if (ru != rv || zu == zv) continue;
      for (int z = min(zu, zv); z <= max(zu, zv); ++z) {
        const int32_t nd = z * plane + ru;
        if (mark[nd] != stamp || owner_count[nd] < 2) continue;
        const long long i = list_slot(counts, 3, cap);
        if (i >= 0) { member[2 * i] = nd; member[2 * i + 1] = en; }
      }
    }
  }
}

}  // namespace

extern "C" int ogr_via_pools_rebuild(const int32_t* store_len, const int32_t* store_path, int32_t num_nets,
                                     int64_t slot_cap, int32_t nx, int32_t ny, int32_t nz, int32_t* scratch,
                                     int16_t* col_use, int16_t* seg_use, const int16_t* col_cap,
                                     const int8_t* seg_cap, int64_t* spatial, int32_t* over, int32_t over_cap,
                                     int32_t* over_count, void* stream) {
  if (nx < 1 || ny < 1 || nz < 1 || num_nets < 0 || !scratch || !col_use || !col_cap || !spatial || !over_count)
    return OGR_ERR_ARG;
  const int segZ = nz > 2 ? nz - 2 : 0;
  if (segZ > 0 && (!seg_use || !seg_cap)) return OGR_ERR_ARG;
  if (num_nets > 0 && (!store_len || !store_path)) return OGR_ERR_ARG;
  if (over_cap > 0 && !over) return OGR_ERR_ARG;
  cudaStream_t s = ogr_stream(stream);
  const int64_t plane = (int64_t)nx * ny;
  int32_t* col = scratch;
  int32_t* seg = scratch + plane;
  OGR_CUDA_TRY(cudaMemsetAsync(scratch, 0, sizeof(int32_t) * (size_t)plane * (1 + segZ), s));
  OGR_CUDA_TRY(cudaMemsetAsync(spatial, 0, sizeof(int64_t), s));
  OGR_CUDA_TRY(cudaMemsetAsync(over_count, 0, sizeof(int32_t), s));
  if (num_nets > 0) {
    via_use_kernel<<<ogr_blocks(num_nets, 128), 128, 0, s>>>(store_len, store_path, num_nets, slot_cap, nx, ny, nz,
                                                             col, seg);
    OGR_LAUNCH_CHECK();
  }
  via_use_finish_kernel<<<ogr_blocks(plane, 256), 256, 0, s>>>(
      nx, ny, nz, col, seg, col_use, seg_use, col_cap, seg_cap, reinterpret_cast<unsigned long long*>(spatial), over,
      over_cap, over_count);
  OGR_LAUNCH_CHECK();
  return OGR_OK;
}

extern "C" int ogr_via_pools_presence(int32_t nx, int32_t ny, int32_t nz, const int16_t* col_use,
                                      const int16_t* col_cap, const int16_t* seg_use, const int8_t* seg_cap,
                                      float* col_pres, float* seg_pres, float* seg_prefix, void* stream) {
  const int segZ = nz > 2 ? nz - 2 : 0;
  if (nx < 1 || ny < 1 || !col_use || !col_cap || !col_pres) return OGR_ERR_ARG;
  if (segZ > 0 && (!seg_use || !seg_cap || !seg_pres || !seg_prefix)) return OGR_ERR_ARG;
  const int64_t plane = (int64_t)nx * ny;
  via_presence_kernel<<<ogr_blocks(plane, 256), 256, 0, ogr_stream(stream)>>>(nx, ny, nz, col_use, col_cap, seg_use,
                                                                            seg_cap, col_pres, seg_pres, seg_prefix);
  OGR_LAUNCH_CHECK();
  return OGR_OK;
}

extern "C" int ogr_nets_overuse(const int32_t* store_len, const int32_t* store_arcs, int32_t num_nets,
                                int64_t arc_stride, const float* present, const float* capacity,
                                const int32_t* edge_src, const int32_t* indices, int32_t canonical_only,
                                double* sums, uint8_t* hit, void* stream) {
  if (num_nets < 0 || arc_stride < 0 || (num_nets > 0 && (!store_len || !store_arcs || !present || !capacity ||
                                                          !sums || !hit)))
    return OGR_ERR_ARG;
  if (canonical_only && (!edge_src || !indices)) return OGR_ERR_ARG;
  if (num_nets == 0) return OGR_OK;
  const int threads = 256;
  const int64_t blocks = ((int64_t)num_nets * 32 + threads - 1) / threads;
  nets_overuse_kernel<<<(int)(blocks < 152 * 16 ? blocks : 152 * 16), threads, 0, ogr_stream(stream)>>>(
      store_len, store_arcs, num_nets, arc_stride, present, capacity, edge_src, indices, canonical_only, sums, hit);
  OGR_LAUNCH_CHECK();
  return OGR_OK;
}

extern "C" int ogr_via_pools_apply(int64_t E, int32_t nx, int32_t ny, int32_t nz, const int32_t* edge_src,
                                   const int32_t* indices, const uint8_t* edge_kind, const float* col_pres,
                                   const float* seg_prefix, const int16_t* col_use, const int16_t* col_cap,
                                   const int16_t* seg_use, const int8_t* seg_cap, const double* discount,
                                   float col_weight, float seg_weight, float pres_fac, int32_t apply_penalty,
                                   int32_t apply_block, float* total_cost, void* stream) {
  if (nz < 2 || !edge_src || !indices || !edge_kind || !total_cost) return OGR_ERR_ARG;
  if (apply_penalty && !col_pres) return OGR_ERR_ARG;
  if (apply_block && (!col_use || !col_cap)) return OGR_ERR_ARG;
  via_pool_kernel<<<ogr_blocks(E, kThreads, 152 * 32), kThreads, 0, ogr_stream(stream)>>>(
      E, nx, ny, nz, edge_src, indices, edge_kind, col_pres, seg_prefix, col_use, col_cap, seg_use, seg_cap, discount,
      col_weight, seg_weight, pres_fac, apply_penalty, apply_block, total_cost);
  OGR_LAUNCH_CHECK();
  return OGR_OK;
}

extern "C" int ogr_overused_arcs(int64_t E, const float* present, const float* capacity, int32_t* out_idx,
                                 float* out_val, int32_t out_cap, uint32_t* count, void* stream) {
  if (!present || !capacity || !out_idx || !out_val || !count) return OGR_ERR_ARG;
  cudaStream_t s = ogr_stream(stream);
  OGR_CUDA_TRY(cudaMemsetAsync(count, 0, sizeof(uint32_t), s));
  overused_kernel<<<ogr_blocks(E, kThreads, 152 * 32), kThreads, 0, s>>>(E, present, capacity, out_idx, out_val,
                                                                          out_cap, count);
  OGR_LAUNCH_CHECK();
  return OGR_OK;
}

extern "C" int ogr_barrel_scan(const int32_t* store_len, const int32_t* store_path, const int32_t* net_id,
                               int32_t num_nets, int64_t slot_cap, int32_t nx, int32_t ny,
                               const int32_t* owner_count, const int32_t* owner_xor, const int32_t* path_node_use,
                               int32_t* mark, int32_t stamp, int64_t cap, int32_t* occ, int32_t* cnode,
                               int32_t* member, int32_t* shared, int64_t* counts, void* stream) {
  if (num_nets < 0 || nx < 1 || ny < 1 || cap < 0 || slot_cap < 2 || !counts) return OGR_ERR_ARG;
  if (num_nets > 0 && (!store_len || !store_path || !net_id || !owner_count || !owner_xor || !path_node_use ||
                       !mark || (cap > 0 && (!occ || !cnode || !member || !shared))))
    return OGR_ERR_ARG;
  cudaStream_t s = ogr_stream(stream);
  OGR_CUDA_TRY(cudaMemsetAsync(counts, 0, 5 * sizeof(int64_t), s));
  if (num_nets == 0) return OGR_OK;
  unsigned long long* c = reinterpret_cast<unsigned long long*>(counts);
  const int threads = 256;
  const int blocks = ogr_blocks((int64_t)num_nets * 32, threads);
  barrel_hops_kernel<<<blocks, threads, 0, s>>>(store_len, store_path, net_id, num_nets, slot_cap, owner_count,
                                                owner_xor, path_node_use, mark, stamp, cap, occ, cnode, shared, c);
  OGR_LAUNCH_CHECK();
  barrel_members_kernel<<<blocks, threads, 0, s>>>(store_len, store_path, net_id, num_nets, slot_cap, nx * ny,
                                                   owner_count, mark, stamp, cap, member, c);
  OGR_LAUNCH_CHECK();
  return OGR_OK;
}
