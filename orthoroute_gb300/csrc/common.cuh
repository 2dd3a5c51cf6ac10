// Shared helpers for the GB300 PathFinder kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/orthoroute_gb300.h"

#define OGR_CUDA_TRY(expr)                                   \
  do {                                                       \
    cudaError_t _e = (expr);                                 \
    if (_e != cudaSuccess) return OGR_ERR_CUDA;              \
  } while (0)

#define OGR_LAUNCH_CHECK() OGR_CUDA_TRY(cudaGetLastError())

static inline cudaStream_t ogr_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

static inline int ogr_blocks(int64_t n, int threads, int cap = 152 * 16) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (int)b;
}

// Non-negative doubles order like their bit patterns as unsigned integers.
__device__ __forceinline__ unsigned long long ogr_dbits(double d) {
  return (unsigned long long)__double_as_longlong(d);
}

// Node penalty of the search (_build_owner_penalty, unified_pathfinder.py:
// 5308-5384): foreign barrel owner + occupied path node + history, float32.
// The four loads are unconditional so they issue together.
__device__ __forceinline__ float ogr_node_penalty(const ogr_state& st, const ogr_net_args& a, int32_t gid) {
  if (!a.penalty_enabled) return 0.0f;
  const int32_t cnt = st.owner_count[gid];
  const int32_t xr = st.owner_xor[gid];
  const int32_t use = st.path_node_use[gid];
  const float hist = st.node_history[gid];
  const int32_t owner = (cnt == 0) ? -1 : (cnt == 1 ? xr : -2);
  const bool foreign = (owner != -1) && (owner != a.net_id);
  const float f = foreign ? a.owner_weight : 0.0f;
  const float o = use > 0 ? a.path_weight : 0.0f;
  return __fadd_rn(__fadd_rn(f, o), __fmul_rn(hist, a.history_weight));
}

// Any double to an unsigned key with the same order (negatives reversed).
__device__ __forceinline__ unsigned long long ogr_order_bits(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// (a32, lu, u) lexicographic less-than.
__device__ __forceinline__ bool ogr_key_lt(float a1, double l1, int32_t u1, float a2, double l2, int32_t u2) {
  if (a1 != a2) return a1 < a2;
  if (l1 != l2) return l1 < l2;
  return u1 < u2;
}

// Search parameters of net n of a pass (fallback = 1: the larger retry ROI).
__device__ inline ogr_net_args ogr_pass_net_args(const ogr_net_table& t, const ogr_pass_args& pa, int32_t n,
                                             int fallback) {
  ogr_net_args a;
  a.net_id = t.net_id[n];
  a.src = t.net_src[n];
  a.dst = t.net_dst[n];
  a.full_graph = fallback ? 0 : t.net_full[n];
  a.bfs_max_depth = t.net_depth[2 * n + fallback];
  a.bfs_halo = t.net_halo[2 * n + fallback];
  a.bfs_stop_count = pa.bfs_stop_count;
  a.max_roi_nodes = pa.max_roi_nodes;
  a.owner_weight = pa.owner_weight;
  a.path_weight = pa.path_weight;
  a.history_weight = pa.history_weight;
  a.penalty_enabled = pa.penalty_enabled;
  return a;
}

