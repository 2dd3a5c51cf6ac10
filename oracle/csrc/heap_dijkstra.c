/*
 * Oracle (test infrastructure): C restatement of the reference's ROI heap
 * Dijkstra, SimpleDijkstra.find_path_roi
 * (orthoroute/algorithms/manhattan/unified_pathfinder.py:2451-2548).
 *
 *  - heap of (double label, roi index), popped in lexicographic order;
 *  - dist is float32; a relaxation alt = (du + cost) + pen is accepted iff
 *    (float)alt < dist[v] (numpy 2 compares a Python float with a float32 in
 *    float32), then dist[v] = (float)alt, parent[v] = u, push (alt, v);
 *  - a node is settled once; the search stops when dst is popped.
 *
 * Every heap entry (label, index) is distinct (a node is pushed again only
 * with a strictly smaller float32 value), so any exact priority queue pops
 * them in the same order as Python's heapq; a 4-ary heap is used because it
 * touches fewer cache lines per pop.  When the ROI is the whole lattice in
 * id order (full-graph nets) the global->ROI lookups are the identity and
 * are skipped.
 *
 * It is used only by the CPU baseline and by tests, never by the product.
 * Compile with -ffp-contract=off so no operation is fused.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
typedef struct { double key; int32_t idx; int32_t pad; } item;
static inline int less(const item* a, const item* b) {
  return a->key < b->key || (a->key == b->key && a->idx < b->idx);
}
static inline void push(item* h, int64_t* n, item it) {
  int64_t i = (*n)++;
  while (i > 0) {
    int64_t p = (i - 1) >> 2;
    if (!less(&it, &h[p])) break;
    h[i] = h[p];
    i = p;
  }
  h[i] = it;
}
static inline item pop(item* h, int64_t* n) {
  item top = h[0];
  item last = h[--(*n)];
  int64_t m = *n, i = 0;
  for (;;) {
    int64_t c = 4 * i + 1;
    if (c >= m) break;
    int64_t b = c;
    int64_t e = c + 4 < m ? c + 4 : m;
    for (int64_t k = c + 1; k < e; ++k) if (less(&h[k], &h[b])) b = k;
    if (!less(&h[b], &last)) break;
    h[i] = h[b];
    i = b;
  }
  if (m > 0) h[i] = last;
  return top;
}
/* Returns 0 = path found, 1 = no path, -1 = allocation failure.  n_nodes is
 * the lattice's node count (len(indptr) - 1). */
int oracle_heap_dijkstra(int32_t src, int32_t dst, const int32_t* indptr, const int32_t* indices,
                         const float* costs, const int32_t* roi_nodes, int32_t R, const int32_t* g2r,
                         const float* pen, int32_t* path_out, int32_t* path_len, int64_t* stats,
                         int32_t n_nodes) {
  int32_t rs = g2r[src], rd = g2r[dst];
  *path_len = 0;
  if (rs < 0 || rd < 0) return 1;
  float* dist = (float*)malloc(sizeof(float) * (size_t)R);
  int32_t* parent = (int32_t*)malloc(sizeof(int32_t) * (size_t)R);
  unsigned char* visited = (unsigned char*)calloc((size_t)R, 1);
  int64_t cap = 1024, n = 0;
  item* h = (item*)malloc(sizeof(item) * (size_t)cap);
  if (!dist || !parent || !visited || !h) return -1;
  for (int32_t i = 0; i < R; ++i) { dist[i] = INFINITY; parent[i] = -1; }
  dist[rs] = 0.0f;
  item first = {0.0, rs, 0};
  push(h, &n, first);
  int64_t scanned = 0, settled = 0;
  /* the identity ROI (the whole lattice in id order): g2r[v] == v for every node */
  int ident = R == n_nodes;
  for (int32_t i = 0; i < R && ident; ++i) ident = roi_nodes[i] == i;
  while (n > 0) {
    item it = pop(h, &n);
    int32_t u = it.idx;
    if (visited[u]) continue;
    visited[u] = 1;
    ++settled;
    if (u == rd) break;
    if (n > 0) {
      int32_t nu = h[0].idx;
      __builtin_prefetch(&visited[nu]);
      __builtin_prefetch(&indptr[ident ? nu : roi_nodes[nu]]);
    }
    int32_t ug = ident ? u : roi_nodes[u];
    int32_t e0 = indptr[ug], e1 = indptr[ug + 1];
    scanned += e1 - e0;
    for (int32_t e = e0; e < e1; ++e) {
      int32_t v = ident ? indices[e] : g2r[indices[e]];
      if (v < 0 || visited[v]) continue;
      double alt = it.key + (double)costs[e];
      if (pen) alt = alt + (double)pen[v];
      float a32 = (float)alt;
      if (a32 < dist[v]) {
        dist[v] = a32;
        parent[v] = u;
        if (n == cap) {
          cap *= 2;
          item* nh = (item*)realloc(h, sizeof(item) * (size_t)cap);
          if (!nh) { free(h); free(dist); free(parent); free(visited); return -1; }
          h = nh;
        }
        item ni = {alt, v, 0};
        push(h, &n, ni);
      }
    }
  }
  int rc = 1;
  if (isfinite(dist[rd])) {
    int32_t len = 0;
    for (int32_t c = rd; c != -1; c = parent[c]) ++len;
    int32_t i = len - 1;
    for (int32_t c = rd; c != -1; c = parent[c]) path_out[i--] = roi_nodes[c];
    *path_len = len;
    rc = len > 1 ? 0 : 1;
  }
  if (stats) { stats[0] += scanned; stats[1] += settled; }
  free(h); free(dist); free(parent); free(visited);
  return rc;
}
