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
 * It is used only by the CPU baseline and by tests, never by the product.
 * Compile with -ffp-contract=off so no operation is fused.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

typedef struct { double key; int32_t idx; } item;

static int less(const item* a, const item* b) {
  if (a->key != b->key) return a->key < b->key;
  return a->idx < b->idx;
}

static void push(item* h, int64_t* n, item it) {
  int64_t i = (*n)++;
  h[i] = it;
  while (i > 0) {
    int64_t p = (i - 1) / 2;
    if (!less(&h[i], &h[p])) break;
    item t = h[i]; h[i] = h[p]; h[p] = t;
    i = p;
  }
}

static item pop(item* h, int64_t* n) {
  item top = h[0];
  h[0] = h[--(*n)];
  int64_t i = 0;
  for (;;) {
    int64_t l = 2 * i + 1, r = l + 1, m = i;
    if (l < *n && less(&h[l], &h[m])) m = l;
    if (r < *n && less(&h[r], &h[m])) m = r;
    if (m == i) break;
    item t = h[i]; h[i] = h[m]; h[m] = t;
    i = m;
  }
  return top;
}

/* Returns 0 = path found, 1 = no path, -1 = allocation failure. */
int oracle_heap_dijkstra(int32_t src, int32_t dst, const int32_t* indptr, const int32_t* indices,
                         const float* costs, const int32_t* roi_nodes, int32_t R, const int32_t* g2r,
                         const float* pen, int32_t* path_out, int32_t* path_len, int64_t* stats) {
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
  item first = {0.0, rs};
  push(h, &n, first);
  int64_t scanned = 0, settled = 0;
  while (n > 0) {
    item it = pop(h, &n);
    int32_t u = it.idx;
    if (visited[u]) continue;
    visited[u] = 1;
    ++settled;
    if (u == rd) break;
    int32_t ug = roi_nodes[u];
    for (int32_t e = indptr[ug]; e < indptr[ug + 1]; ++e) {
      ++scanned;
      int32_t v = g2r[indices[e]];
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
        item ni = {alt, v};
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
