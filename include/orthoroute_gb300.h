/*
 * orthoroute_gb300 — C ABI of the GB300 (sm_103a) PathFinder hot path.
 *
 * Drop-in boundary for OrthoRoute's negotiated-congestion inner loop
 * (orthoroute/algorithms/manhattan/unified_pathfinder.py).  Every entry point
 * takes plain pointers and sizes; every device buffer is owned by the caller
 * (the Python host allocates them as torch tensors and passes data_ptr()).
 * Scratch memory is a caller-provided workspace whose size is queried first.
 *
 * Conventions
 *   - return value: OGR_OK (0), OGR_NO_PATH (1) or a negative error;
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy stream);
 *   - no entry point synchronises the host unless it says so;
 *   - float scalars are the float32 roundings numpy would apply to the
 *     reference's Python floats (numpy 2 weak-scalar rule).
 */
#ifndef ORTHOROUTE_GB300_H
#define ORTHOROUTE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  OGR_OK = 0,
  OGR_NO_PATH = 1,
  OGR_ERR_ARG = -1,
  OGR_ERR_CUDA = -2,
  OGR_ERR_CAPACITY = -3,  /* a queue, ROI or path buffer is too small     */
  OGR_ERR_ITER_CAP = -4,  /* a device loop reached its iteration limit     */
  OGR_ERR_NUMERIC = -5,   /* an input violated an exactness precondition  */
  OGR_ERR_TIMEOUT = -6    /* a grid-wide barrier gave up waiting           */
};

/* ------------------------------------------------------------------ A1 ---
 * 3-D lattice → CSR.  Replaces Lattice3D.build_graph + CSRGraph.finalize
 * (unified_pathfinder.py:1656-1955 and :881-1002).  Rows are sorted by
 * destination id, exactly like the reference's structured sort
 * (order='src' breaks ties on dst then cost, :935).
 */
typedef struct {
  int32_t nx, ny, nz;
  float lateral_cost;          /* float32(pitch)                            */
  float wrong_way_cost;        /* <= 0: strict H/V discipline               */
  const uint8_t* layer_axis;   /* host [nz]: 0 none, 1 'h', 2 'v'           */
  const int32_t* partner_ptr;  /* host [nz+1]: via partners of each layer   */
  const int32_t* partner_z;    /* host, ascending within each layer         */
  const float* partner_cost;   /* host, float32 via cost of that pair       */
  const int32_t* partner_site; /* host, 0 all, 1 checkerboard, k>=2 stride  */
} ogr_lattice_desc;

int ogr_csr_num_edges(const ogr_lattice_desc* d, int64_t* num_edges);
size_t ogr_csr_workspace_bytes(const ogr_lattice_desc* d);
/* Builds indptr[N+1], indices[E], base_costs[E], edge_layer[E], edge_kind[E],
 * edge_src[E] and rev[E] (index of the opposite arc). */
int ogr_csr_build(const ogr_lattice_desc* d, int32_t* indptr, int32_t* indices,
                  float* base_costs, uint8_t* edge_layer, uint8_t* edge_kind,
                  int32_t* edge_src, int32_t* rev, void* workspace,
                  size_t workspace_bytes, void* stream);

/* --------------------------------------------------------------- A2–A4 ---
 * EdgeAccountant.update_costs (unified_pathfinder.py:1301-1384):
 *   total = base*vmult*bw*bias + (pres*bias)*max(0,ema-cap) + hw*history,
 *   +inf on blocked arcs, + float32(e) % 9973 * 1e-6.
 * layer_bias may be NULL (no per-layer bias).  blocked may be NULL.
 */
typedef struct {
  int64_t num_edges;
  const float* base_costs;
  const uint8_t* edge_layer;
  const uint8_t* edge_kind;
  const float* present_ema;
  const float* capacity;
  const float* history;
  const uint8_t* blocked;
  const float* layer_bias;     /* device [nz] float32 or NULL */
  float via_cost_multiplier;
  float base_cost_weight;
  float pres_fac;
  float hist_weight;
  int32_t add_jitter;
} ogr_cost_args;

int ogr_costs_update(const ogr_cost_args* a, float* total_cost, void* stream);

/* begin_live_present_costs (unified_pathfinder.py:1386-1401):
 * live_static = total - scale*max(0,ema-cap); total = live_static +
 * scale*max(0,present+1-cap); scale = pres_fac*bias (vias: pres_fac). */
int ogr_live_begin(const ogr_cost_args* a, const float* present, float* total_cost,
                   float* live_static, void* stream);

/* rcost[e] = total_cost[rev[e]]: the cost of the arc into each CSR row's
 * node, read by the searches in row order (no counterpart in the reference). */
int ogr_reverse_costs(int64_t num_edges, const int32_t* rev, const float* total_cost, float* rcost,
                      void* stream);

/* update_present_ema (unified_pathfinder.py:1291-1299). */
int ogr_present_ema(int64_t num_edges, const float* present, float* present_ema,
                    float beta, float one_minus_beta, void* stream);

/* update_history (unified_pathfinder.py:1226-1289) with the loop's raw-present
 * and 15x base-cost cap settings passed in. base_costs NULL = no cap. */
int ogr_history_update(int64_t num_edges, float* history, const float* present,
                       const float* present_ema, const float* capacity,
                       const float* base_costs, float gain, float cap_mult,
                       float decay, int32_t use_raw_present, void* stream);

/* ------------------------------------------------------------------ A5 ---
 * Via pools: penalties (_apply_via_pooling_penalties, CPU branch,
 * unified_pathfinder.py:5884-5980) and the hard block of saturated columns /
 * segments (_block_via_edges_with_collisions, :6094-6161) applied to every
 * via arc of total_cost.  Pools are x-major [nx][ny] and [nx][ny][nz-2];
 * discount[z_lo*nz+z_hi] (double, may be NULL) is the leave-hot-layer factor.
 */
int ogr_via_pools_apply(int64_t num_edges, int32_t nx, int32_t ny, int32_t nz,
                        const int32_t* edge_src, const int32_t* indices,
                        const uint8_t* edge_kind, const float* col_pres,
                        const float* seg_prefix, const int16_t* col_use,
                        const int16_t* col_cap, const int16_t* seg_use,
                        const int8_t* seg_cap, const double* discount, float col_weight,
                        float seg_weight, float pres_fac, int32_t apply_penalty,
                        int32_t apply_block, float* total_cost, void* stream);

/* Via pool use rebuilt from a path store (_rebuild_via_usage_from_committed,
 * unified_pathfinder.py:4548-4615; per path _accumulate_via_usage_for_path
 * :4470-4546): every maximal run of via hops in one column adds 1 to the
 * column and 1 to every segment z - 1 of the run's z hull clamped to
 * [1, nz-2].  store_len[k] / store_path[k * slot_cap] as ogr_route_pass
 * keeps them.  scratch: device int32[nx*ny*(1 + max(0, nz-2))].  Writes
 * col_use[nx][ny] and seg_use[nx][ny][nz-2] (int16, x-major), *spatial
 * (device int64) = Σ max(0, use - cap) over columns and segments, and the
 * over-full pools into over[5 * k] = {0 column / 1 segment, x, y, s, use}
 * with *over_count (device) their number (entries past over_cap are
 * dropped; call again with more room).  Asynchronous. */
int ogr_via_pools_rebuild(const int32_t* store_len, const int32_t* store_path, int32_t num_nets,
                          int64_t slot_cap, int32_t nx, int32_t ny, int32_t nz, int32_t* scratch,
                          int16_t* col_use, int16_t* seg_use, const int16_t* col_cap,
                          const int8_t* seg_cap, int64_t* spatial, int32_t* over, int32_t over_cap,
                          int32_t* over_count, void* stream);

/* The via-present EMA and z prefix (unified_pathfinder.py:6279-6303):
 * col_pres = 0.6 * max(0, col_use - cap) + 0.4 * col_pres, the same for
 * seg_pres, seg_prefix = its float32 running sum over z; float32 in numpy's
 * operation order.  Asynchronous. */
int ogr_via_pools_presence(int32_t nx, int32_t ny, int32_t nz, const int16_t* col_use,
                           const int16_t* col_cap, const int16_t* seg_use, const int8_t* seg_cap,
                           float* col_pres, float* seg_pres, float* seg_prefix, void* stream);

/* Compact the arcs with present > capacity (any order) into out_idx/out_val
 * (max(0,present-cap)); *count (device) receives the total, which may exceed
 * out_cap (then only out_cap entries are written). */
int ogr_overused_arcs(int64_t num_edges, const float* present, const float* capacity,
                      int32_t* out_idx, float* out_val, int32_t out_cap, uint32_t* count,
                      void* stream);

/* Per-net overuse for the negotiation policy's net order, hotset and rip-up
 * choice (the reference sums max(0, present - capacity) over each net's arcs,
 * _order_nets_by_difficulty :7840-7901, _rip_top_k_offenders :9751-9781):
 * for each of num_nets store slots (store_len[k] nodes, arcs at
 * store_arcs[k * arc_stride], forward then reverse as ogr_route_pass writes
 * them) sums[k] (double) = the sum over its arcs, hit[k] = 1 if any arc is
 * overused; canonical_only = 1 counts only arcs with src < dst.  The values
 * are whole numbers, so the sums are exact.  Asynchronous. */
int ogr_nets_overuse(const int32_t* store_len, const int32_t* store_arcs, int32_t num_nets,
                     int64_t arc_stride, const float* present, const float* capacity,
                     const int32_t* edge_src, const int32_t* indices, int32_t canonical_only,
                     double* sums, uint8_t* hit, void* stream);

/* Exact barrel conflicts and shared path nodes of the stored paths
 * (_detect_barrel_conflicts, unified_pathfinder.py:10778-11111, with
 * _detect_path_node_conflicts :10564-10606), as device lists the host turns
 * into the conflict sets, pairs and scores.  For every hop (u, v) of the
 * stored path of slot n (net id net_id[n]) an endpoint conflicts when its
 * barrel owner (from owner_count / owner_xor: -1 none, the id for one net,
 * -2 for several) is neither -1 nor the net's id.  counts (device int64[5],
 * zeroed here) = {conflicting hops, occ entries, cnode entries, member
 * entries, shared entries}; each list holds min(count, cap) entries:
 *   occ[2i..]    (endpoint node, net id) of every conflicting endpoint of
 *                every conflicting hop (two for a hop conflicting at both);
 *   cnode[3i..]  (node, owner_count, owner_xor) of each distinct conflict node;
 *   member[2i..] (node, net id) of the nets whose via hops span a conflict
 *                node that several nets own (repeats possible);
 *   shared[2i..] (node, slot) of every stored-path node with path-node use
 *                above 1.
 * mark: device int32[num_nodes] scratch whose entries differ from `stamp` on
 * entry (use a new stamp per call).  Asynchronous. */
int ogr_barrel_scan(const int32_t* store_len, const int32_t* store_path, const int32_t* net_id,
                    int32_t num_nets, int64_t slot_cap, int32_t nx, int32_t ny,
                    const int32_t* owner_count, const int32_t* owner_xor, const int32_t* path_node_use,
                    int32_t* mark, int32_t stamp, int64_t cap, int32_t* occ, int32_t* cnode,
                    int32_t* member, int32_t* shared, int64_t* counts, void* stream);

/* ------------------------------------------------------------------ A9 ---
 * Tallies (compute_overuse :1137-1190, _compute_path_node_overuse
 * :10718-10726, _compute_layer_bias's bincount :8473-8500).
 * out[0] = Σ max(0,present-cap) over canonical arcs (src<dst) or all arcs,
 * out[1] = number of such arcs > 0, out[2] = Σ max(0,use-1) over nodes,
 * out[3] = nodes with use > 1; layer_units[z] = Σ over arcs of layer z of
 * max(0,ema-cap) in units of 2^-23 plus Σ max(0,use-1) of layer z in units
 * of 2^-23 (exact integers; the host divides).  out[4] != 0 flags an EMA
 * value off the 2^-23 grid.  out (int64[5]) and layer_units (int64[nz]) are
 * device arrays, zeroed here. */
int ogr_tally(int64_t num_edges, int32_t num_nodes, int32_t nz, const float* present,
              const float* present_ema, const float* capacity, const int32_t* edge_src,
              const int32_t* indices, const uint8_t* edge_layer, const int32_t* path_node_use,
              int32_t canonical_only, int64_t* out, int64_t* layer_units, void* stream);

/* ------------------------------------------------------------- A6–A8 ---
 * Route one net: rip-up of its old path (optional), bidirectional BFS ROI
 * (extract_roi_bfs :2257-2384), exact ROI SSSP (find_path_roi :2451-2548),
 * backtrace, and commit (commit_path :1096, refresh_live_present_costs
 * :1403, _mark_path_node_use :4635, _mark_via_barrel_ownership_for_path
 * :4934, _path_to_edges :9981-10046).
 */
typedef struct {
  int32_t nx, ny, nz;
  int32_t num_nodes;
  int64_t num_edges;
  const int32_t* indptr;
  const int32_t* indices;
  const int32_t* rev;
  const uint8_t* blocked;      /* NULL: none */
} ogr_graph;

typedef struct {
  float* total_cost;           /* live total cost (read by the search)       */
  const float* live_static;    /* static part for live-present refresh        */
  float* present;
  const float* capacity;
  const float* layer_bias;     /* device [nz] float32 of the cost update, or NULL */
  const uint8_t* edge_layer;
  const uint8_t* edge_kind;
  int32_t* path_node_use;
  int32_t* owner_count;        /* barrel ownership: #nets per node            */
  int32_t* owner_xor;          /* XOR of those net ids (= id when count==1)   */
  const float* node_history;
  float* rcost;                /* NULL, or rcost[e] = total_cost[rev[e]] kept in
                                  sync by ogr_path_apply / ogr_route_pass; after
                                  any other change of total_cost call
                                  ogr_reverse_costs before the next search     */
} ogr_state;

typedef struct {
  int32_t net_id;
  int32_t src, dst;
  int32_t full_graph;          /* 1: ROI = whole graph (Manhattan >= 125)     */
  int32_t bfs_max_depth;       /* min(int(radius + 2*bonus), 80)              */
  int32_t bfs_halo;            /* min(16, 2 + int(max(0,bonus)/0.6))          */
  double bfs_stop_count;       /* early stop when seen > this (1.5*max nodes) */
  int32_t max_roi_nodes;       /* 50,000 in the reference                     */
  float owner_weight;          /* float32(25*pres_fac) (or the cleanup value) */
  float path_weight;           /* float32(25*pres_fac)                        */
  float history_weight;        /* float32(5.0)                                */
  int32_t penalty_enabled;     /* 0: no node penalty at all                   */
} ogr_net_args;

/* Per-search scratch (one "slot"): about 70 bytes per lattice node.  It must
 * be initialised once with ogr_route_workspace_init; every search leaves it
 * initialised again.  Two searches must not share a slot concurrently. */
size_t ogr_route_workspace_bytes(int32_t num_nodes);
int ogr_route_workspace_init(void* workspace, size_t workspace_bytes, int32_t num_nodes,
                             void* stream);

/* Search only (no state change).  path_out: device int32[path_cap];
 * *path_len_out (host) = nodes written.  stats (device int64[4], may be
 * NULL): arcs the sequential heap search scans before it pops dst, nodes it
 * pops, ROI size, settle phases.  Returns OGR_OK / OGR_NO_PATH / an error;
 * synchronises the stream to read the status. */
int ogr_find_path(const ogr_graph* g, const ogr_state* st, const ogr_net_args* net,
                  void* workspace, size_t workspace_bytes, int32_t* path_out,
                  int32_t path_cap, int32_t* path_len_out, int64_t* stats, void* stream);

/* The reference's solver seam, SimpleDijkstra.find_path_roi(src, dst, costs,
 * roi_nodes, global_to_roi, node_penalty) (unified_pathfinder.py:2451-2548):
 * search the given ROI (device int32[n_roi], global ids; its order is the
 * heap's tie order) with arc costs `costs` (device float32[E]) and the
 * ROI-local node penalty roi_penalty (device float32[n_roi], or NULL).
 * Duplicate ROI entries are not allowed.  Same outputs, statistics and
 * status codes as ogr_find_path; synchronises. */
int ogr_find_path_roi(const ogr_graph* g, const float* costs, const int32_t* roi_nodes, int32_t n_roi,
                      const float* roi_penalty, int32_t src, int32_t dst, void* workspace,
                      size_t workspace_bytes, int32_t* path_out, int32_t path_cap,
                      int32_t* path_len_out, int64_t* stats, void* stream);

/* The multi-source multi-sink seam, SimpleDijkstra.find_path_multisource_multisink(
 * src_seeds, dst_targets, costs, roi_nodes, global_to_roi, node_penalty)
 * (unified_pathfinder.py:2550-2659), used for portal-seeded nets (:8321,
 * :8355): seeds (device int32[n_seeds], global ids) start with label
 * seed_cost (device float64) + their node penalty; targets (device
 * int32[n_targets]) are settled but never expanded, each with target_cost
 * (device float64); the search exhausts the ROI and returns the path to the
 * target with the least label + target cost (first in the heap's pop order
 * among equals), seed first.  Seeds or targets outside the ROI are ignored;
 * a repeated seed or target id is OGR_ERR_ARG.  The path's first and last
 * nodes give the reference's entry and exit layers.  Workspace:
 * ogr_multi_workspace_bytes (the route workspace + 16 bytes per node),
 * initialised with ogr_route_workspace_init.  stats (may be NULL): arcs of
 * the expanded nodes, nodes popped, ROI size, settle phases.  Synchronises. */
size_t ogr_multi_workspace_bytes(int32_t num_nodes);
int ogr_find_path_multi(const ogr_graph* g, const float* costs, const int32_t* roi_nodes, int32_t n_roi,
                        const float* roi_penalty, const int32_t* seeds, const double* seed_cost,
                        int32_t n_seeds, const int32_t* targets, const double* target_cost,
                        int32_t n_targets, void* workspace, size_t workspace_bytes,
                        int32_t* path_out, int32_t path_cap, int32_t* path_len_out,
                        int64_t* stats, void* stream);

/* Commit many paths in one launch, as the best-state restore re-commits
 * every path (_restore_routing_state, unified_pathfinder.py:7806-7838, with
 * commit_path :1096-1135, _rebuild_path_node_use :4623, _rebuild_node_owner
 * :4744): present +1 on both arcs of each hop, path-node use +1, barrel
 * ownership of every via-spanned node, no live refresh.  Path k is
 * nodes[offsets[k] .. offsets[k+1]) (device int32, >= 2 nodes each) of net
 * net_ids[k]; its arcs (forward then reverse) go to
 * arcs_out[2 * (offsets[k] - k) ..].  With store_path / store_len /
 * store_arcs (each may be NULL) the path, its length and its arcs are also
 * written to slot store_slot[k] of a path store with slot_cap nodes and
 * 2 * slot_cap arcs per slot.  The paths must not be committed already; the
 * result equals committing them one by one in any order.  *status_dev:
 * 0, 1 (a hop is not an arc) or 2 (capacity).  Asynchronous. */
int ogr_paths_commit(const ogr_graph* g, const ogr_state* st, const int32_t* nodes, const int32_t* offsets,
                     const int32_t* net_ids, int32_t n_paths, int32_t* arcs_out, int32_t* store_path,
                     int32_t* store_len, int32_t* store_arcs, const int32_t* store_slot, int32_t slot_cap,
                     int32_t* status_dev, void* stream);

/* Commit (sign=+1) or rip up (sign=-1) a path given as device node ids:
 * present +-1 (floored at 0), live-present refresh of those arcs when
 * live != 0, path-node use +-1, barrel ownership of every node spanned by a
 * via hop.  Writes the arc list (forward then reverse, like _path_to_edges)
 * into arcs_out[2*(len-1)] when not NULL, and OGR_OK / OGR_ERR_ARG (a hop is
 * not an arc) into the device word *status_dev.  Asynchronous. */
int ogr_path_apply(const ogr_graph* g, const ogr_state* st, const int32_t* path, int32_t len,
                   int32_t net_id, int32_t sign, float pres_fac_f32, int32_t live,
                   int32_t* arcs_out, int32_t* status_dev, void* stream);

/* ROI only (for tests / scheduling): writes the ROI node list in the
 * reference's order and its size.  Synchronises. */
int ogr_extract_roi(const ogr_graph* g, const ogr_net_args* net, void* workspace,
                    size_t workspace_bytes, int32_t* roi_out, int32_t roi_cap,
                    int32_t* roi_len_out, void* stream);

/* --------------------------------------------------------------- A8/A10 ---
 * One routing pass in one launch: for each net of `order`, in order, the
 * sequence of _route_all (unified_pathfinder.py:7949-8449): rip up its stored
 * path, search its ROI (or the whole graph), retry once with the larger
 * fallback ROI while the pass has fallbacks left (< 5 per iteration,
 * :8337-8370), commit the new path.  Paths live in a device store of
 * num_nets slots of slot_cap nodes; store_arcs receives each committed path's
 * arcs (forward then reverse).  net_status[k] = 1 if the k-th net failed,
 * | 2 if it used a fallback.  Synchronises; returns OGR_OK or an error. */
typedef struct {
  int32_t num_nets;
  int32_t slot_cap;
  int32_t* store_len;          /* [num_nets] nodes of the current path (0 = none) */
  int32_t* store_path;         /* [num_nets * slot_cap]                           */
  int32_t* store_arcs;         /* [num_nets * 2 * slot_cap]                       */
  const int32_t* net_src;
  const int32_t* net_dst;
  const int32_t* net_id;       /* ownership id of each net                        */
  const int32_t* net_full;     /* 1: full-graph search (Manhattan >= 125)         */
  const int32_t* net_depth;    /* [2*num_nets] BFS depth: normal, fallback        */
  const int32_t* net_halo;     /* [2*num_nets] BFS halo: normal, fallback         */
} ogr_net_table;

typedef struct {
  const int32_t* order;
  int32_t count;
  int32_t fallback_quota;
  int32_t max_roi_nodes;
  double bfs_stop_count;
  float owner_weight;
  float path_weight;
  float history_weight;
  int32_t penalty_enabled;
  float pres_fac;              /* float32(pres_fac) for the live refresh          */
  int32_t live;
  int32_t* net_status;         /* [count]                                         */
  int64_t* stats;              /* [4] accumulated search statistics               */
} ogr_pass_args;

/* Optional batched ROI extraction for a pass: before the sequential part,
 * `slots` CTAs extract the ROIs of all ROI nets of `order` in parallel (the
 * BFS reads no costs), each into roi_pool[n*roi_cap] (roi_cap >= the pass's
 * max_roi_nodes), roi_len[n] = size or -1 (queue overflow: that net's ROI
 * is then extracted inline).  bfs_ws holds `slots` slots of slot_bytes
 * (ogr_bfs_workspace_bytes / ogr_bfs_workspace_init); next is a device int. */
typedef struct {
  int32_t slots;
  size_t slot_bytes;
  int64_t qcap;
  void* bfs_ws;
  int32_t* roi_pool;
  int32_t* roi_len;
  int32_t roi_cap;
  int32_t* next;
  int32_t* roi_box;            /* NULL, or [4*num_nets]: x0, x1, y0, y1 of the
                                  BFS region holding each ROI                   */
} ogr_roi_batch;

/* Batched disjoint-ROI windows for the ROI nets of a pass.  Consecutive ROI
 * nets whose footprints (the ROI's box and the box of the net's old path) are
 * pairwise disjoint are ripped up and searched together, one CTA each, in one
 * cooperative launch; they then commit in order.  A net whose ROI search
 * fails ends its window: the later nets' rip-ups are undone and it takes its
 * fallback in order.  The results are those of the sequential pass.
 * ws holds `slots` search slots of slot_bytes (ogr_window_workspace_*),
 * scratch holds slots x slot_cap path nodes, ctl is device scratch of
 * ogr_window_ctl_bytes(slots) bytes.  discarded (device int64[3], may be
 * NULL) accumulates {searches, arcs scanned, nodes popped} of the window
 * searches whose results were undone because an earlier member of their
 * window failed: those nets are searched again later, and only accepted
 * searches count in the pass's `stats`. */
typedef struct {
  int32_t slots;
  size_t slot_bytes;
  void* ws;
  int32_t* scratch;
  void* ctl;
  int64_t* discarded;
} ogr_window_args;

size_t ogr_window_workspace_bytes(int32_t num_nodes, int32_t max_roi_nodes, int32_t slots);
int ogr_window_workspace_init(void* workspace, int32_t num_nodes, int32_t max_roi_nodes, int32_t slots,
                              void* stream);
size_t ogr_window_ctl_bytes(int32_t slots);

size_t ogr_bfs_workspace_bytes(int32_t num_nodes, int64_t qcap, int32_t slots);
int ogr_bfs_workspace_init(void* workspace, int32_t num_nodes, int64_t qcap, int32_t slots,
                           void* stream);

/* rb may be NULL (every ROI is extracted inline, in order).  win (may be
 * NULL) batches the ROI nets into disjoint windows; it needs rb with
 * roi_box.
 * order_full (HOST uint8[count], may be NULL) marks the entries of `order`
 * that are full-graph nets; each of those is searched by the whole-lattice
 * search (ogr_find_path_full) in full_workspace, the ROI nets between them by
 * single-CTA launches, in the same order.  With order_full NULL every net,
 * long or not, is searched by the single-CTA pass. */
int ogr_route_pass(const ogr_graph* g, const ogr_state* st, const ogr_net_table* t,
                   const ogr_pass_args* pa, const ogr_roi_batch* rb, void* workspace,
                   size_t workspace_bytes, const uint8_t* order_full, void* full_workspace,
                   size_t full_workspace_bytes, const ogr_window_args* win, int32_t* status_out,
                   void* stream);

/* Whole-lattice search for nets with Manhattan length >= 125 (the
 * reference's full-graph branch of _route_all, unified_pathfinder.py:
 * 8219-8262, into find_path_roi :2451-2548 with roi_nodes = all nodes).  Same
 * result, statistics and status codes as ogr_find_path with
 * net->full_graph = 1, computed by one cooperative launch on all SMs.  The
 * workspace (about 108 bytes per node + 4 per arc) is initialised once with
 * ogr_full_workspace_init; a search rewrites the 8-byte key word of every
 * node and otherwise touches only the nodes it reaches.
 * OGR_ERR_TIMEOUT: a grid barrier gave up (not expected; the launch is
 * sized so every CTA is resident).  Synchronises. */
size_t ogr_full_workspace_bytes(int32_t num_nodes, int64_t num_edges);
int ogr_full_workspace_init(void* workspace, size_t workspace_bytes, int32_t num_nodes,
                            int64_t num_edges, void* stream);
int ogr_find_path_full(const ogr_graph* g, const ogr_state* st, const ogr_net_args* net,
                       void* workspace, size_t workspace_bytes, int32_t* path_out,
                       int32_t path_cap, int32_t* path_len_out, int64_t* stats, void* stream);

/* Whole-lattice multi-source multi-sink search: the portal-seeded route of a
 * long net (the reference's full-graph seeded search,
 * find_path_fullgraph_gpu_seeds, pathfinder/cuda_dijkstra.py:5516, with the
 * CPU semantics of SimpleDijkstra.find_path_multisource_multisink,
 * unified_pathfinder.py:2550-2659, on roi_nodes = all nodes).  seeds
 * (device int32[n_seeds], distinct) start with label seed_cost (device
 * float64, >= 0) + their node penalty and no parent, ahead of every
 * relaxation with the same float32 value; targets (device int32[n_targets],
 * distinct) settle but never expand; the search runs until nothing is left
 * and returns the path to the target with the least (label + target_cost,
 * label, node id), seed first.  The node penalty and net id come from `net`
 * (its src / dst are not used).  A repeated or out-of-range seed or target,
 * a negative or NaN seed cost or a NaN target cost is OGR_ERR_ARG.
 * Workspace as ogr_find_path_full.  stats (may be NULL): arcs of the
 * expanded nodes, nodes settled, lattice size, settle phases.  Synchronises. */
int ogr_find_path_full_multi(const ogr_graph* g, const ogr_state* st, const ogr_net_args* net,
                             const int32_t* seeds, const double* seed_cost, int32_t n_seeds,
                             const int32_t* targets, const double* target_cost, int32_t n_targets,
                             void* workspace, size_t workspace_bytes, int32_t* path_out, int32_t path_cap,
                             int32_t* path_len_out, int64_t* stats, void* stream);

/* Grid of the whole-lattice search on the current device (a tuning knob;
 * results do not depend on it): ctas > 0 sets the number of cooperative CTAs
 * (at most *limit = SMs x resident CTAs per SM), 0 only reads.  *current and
 * *limit (host, may be NULL) receive the grid in use and the maximum.  The
 * setting is per device and per host thread.  Chosen by the autotuner
 * (orthoroute_gb300/autotune.py); no reference counterpart. */
int ogr_full_grid(int32_t ctas, int32_t* current, int32_t* limit);

/* Lanes per examined frontier node of the whole-lattice search (4, 8 or 16;
 * default 16) for searches launched afterwards; 0 only reads.  A tuning
 * knob (results do not depend on it), per host thread (each job of a
 * server routes in its own thread), chosen by the
 * autotuner; no reference counterpart. */
int ogr_full_lanes(int32_t lanes, int32_t* current);

/* Whether the whole-lattice search keeps the last pull of a carried frontier
 * node none of whose in-neighbours settled since (mode 1) or pulls every
 * frontier node every phase (0, default); -1 only reads.  A tuning knob
 * (results do not depend on it), per host thread, chosen by the autotuner; no
 * reference counterpart. */
int ogr_full_reuse(int32_t mode, int32_t* current);

/* Engine of the whole-lattice search for searches launched afterwards:
 * enable = 1 selects the tile-window engine with window width `delta`
 * (label units, > 0) and tiles of tx x ty cells over all layers (0: sized
 * from the lattice to fit shared memory); enable = 0 keeps the
 * phase-settled engine; -1 only reads (*cur_enable, *cur_delta, host, may be
 * NULL).  The tile engine computes the same fixed point with many hops per
 * grid step; a net it cannot take (a cost or penalty below 2^-7, a label
 * of 2^23 or more, a tile over capacity, an iteration cap) is searched by
 * the phase engine in the same stream, so results, statistics and status
 * codes do not depend on this setting.  Per host thread, chosen by the
 * autotuner; the window width is the delta of a delta-stepping search; no
 * reference counterpart. */
int ogr_full_tile(int32_t enable, double delta, int32_t tx, int32_t ty, int32_t* cur_enable,
                  double* cur_delta);

/* Tracing of the tile-window engine (host int64[24], cumulative since the
 * last reset): searches, grid rounds, windows, kernel ns, searches handed to
 * the phase engine, bit set of the reasons for handing over, local
 * iterations, tile processings; ns summed over CTAs spent loading tile
 * structure, loading labels, iterating and writing back, and waiting at grid
 * barriers; structure loads; the most tiles one CTA took in a round; node
 * evaluations; ns of first sweeps.  Synchronous. */
int ogr_tile_profile(int64_t* out24, int32_t reset);

/* Lanes per node of the single-CTA ROI search (2, 4, 8 or 16; default 4) for
 * every search launched afterwards; 0 only reads.  *current (host, may be
 * NULL) receives the setting.  A tuning knob (results do not depend on it),
 * per host thread, chosen by the autotuner; no reference counterpart. */
int ogr_search_lanes(int32_t lanes, int32_t* current);

/* How many clashing nets a disjoint-ROI window of ogr_route_pass may skip
 * to take later nets (0..16, default 8; 0 = consecutive nets only); -1 only
 * reads.  A later net joins only if its footprint also misses every skipped
 * net's footprint grown to its fallback ROI bound, and a member that fails
 * while nets before it are pending is undone and retried in its turn, so
 * results equal the sequential pass.  Per host thread; no reference
 * counterpart. */
int ogr_window_lookahead(int32_t nets, int32_t* current);

/* Limits for tests of failure handling in the phase-settled whole-lattice
 * search: barrier_spin = n > 0 lets a CTA poll the grid barrier n - 1 times
 * before it gives up (the search then returns OGR_ERR_TIMEOUT), 0 restores
 * the default bound; max_phases > 0 caps the settle phases (OGR_ERR_ITER_CAP
 * when a search needs more), 0 restores the default (2N + 4, never reached);
 * -1 leaves a setting.  *cur_spin / *cur_phases (host, may be NULL) receive
 * the settings.  Both failures are ordinary bounded exits: the kernel
 * returns, the context stays usable, and the routing pass stops before
 * committing the failed net, so the congestion state matches the stored
 * paths.  Per host thread; no reference counterpart (the reference raises on a
 * full queue, pathfinder/persistent_kernel.py:699-700). */
int ogr_debug_limits(int32_t barrier_spin, int32_t max_phases, int32_t* cur_spin, int32_t* cur_phases);

/* Tracing of the whole-lattice search (host int64[8], cumulative since the
 * last reset): searches, phases, kernel ns, init ns, E-step work ns and
 * S-step work ns of the busiest CTA, barrier wait ns and statistics +
 * backtrace ns of CTA 0.  Synchronous. */
int ogr_full_profile(int64_t* out8, int32_t reset);

/* Tracing: cumulative per-stage cycle counters of all searches on the
 * current device since the last reset (host int64[16]: BFS, compaction,
 * search init, queueing, recompute, frontier min, settle, statistics and
 * backtrace, cleanup; then searches, settle phases, BFS waves, ROI nodes,
 * recomputed nodes).  Synchronous. */
int ogr_search_profile(int64_t* out16, int32_t reset);

/* Allocation-free variant of ogr_find_path.  It has no counterpart in the
 * reference: it exists for callers that cannot allocate device memory for a
 * workspace (a plugin inside an application that owns the device allocator,
 * or a serving process whose memory budget is fixed at start-up).  Its
 * scratch is a fixed array inside the library (36 MB: about 76 bytes per
 * node for OGR_NOALLOC_MAX_NODES nodes plus a 16 MB local adjacency, resident on each GPU that loads the library
 * until exit), so lattices above OGR_NOALLOC_MAX_NODES nodes are refused with
 * OGR_ERR_CAPACITY.  The first call on a device looks up that array's device
 * address and keeps it for the process; make it before any stream capture,
 * and do not call this entry point again after resetting that device
 * (cudaDeviceReset ends the context that address belongs to).  Calls share
 * the array: do not let two calls overlap on the GPU.  Synchronises like
 * ogr_find_path. */
#define OGR_NOALLOC_MAX_NODES 262144
int ogr_find_path_noalloc(const ogr_graph* g, const ogr_state* st, const ogr_net_args* net,
                          int32_t* path_out, int32_t path_cap, int32_t* path_len_out,
                          int64_t* stats, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* ORTHOROUTE_GB300_H */
