// Internal interface of the whole-lattice search (fullgraph.cu) used by the
// routing pass in route.cu.
#pragma once
#include "common.cuh"

namespace ogr_full {

// Which net to search: explicit arguments, or net order[k] of a pass (then
// the path goes to that net's store slot and the search is skipped when
// pass_result[0] < 0, i.e. an earlier step of the pass failed).
struct Job {
  ogr_net_args a;
  int32_t* path_out;
  int32_t path_cap;
  int32_t from_pass;
  ogr_net_table t;
  ogr_pass_args pa;
  int32_t k;
  const int64_t* pass_result;
  unsigned long long* stats;
  int32_t gated;   // 1: run only when the tile engine handed the net over
  // multi-source multi-sink search (multi = 1; src / dst unused): distinct
  // seeds start with label seed_cost + penalty and no parent, distinct
  // targets settle but never expand; the result is the target with the least
  // (label + target cost, label, node id).  Device arrays.
  int32_t multi;
  const int32_t* seeds;
  const double* seed_cost;
  int32_t n_seeds;
  const int32_t* targets;
  const double* target_cost;
  int32_t n_targets;
};

size_t workspace_bytes(int32_t num_nodes, int64_t num_edges);

// Device int32[4] the search writes: status, path length, phases, 0.
int32_t* result_words(void* ws, int32_t num_nodes, int64_t num_edges);

// Clears the barrier words and launches the cooperative search on `s`: the
// tile-window engine when it is enabled (tilesearch.cu), followed by the
// phase-settled engine, which runs only for a net the first one handed over.
int launch(const ogr_graph& g, const ogr_state& st, const Job& job, void* ws, cudaStream_t s);

}  // namespace ogr_full

namespace ogr_tile {

bool enabled();
// Scratch of the tile engine (node words, winners, per-tile arrays, control).
size_t workspace_bytes(int32_t num_nodes);
size_t ctl_bytes();
// Launches the tile-window search; res (int32[3]) and *gate (1 = the phase
// engine must search this net) are device words.  OGR_ERR_CAPACITY: the
// lattice does not fit the engine's tiles (nothing launched).
int launch(const ogr_graph& g, const ogr_state& st, const ogr_full::Job& job, void* tws, int32_t* res,
           int32_t* gate, cudaStream_t s);

}  // namespace ogr_tile
