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
};

size_t workspace_bytes(int32_t num_nodes, int64_t num_edges);

// Device int32[4] the search writes: status, path length, phases, 0.
int32_t* result_words(void* ws, int32_t num_nodes, int64_t num_edges);

// Clears the barrier words and launches the cooperative search on `s`.
int launch(const ogr_graph& g, const ogr_state& st, const Job& job, void* ws, cudaStream_t s);

}  // namespace ogr_full
