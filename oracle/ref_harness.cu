// ref_harness.cu -- exposes the reference's own host code through a C ABI.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/build.py from the reference
// sources where they lie (the include below is resolved with -I<reference
// root>); the output goes to oracle/_ref/ and is never committed.  Nothing
// here touches a GPU: only host functions of the reference are called, so
// the library runs on a machine without one.
//
// What it pins (file:line in anonymous-artifacts/MISFIT):
//   HybridGraph open/isAdjacent/insert/remove/neighbors_into/degree
//                                  core/FlashGraph.h:21-311
//   batch apply loop               src/misfit_async/misfit_async.cu:722-728
//   get_h_hop_neighborhood         src/misfit_async/misfit_async.cu:153-195
//   parse_batch_file, list_batch_files_sorted   core/cli_setup.h:49-82
//   compact_flash_graph            core/flash_compactor.h:20-105
//   greedy MIS (tools/compute_initial_mis.py) is pinned from Python instead.

#define main misfit_async_reference_main
#include "src/misfit_async/misfit_async.cu"
#undef main

#include <cstdint>
#include <string>
#include <vector>

extern "C" {

void* ref_open(const char* path) {
  HybridGraph* g = new HybridGraph();
  g->open(path);
  return g;
}

void ref_close(void* h) { delete static_cast<HybridGraph*>(h); }

int32_t ref_num_nodes(void* h) { return static_cast<HybridGraph*>(h)->num_nodes; }

uint64_t ref_base_edges(void* h) { return static_cast<HybridGraph*>(h)->base.edges; }

int ref_is_adjacent(void* h, int32_t u, int32_t v) {
  return static_cast<HybridGraph*>(h)->isAdjacent(u, v) ? 1 : 0;
}

// The graph-update half of processBatchGPUVertexClustering, calling the
// reference's own overlay methods.
void ref_apply_updates(void* h, const int32_t* u, const int32_t* v, const uint8_t* ins, int64_t m) {
  HybridGraph& g = *static_cast<HybridGraph*>(h);
  for (int64_t i = 0; i < m; ++i) {
    if (ins[i] && !g.isAdjacent(u[i], v[i])) g.insertEdge(u[i], v[i]);
    else if (!ins[i] && g.isAdjacent(u[i], v[i])) g.removeEdge(u[i], v[i]);
  }
}

int64_t ref_row(void* h, int32_t x, int32_t* out, int64_t cap) {
  std::vector<int> r;
  static_cast<HybridGraph*>(h)->neighbors_into(x, r);
  for (int64_t i = 0; i < (int64_t)r.size() && i < cap; ++i) out[i] = r[i];
  return (int64_t)r.size();
}

int32_t ref_degree(void* h, int32_t x) { return static_cast<HybridGraph*>(h)->degree(x); }

// 2-hop list of s plus the hop-1 vertices whose rows the reference records
// (the candidate-row keys), both in the reference's own order.
int64_t ref_two_hop(void* h, int32_t s, int32_t* out, int64_t cap, int32_t* hop1_out,
                    int64_t hop1_cap, int64_t* hop1_len) {
  HybridGraph* g = static_cast<HybridGraph*>(h);
  vector<char> visited(g->num_nodes, 0);
  vector<int> tracker, cur, next, scratch;
  unordered_map<int, vector<int>> hop1;
  vector<int> list = get_h_hop_neighborhood(s, g, 2, visited, tracker, cur, next, scratch, &hop1);
  for (int64_t i = 0; i < (int64_t)list.size() && i < cap; ++i) out[i] = list[i];
  // The keys of hop1 are exactly the hop-1 frontier; report them sorted.
  vector<int> keys;
  for (auto& kv : hop1) keys.push_back(kv.first);
  std::sort(keys.begin(), keys.end());
  for (int64_t i = 0; i < (int64_t)keys.size() && i < hop1_cap; ++i) hop1_out[i] = keys[i];
  *hop1_len = (int64_t)keys.size();
  return (int64_t)list.size();
}

// parse_batch_file: 1-indexed "u v" lines, range/self-loop filter, flag
// is_insertion = !isAdjacent against the graph as it is now.
int64_t ref_parse_batch_file(void* h, const char* path, int32_t* u, int32_t* v, uint8_t* ins,
                             int64_t cap) {
  HybridGraph* g = static_cast<HybridGraph*>(h);
  std::vector<EdgeUpdate> b = parse_batch_file(std::filesystem::path(path), *g, g->num_nodes);
  for (int64_t i = 0; i < (int64_t)b.size() && i < cap; ++i) {
    u[i] = b[i].u;
    v[i] = b[i].v;
    ins[i] = b[i].is_insertion ? 1 : 0;
  }
  return (int64_t)b.size();
}

// list_batch_files_sorted: writes the sorted file names, '\n'-separated.
int64_t ref_list_batch_files(const char* dir, char* out, int64_t cap) {
  std::string s;
  for (const auto& p : list_batch_files_sorted(dir)) s += p.filename().string() + "\n";
  for (int64_t i = 0; i < (int64_t)s.size() && i < cap; ++i) out[i] = s[i];
  return (int64_t)s.size();
}

void ref_compact(void* h, const char* out_path) {
  HybridGraph* g = static_cast<HybridGraph*>(h);
  compact_flash_graph(g->base, g->delta, out_path);
}

}  // extern "C"
