// ref_emul.cpp -- the reference engine's own source, run on a CPU.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build.py generates REFEMUL_SOURCE under
// oracle/_ref/ from the reference's src/misfit/misfit.cu or
// src/misfit_async/misfit_async.cu (read where they lie, never copied into
// the repository) and compiles this file against it with g++; the library
// goes to oracle/_ref/.  The generated copy differs from the reference file
// only in:
//   * each `kernel<<<grid, block, 0, stream>>>(args);` is written as
//     REFEMUL_LAUNCH(kernel, grid, block, args); -- a launch that runs the
//     unmodified kernel body thread by thread (cuda_runtime.h here);
//   * with the canonical orders on (the default), the sub-batch seed set
//     `unordered_set<int> unique_vertices` (misfit.cu:495) iterates in first
//     appearance order and `unordered_map<int, vector<int>> candidate_rows`
//     (misfit.cu:550) in ascending vertex id.  Both containers leave their
//     iteration order unspecified; these are the orders the oracle and the
//     GPU library pin.
// Everything else -- overlay, parse-time flags, the split rule and its
// estimate, get_h_hop_neighborhood, row packing and MAX_CSR_ELEMENTS growth,
// the six kernels, the final-MIS file and the compaction -- is the
// reference's code as written.
//
// Exposed through a C ABI:
//   re_main            the engine's own main() (the 5-argument CLI)
//   re_open ... re_close  one HybridGraph + GPUVertexClusteringGraph driven a
//                      batch at a time through processBatchGPUVertexClustering
//                      (sync engine only), with the membership, the cluster
//                      ids, MAX_CSR_ELEMENTS and each sub-batch's edges, rows
//                      and cluster count read back after every batch.

// Every standard header the engines include comes first, so that the access
// override below reaches only the engine's own classes.
#include <malloc.h>
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <queue>
#include <sstream>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "cuda_runtime.h"

#define private public
#define main refemul_reference_main
#include REFEMUL_SOURCE
#undef main
#undef private

extern "C" {

int re_main(int argc, char** argv) { return refemul_reference_main(argc, argv); }

// 0 = bulk-synchronous clustering (the oracle's and the library's schedule),
// 1 = serial clustering (each thread sees the earlier threads' writes).
void re_set_schedule(int s) {
  refemul::g_schedule = s == 1 ? refemul::kSerial : refemul::kBulkSynchronous;
}

long long re_launches() { return refemul::g_launches; }

#ifdef REFEMUL_FINE_API

struct RefEngine {
  HybridGraph graph;
  GPUVertexClusteringGraph* gpu = nullptr;
  std::vector<refemul::SubBatchRecord> last;
};

void* re_open(const char* egr, long long max_csr) {
  RefEngine* r = new RefEngine();
  r->graph.open(egr);
  r->gpu = new GPUVertexClusteringGraph(r->graph.num_nodes, max_csr);
  return r;
}

void re_close(void* h) {
  RefEngine* r = static_cast<RefEngine*>(h);
  delete r->gpu;
  delete r;
}

int re_num_nodes(void* h) { return static_cast<RefEngine*>(h)->graph.num_nodes; }

void re_set_mis(void* h, const uint8_t* mis) {
  RefEngine* r = static_cast<RefEngine*>(h);
  std::vector<bool> m((size_t)r->graph.num_nodes);
  for (size_t i = 0; i < m.size(); ++i) m[i] = mis[i] != 0;
  r->gpu->setMISFromHost(m);
}

// One batch through processBatchGPUVertexClustering (misfit.cu:704-730):
// the conditional overlay apply, then every sub-batch.  Returns the number
// of sub-batches.
long long re_apply_batch(void* h, const int32_t* u, const int32_t* v, const uint8_t* ins, long long m) {
  RefEngine* r = static_cast<RefEngine*>(h);
  std::vector<Edge> batch;
  batch.reserve((size_t)m);
  for (long long i = 0; i < m; ++i) batch.emplace_back(u[i], v[i], ins[i] != 0);
  refemul::g_records.clear();
  refemul::g_num_nodes = r->graph.num_nodes;
  DetailedTimings t;
  processBatchGPUVertexClustering(batch, r->graph, *r->gpu, 2, t);
  r->last = refemul::g_records;
  return (long long)r->last.size();
}

// out = {edges, rows, clusters} of sub-batch i of the last batch.
int re_sub_batch(void* h, long long i, long long* out) {
  RefEngine* r = static_cast<RefEngine*>(h);
  if (i < 0 || i >= (long long)r->last.size()) return -1;
  out[0] = r->last[(size_t)i].edges;
  out[1] = r->last[(size_t)i].rows;
  out[2] = r->last[(size_t)i].clusters;
  return 0;
}

void re_get_mis(void* h, uint8_t* out) {
  RefEngine* r = static_cast<RefEngine*>(h);
  std::vector<bool> m = r->gpu->getMISToHost();
  for (size_t i = 0; i < m.size(); ++i) out[i] = m[i] ? 1 : 0;
}

void re_get_cluster_ids(void* h, int32_t* out) {
  RefEngine* r = static_cast<RefEngine*>(h);
  for (int i = 0; i < r->graph.num_nodes; ++i) out[i] = r->gpu->d_nodes[i].cluster_id;
}

long long re_max_csr(void* h) { return static_cast<RefEngine*>(h)->gpu->MAX_CSR_ELEMENTS; }

int re_degree(void* h, int x) { return static_cast<RefEngine*>(h)->graph.degree(x); }

#endif  // REFEMUL_FINE_API

}  // extern "C"
