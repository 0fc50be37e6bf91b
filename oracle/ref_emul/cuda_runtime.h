// cuda_runtime.h -- host-only stand-in for the CUDA runtime, used to run the
// reference engine's own source on a CPU.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build.py compiles the reference's
// src/misfit/misfit.cu and src/misfit_async/misfit_async.cu with g++ against
// this directory (it shadows the real <cuda_runtime.h>), after rewriting each
// `kernel<<<grid, block, 0, stream>>>(args);` into REFEMUL_LAUNCH(...) in a
// generated copy under oracle/_ref/.  Nothing here runs on a GPU.
//
// What the emulation does:
//  * "device" and pinned allocations are host memory (anonymous mappings,
//    zero-filled, so uninitialised device memory reads as zero);
//  * every copy, memset and synchronisation is immediate, so a stream is the
//    program order of the host thread;
//  * a kernel launch runs its threads one after another, block by block and
//    thread by thread in ascending order, each to completion.  With that
//    order the reference's atomic head insertion (misfit.cu:271-273) builds
//    every cluster list in ascending edge index, and process_clusters_csr
//    runs the clusters in ascending id (misfit.cu:277-349);
//  * vertex_clustering_csr_kernel (misfit.cu:219-259), the one kernel whose
//    result depends on how its threads interleave, runs under a selectable
//    schedule (refemul::g_schedule):
//      kBulkSynchronous -- every thread reads the cluster ids as they were
//        before the launch, then the threads' writes land in ascending thread
//        order (the highest thread index writes each element last).  New ids
//        come from the atomic counter in ascending thread order.  The
//        unmodified kernel body runs once per thread against a private copy of
//        the pre-launch node array; the copy tells which id the thread chose,
//        and its writes are then applied to the real array in thread order.
//      kSerial -- each thread runs to completion before the next starts, so a
//        thread sees every earlier thread's writes (and may return early
//        because of them).
#pragma once

#include <sys/mman.h>

#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __align__(n) alignas(n)

typedef int cudaError_t;
enum : int { cudaSuccess = 0 };
enum cudaMemcpyKind {
  cudaMemcpyHostToHost = 0,
  cudaMemcpyHostToDevice = 1,
  cudaMemcpyDeviceToHost = 2,
  cudaMemcpyDeviceToDevice = 3,
  cudaMemcpyDefault = 4
};
enum : unsigned { cudaHostAllocDefault = 0, cudaHostAllocMapped = 2 };
struct refemul_stream_tag {};
struct refemul_event_tag {};
typedef refemul_stream_tag* cudaStream_t;
typedef refemul_event_tag* cudaEvent_t;

struct cudaDeviceProp {
  char name[256];
  int multiProcessorCount;
  int maxThreadsPerMultiProcessor;
  int integrated;
  size_t totalGlobalMem;
};

struct refemul_dim3 {
  unsigned int x = 0, y = 1, z = 1;
};
inline refemul_dim3 blockIdx, threadIdx, blockDim, gridDim;

namespace refemul {

// ---- memory ---------------------------------------------------------------

inline std::mutex g_mem_mu;
inline std::unordered_map<void*, size_t> g_maps;

inline void* alloc_zeroed(size_t bytes) {
  const size_t len = bytes ? bytes : 1;
  void* p = mmap(nullptr, len, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
  if (p == MAP_FAILED) return nullptr;
  std::lock_guard<std::mutex> lk(g_mem_mu);
  g_maps[p] = len;
  return p;
}

inline void release(void* p) {
  if (!p) return;
  size_t len = 0;
  {
    std::lock_guard<std::mutex> lk(g_mem_mu);
    auto it = g_maps.find(p);
    if (it == g_maps.end()) return;
    len = it->second;
    g_maps.erase(it);
  }
  munmap(p, len);
}

// ---- kernel launches ------------------------------------------------------

enum Schedule : int { kBulkSynchronous = 0, kSerial = 1 };
inline Schedule g_schedule = kBulkSynchronous;

// What the launches of one sub-batch showed (filled in launch order).
struct SubBatchRecord {
  long long rows = -1;      // build_vertex_map_kernel: num_vertices
  long long clusters = -1;  // *cluster_count after vertex_clustering_csr_kernel
  long long edges = -1;     // assign_edges_to_clusters_kernel: num_edges
};
inline std::vector<SubBatchRecord> g_records;
inline long long g_num_nodes = 0;   // node count of the engine being driven (from init_nodes_kernel)
inline long long g_launches = 0;

template <class F>
inline void run_thread(long long b, long long t, F& body) {
  blockIdx.x = (unsigned)b;
  threadIdx.x = (unsigned)t;
  body();
}

template <class F>
inline void run_all(long long grid, long long block, F& body) {
  for (long long b = 0; b < grid; ++b)
    for (long long t = 0; t < block; ++t) run_thread(b, t, body);
}

// vertex_clustering_csr_kernel(mapped, num_vertices, offsets, elements,
// nodes, clusters, cluster_count) under the bulk-synchronous schedule.
// `nodes` is the caller's own pointer variable (the launch argument, bound
// by reference), so the body sees the private copy while it runs.
template <class F, class Nodes>
inline void clustering_bulk_synchronous(long long grid, long long block, F& body, const int* mapped,
                                        long long num_vertices, const long long* offsets, const int* elements,
                                        Nodes*& nodes, long long num_nodes) {
  Nodes* live = nodes;
  std::vector<Nodes> before(live, live + num_nodes);   // state at launch
  std::vector<Nodes> priv(before);                     // what every thread reads
  std::vector<std::pair<long long, int>> chosen;       // (thread, id written)
  nodes = priv.data();
  for (long long b = 0; b < grid; ++b) {
    for (long long t = 0; t < block; ++t) {
      const long long tid = b * block + t;
      run_thread(b, t, body);
      if (tid >= num_vertices) continue;
      const long long s = offsets[tid], e = offsets[tid + 1];
      if (before[mapped[tid]].cluster_id != -1 || s == e) continue;   // returned early / wrote nothing
      chosen.emplace_back(tid, priv[elements[s]].cluster_id);
      for (long long i = s; i < e; ++i) priv[elements[i]] = before[elements[i]];
    }
  }
  nodes = live;
  for (const auto& c : chosen)
    for (long long i = offsets[c.first]; i < offsets[c.first + 1]; ++i) live[elements[i]].cluster_id = c.second;
}

template <class F, class Args>
inline void launch(const char* name, long long grid, long long block, F&& body, Args&& args) {
  using T = std::remove_reference_t<Args>;
  constexpr size_t N = std::tuple_size<T>::value;
  ++g_launches;
  gridDim.x = (unsigned)grid;
  blockDim.x = (unsigned)block;
  if constexpr (N == 2) {   // init_nodes_kernel(nodes, num_nodes): the engine's constructor
    if (std::strcmp(name, "init_nodes_kernel") == 0) g_num_nodes = (long long)std::get<1>(args);
  }
  if constexpr (N == 3) {   // build_vertex_map_kernel: a sub-batch starts
    if (std::strcmp(name, "build_vertex_map_kernel") == 0) {
      g_records.emplace_back();
      g_records.back().rows = (long long)std::get<1>(args);
    }
  }
  if constexpr (N == 7) {   // vertex_clustering_csr_kernel
    if (std::strcmp(name, "vertex_clustering_csr_kernel") == 0) {
      if (g_schedule == kBulkSynchronous)
        clustering_bulk_synchronous(grid, block, body, std::get<0>(args), (long long)std::get<1>(args),
                                    std::get<2>(args), std::get<3>(args), std::get<4>(args), g_num_nodes);
      else
        run_all(grid, block, body);
      if (!g_records.empty()) g_records.back().clusters = *std::get<6>(args);
      return;
    }
  }
  run_all(grid, block, body);
  if constexpr (N == 5) {   // assign_edges_to_clusters_kernel
    if (std::strcmp(name, "assign_edges_to_clusters_kernel") == 0 && !g_records.empty())
      g_records.back().edges = (long long)std::get<1>(args);
  }
}

// Seed set of a sub-batch with first-appearance iteration order.  It stands
// in for the reference's std::unordered_set<int> (misfit.cu:495), whose
// iteration order the language leaves unspecified; the interface is the
// part the engine uses (find/end/insert/count/begin).
class FirstAppearanceSet {
 public:
  using const_iterator = std::vector<int>::const_iterator;
  const_iterator begin() const { return order_.begin(); }
  const_iterator end() const { return order_.end(); }
  const_iterator find(int x) const {
    auto it = pos_.find(x);
    return it == pos_.end() ? order_.end() : order_.begin() + (std::ptrdiff_t)it->second;
  }
  size_t count(int x) const { return pos_.count(x); }
  size_t size() const { return order_.size(); }
  void insert(int x) {
    if (pos_.emplace(x, order_.size()).second) order_.push_back(x);
  }

 private:
  std::vector<int> order_;
  std::unordered_map<int, size_t> pos_;
};

}  // namespace refemul

#define REFEMUL_LAUNCH(kernel, grid, block, ...) \
  ::refemul::launch(#kernel, (long long)(grid), (long long)(block), [&]() { kernel(__VA_ARGS__); }, \
                    std::forward_as_tuple(__VA_ARGS__))

// ---- runtime API subset used by the reference engines ----------------------

inline const char* cudaGetErrorString(cudaError_t) { return "no error (host emulation)"; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline cudaError_t cudaSetDevice(int) { return cudaSuccess; }
inline cudaError_t cudaFree(void* p) {
  refemul::release(p);
  return cudaSuccess;
}
inline cudaError_t cudaFreeHost(void* p) { return cudaFree(p); }
template <class T>
inline cudaError_t cudaMalloc(T** p, size_t bytes) {
  *p = static_cast<T*>(refemul::alloc_zeroed(bytes));
  return cudaSuccess;
}
template <class T>
inline cudaError_t cudaMallocHost(T** p, size_t bytes) {
  return cudaMalloc(p, bytes);
}
template <class T>
inline cudaError_t cudaHostAlloc(T** p, size_t bytes, unsigned) {
  return cudaMalloc(p, bytes);
}
template <class T>
inline cudaError_t cudaHostGetDevicePointer(T** d, void* h, unsigned) {
  *d = static_cast<T*>(h);
  return cudaSuccess;
}
inline cudaError_t cudaMemset(void* p, int v, size_t bytes) {
  std::memset(p, v, bytes);
  return cudaSuccess;
}
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t bytes, cudaMemcpyKind) {
  if (bytes) std::memmove(d, s, bytes);
  return cudaSuccess;
}
inline cudaError_t cudaMemcpyAsync(void* d, const void* s, size_t bytes, cudaMemcpyKind k, cudaStream_t = nullptr) {
  return cudaMemcpy(d, s, bytes, k);
}
inline cudaError_t cudaStreamCreate(cudaStream_t* s) {
  static refemul_stream_tag tag;
  *s = &tag;
  return cudaSuccess;
}
inline cudaError_t cudaStreamDestroy(cudaStream_t) { return cudaSuccess; }
inline cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaEventCreate(cudaEvent_t* e) {
  static refemul_event_tag tag;
  *e = &tag;
  return cudaSuccess;
}
inline cudaError_t cudaEventDestroy(cudaEvent_t) { return cudaSuccess; }
inline cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t = nullptr) { return cudaSuccess; }
inline cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
inline cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t, cudaEvent_t) {
  *ms = 0.0f;
  return cudaSuccess;
}
inline cudaError_t cudaMemGetInfo(size_t* free_bytes, size_t* total_bytes) {
  *free_bytes = (size_t)1 << 40;
  *total_bytes = (size_t)1 << 40;
  return cudaSuccess;
}
inline cudaError_t cudaGetDeviceProperties(cudaDeviceProp* p, int) {
  std::memset(p, 0, sizeof(*p));
  std::strcpy(p->name, "host emulation");
  p->multiProcessorCount = 1;
  p->maxThreadsPerMultiProcessor = 1;
  p->integrated = 0;
  p->totalGlobalMem = (size_t)1 << 40;
  return cudaSuccess;
}
inline int atomicAdd(int* p, int v) {
  const int old = *p;
  *p = old + v;
  return old;
}
inline int atomicExch(int* p, int v) {
  const int old = *p;
  *p = v;
  return old;
}
