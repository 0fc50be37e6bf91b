// mf_internal.cuh -- shared declarations of libmisfit_gb (not installed).
//
// Device layout of one graph context (all in HBM):
//   base CSR     nindex int64[n+1], nlist int32[E]    (both .egr layouts are
//                widened to int64 offsets on upload)
//   live bits    uint32[(E+31)/32]: bit k clear <=> base entry k is tombstoned
//   dead[n]      cleared base entries per row, rcnt[n] tombstone-set sizes
//   added CSR    aoff int64[n+1], aadj/aown int32[A]: added neighbours per
//                vertex in insertion order (the DeltaOverlay's vectors)
//   deg[n]       DeltaOverlay::degree (base - |tombstones| + |added|)
//   mis[n]       uint8 membership, cid[n] int32 cluster ids (persist across
//                sub-batches like DeviceNode::cluster_id), v2i[n] row map
//   scratch      n-sized epoch-tagged marks and per-batch buffers
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <utility>
#include <string>
#include <vector>

#include "../../include/misfit_gb.h"

namespace mf {

// Fixed sizes of the reference engine (src/misfit/misfit.cu:37,560).
constexpr int64_t kMaxBatchEdges = 1048576;          // MAX_BATCH_SIZE
constexpr int64_t kMaxRows = 2 * kMaxBatchEdges;     // 2*MAX_BATCH_SIZE rows
constexpr int64_t kEstimateWeight = 1000;            // hop_limit 2 estimate
constexpr int kRowBits = 21;                         // row index < 2^21
constexpr uint32_t kRowMask = (1u << kRowBits) - 1;
constexpr uint32_t kMaxEpoch = (1u << (32 - kRowBits)) - 1;

// ---- error handling ------------------------------------------------------

void set_error(const std::string& msg);
const char* get_error();

struct Failure {
  int status;
};

#define MF_CUDA(call)                                                          \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      ::mf::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));     \
      throw ::mf::Failure{e_ == cudaErrorMemoryAllocation ? MF_ENOMEM : MF_ECUDA}; \
    }                                                                          \
  } while (0)

#define MF_FAIL(status, msg)            \
  do {                                  \
    ::mf::set_error(msg);               \
    throw ::mf::Failure{status};        \
  } while (0)

// Every kernel launch of the library goes through MF_K so that the number of
// launches can be reported (mf_kernel_launches).
extern std::atomic<long long> g_launches;
inline void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
// Every device or pinned-host allocation of the library counts here
// (mf_allocations), so that a caller can check that a call allocated nothing.
extern std::atomic<long long> g_allocs;
inline void note_alloc() { g_allocs.fetch_add(1, std::memory_order_relaxed); }
// Per-kernel timing (MISFIT_GB_KTIME=1): the device is synchronised around
// every launch and the host-timed milliseconds are summed per kernel name and
// printed to stderr at exit.  Off by default; it slows everything down and is
// only a breakdown tool.
bool ktime_on();
double ktime_begin();
void ktime_end(const char* launch_text, double t0);

#define MF_K(...)                                              \
  do {                                                         \
    const bool kt_ = ::mf::ktime_on();                         \
    const double t_ = kt_ ? ::mf::ktime_begin() : 0.0;         \
    __VA_ARGS__;                                               \
    ::mf::note_launch();                                       \
    if (kt_) ::mf::ktime_end(#__VA_ARGS__, t_);                \
  } while (0)

// ---- programmatic dependent launch -----------------------------------------
// The kernels of a sub-batch form one long chain on the context's stream.
// Launched with launch_pdl, a kernel's CTAs may be scheduled while its
// predecessor's last CTAs still run; they stop at pdl_wait() (PTX
// griddepcontrol.wait), which returns once every prerequisite grid has
// completed and its memory writes are visible.  So a kernel launched this way
// must call pdl_wait() before it touches anything its predecessor writes; the
// kernels that do call it first.  In a kernel launched the ordinary way it
// returns at once.  MISFIT_GB_PDL=0 turns the attribute off.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// Lets the next kernel of the chain be scheduled once every CTA of this one
// has executed it (its CTAs then wait in pdl_wait for this grid to finish).
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

bool pdl_on();

template <typename... KArgs, typename... Args>
void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl_on() ? 1 : 0;
  MF_CUDA(cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...));
}

// Stages timed by the optional profiler (mf_profile_enable).
enum Stage : int {
  kStOverlay = 0,   // batch apply to the overlay
  kStSplit,         // previous-occurrence sort + split rule
  kStSeeds,         // seed compaction
  kStHop1,          // hop-1 marking + candidates
  kStSizes,         // packed-size upper bound
  kStFirst,         // clustering read pass (first existing ids, row decisions)
  kStPush,          // clustering write pass (2-hop max pushes, finalize)
  kStAssign,        // assignment + ordering sort
  kStRepair,        // MIS repair: evaluation rounds and commits
  kStClear,         // clear of mapped vertices
  kStExact,         // exact 2-hop sizes (heavy bitmaps) and limit growth
  kStRepairBig,     // MIS repair: grid-wide hop-2 searches
  kStPushHop,       // the k_lb_push_hop launches alone (part of the clustering write)
  kStFirstNeed,     // clustering read, seeds without an id in their own row (the hop-2 part)
  kStPull,          // clustering write, the candidate rows' ids (pull or push + finalize)
  kStCount
};
extern const char* const kStageNames[kStCount];

// ---- device buffers ------------------------------------------------------

// Stream the calling thread's context works on (set by the entry points,
// cleared when they return).  Device buffers are allocated and freed in that
// stream's order, so growing a buffer does not synchronise the whole device
// (which would stall the other contexts' streams); with no stream set they
// use cudaMalloc / cudaFree.
extern thread_local cudaStream_t g_alloc_stream;

template <typename T>
struct DBuf {
  T* p = nullptr;
  int64_t cap = 0;
  cudaStream_t s = nullptr;   // stream p was allocated on (stream-ordered), or null
  void reserve(int64_t count) {
    if (count <= cap) return;
    release();
    int64_t c = count < 16 ? 16 : count;
    if (g_alloc_stream) {
      note_alloc();
      MF_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&p), sizeof(T) * (size_t)c, g_alloc_stream));
      s = g_alloc_stream;
    } else {
      note_alloc();
      MF_CUDA(cudaMalloc(&p, sizeof(T) * (size_t)c));
    }
    cap = c;
  }
  void release() {
    if (p) {
      if (s) cudaFreeAsync(p, s);
      else cudaFree(p);
    }
    p = nullptr;
    cap = 0;
    s = nullptr;
  }
};

struct AsyncQueue;   // mf_api.cu

// Entries past the end of the row array (nlist): bulk copies start on the
// 16-byte boundary at or below a span and end on the one at or above it, so
// they may read up to 12 bytes beyond the last entry.
constexpr int64_t kNlistPad = 4;

// ---- read-only view of the current graph ----------------------------------

struct GraphView {
  int32_t n;
  const int64_t* nindex;
  const int32_t* nlist;
  const uint32_t* live;
  const int32_t* dead;
  const int64_t* aoff;
  const int32_t* aadj;
};

__device__ __forceinline__ bool live_at(const uint32_t* live, int64_t k) {
  return (__ldg(live + (k >> 5)) >> (k & 31)) & 1u;
}

// Length of the overlay row of x (what neighbors_into returns).
__device__ __forceinline__ int64_t row_len(const GraphView& g, int32_t x) {
  return (g.nindex[x + 1] - g.nindex[x]) - g.dead[x] + (g.aoff[x + 1] - g.aoff[x]);
}

// Calls f(y) for every y of row(x) in order; stops when f returns true.
// Returns true if stopped early.
template <class F>
__device__ __forceinline__ bool thread_row_until(const GraphView& g, int32_t x, F f) {
  const int64_t b = g.nindex[x], e = g.nindex[x + 1];
  if (g.dead[x] == 0) {
    for (int64_t k = b; k < e; ++k)
      if (f(__ldg(g.nlist + k))) return true;
  } else {
    for (int64_t k = b; k < e; ++k)
      if (live_at(g.live, k) && f(__ldg(g.nlist + k))) return true;
  }
  const int64_t ab = g.aoff[x], ae = g.aoff[x + 1];
  for (int64_t k = ab; k < ae; ++k)
    if (f(g.aadj[k])) return true;
  return false;
}

// Warp-cooperative: first element y of row(x) (in order) with pred(y),
// returned in *hit; false when none.  All lanes must call it.
template <class P>
__device__ __forceinline__ bool warp_row_first(const GraphView& g, int32_t x, P pred, int32_t* hit) {
  const int lane = threadIdx.x & 31;
  const int64_t b = g.nindex[x], e = g.nindex[x + 1];
  const bool filt = g.dead[x] != 0;
  for (int64_t k0 = b; k0 < e; k0 += 32) {
    const int64_t k = k0 + lane;
    int32_t y = -1;
    bool ok = false;
    if (k < e) {
      y = __ldg(g.nlist + k);
      ok = (!filt || live_at(g.live, k)) && pred(y);
    }
    const unsigned m = __ballot_sync(0xffffffffu, ok);
    if (m) {
      *hit = __shfl_sync(0xffffffffu, y, __ffs(m) - 1);
      return true;
    }
  }
  const int64_t ab = g.aoff[x], ae = g.aoff[x + 1];
  for (int64_t k0 = ab; k0 < ae; k0 += 32) {
    const int64_t k = k0 + lane;
    int32_t y = -1;
    bool ok = false;
    if (k < ae) {
      y = g.aadj[k];
      ok = pred(y);
    }
    const unsigned m = __ballot_sync(0xffffffffu, ok);
    if (m) {
      *hit = __shfl_sync(0xffffffffu, y, __ffs(m) - 1);
      return true;
    }
  }
  return false;
}

// Warp-cooperative for-each over row(x) (no order guarantee between lanes).
template <class F>
__device__ __forceinline__ void warp_row_each(const GraphView& g, int32_t x, F f) {
  const int lane = threadIdx.x & 31;
  const int64_t b = g.nindex[x], e = g.nindex[x + 1];
  const bool filt = g.dead[x] != 0;
  for (int64_t k = b + lane; k < e; k += 32)
    if (!filt || live_at(g.live, k)) f(__ldg(g.nlist + k));
  const int64_t ab = g.aoff[x], ae = g.aoff[x + 1];
  for (int64_t k = ab + lane; k < ae; k += 32) f(g.aadj[k]);
}

// Load-balanced traversal of the rows of list[0..cnt): offs is the exclusive
// prefix of the row position counts (base positions + added entries; a
// count of 0 skips the row), cnt+1 entries.  f(i, x, y, aux) is called for
// every live element y of row(x = list[i]); aux(i, x) is evaluated once per
// visited row (a per-row value such as the row's push tag).
//
// Every warp owns one contiguous span of positions (the total split evenly
// over the grid's warps), so a hub row is spread over many warps and the
// work per warp is even.  The warp finds the row of its first position once,
// with a 32-way cooperative search over offs, then walks its span 32 rows at
// a time: the rows' ends and metadata (base offset, length, added offset,
// tombstone flag, aux) are loaded in one round of parallel loads into shared
// memory; each lane then maps its position to its row with at most five
// shared-memory probes (none when the whole 32-position window lies in one
// row) and the element loads of four windows are issued before any is used.
// Kernels that call it run blocks of kLbThreads threads.
// Compile-time knobs of the traversal (defaults are the measured best):
// windows loaded before any is used, and the minimum resident blocks per SM
// the traversal kernels are compiled for (1: no register cap).
#ifndef MF_LB_UNROLL
#define MF_LB_UNROLL 4
#endif
#ifndef MF_LB_MIN_BLOCKS
#define MF_LB_MIN_BLOCKS 1
#endif
constexpr int kLbThreads = 256;
constexpr int kLbWarps = kLbThreads / 32;
constexpr int kLbUnroll = MF_LB_UNROLL;

struct LbStage {
  int64_t end[32];    // end position (exclusive) of staged row k
  int64_t b0[32];     // nindex[x]
  int64_t a0[32];     // aoff[x]
  int32_t x[32];
  int32_t nb[32];     // base positions of row(x)
  uint32_t aux[32];
  int64_t start;      // start position of staged row 0
  uint32_t filt;      // bit k: row k has tombstoned base entries
};

struct NoAux {
  __device__ __forceinline__ uint32_t operator()(int64_t, int32_t) const { return 0u; }
};

template <class A, class F>
__device__ __forceinline__ int64_t lb_rows_aux(const GraphView& g, const int32_t* list, const int64_t* offs, int64_t cnt,
                                               A aux, F f) {
  __shared__ LbStage lb_stage[kLbWarps];
  const int lane = threadIdx.x & 31;
  LbStage& st = lb_stage[(threadIdx.x >> 5) & (kLbWarps - 1)];
  const int64_t total = offs[cnt];
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t per = (((total + nwarps - 1) / nwarps) + 31) & ~(int64_t)31;
  int64_t pos = w * per;
  const int64_t stop = pos + per < total ? pos + per : total;
  if (pos >= stop) return 0;
  // the row holding pos: offs[lo] <= pos < offs[hi]
  int64_t lo = 0, hi = cnt;
  while (hi - lo > 1) {
    const int64_t step = (hi - lo + 31) >> 5;
    const int64_t idx = lo + (int64_t)lane * step;
    const bool le = idx < hi && offs[idx] <= pos;
    const unsigned m = __ballot_sync(0xffffffffu, le);
    const int k = 31 - __clz(m);
    lo += (int64_t)k * step;
    const int64_t nh = lo + step;
    hi = nh < hi ? nh : hi;
  }
  int64_t ri = lo;
  int64_t visited = 0;
  while (pos < stop) {
    // stage rows ri .. ri+31
    __syncwarp();
    const int64_t r = ri + lane;
    int64_t e = total, b0 = 0, a0 = 0;
    int32_t x = 0, nb = 0;
    bool tomb = false;
    uint32_t av = 0;
    if (r < cnt) {
      const int64_t s0 = offs[r];
      e = offs[r + 1];
      if (lane == 0) st.start = s0;
      if (e > s0) {
        x = list[r];
        b0 = g.nindex[x];
        nb = (int32_t)(g.nindex[x + 1] - b0);
        a0 = g.aoff[x];
        tomb = g.dead[x] != 0;
        av = aux(r, x);
      }
    }
    st.end[lane] = e;
    st.b0[lane] = b0;
    st.a0[lane] = a0;
    st.x[lane] = x;
    st.nb[lane] = nb;
    st.aux[lane] = av;
    const unsigned fm = __ballot_sync(0xffffffffu, tomb);
    if (lane == 0) st.filt = fm;
    __syncwarp();
    const int64_t last = st.end[31];
    const int64_t cover = last < stop ? last : stop;
    for (; pos < cover; pos += 32 * kLbUnroll) {
      // first staged row that ends after pos (the ends are sorted)
      const int kb = __popc(__ballot_sync(0xffffffffu, st.end[lane] <= pos));
      int32_t yv[kLbUnroll];
      int kr[kLbUnroll];
      bool ok[kLbUnroll];
#pragma unroll
      for (int q = 0; q < kLbUnroll; ++q) {
        const int64_t wbase = pos + 32 * q;
        const int64_t p = wbase + lane;
        ok[q] = false;
        kr[q] = 0;
        yv[q] = 0;
        if (p < cover) {
          int k = kb;
          if (st.end[kb] <= wbase + 31) {
            int l = kb, h = 31;
            while (l < h) {
              const int mid = (l + h) >> 1;
              if (st.end[mid] > p) h = mid; else l = mid + 1;
            }
            k = l;
          }
          const int64_t rs = k == 0 ? st.start : st.end[k - 1];
          const int64_t j = p - rs;
          const int32_t nbk = st.nb[k];
          if (j < nbk) {
            const int64_t gk = st.b0[k] + j;
            yv[q] = __ldg(g.nlist + gk);
            ok[q] = !((st.filt >> k) & 1u) || live_at(g.live, gk);
          } else {
            yv[q] = g.aadj[st.a0[k] + (j - nbk)];
            ok[q] = true;
          }
          kr[q] = k;
        }
      }
#pragma unroll
      for (int q = 0; q < kLbUnroll; ++q) {
        if (ok[q]) {
          ++visited;
          f(ri + kr[q], st.x[kr[q]], yv[q], st.aux[kr[q]]);
        }
      }
    }
    pos = cover;
    ri += 32;
  }
  return visited;
}

template <class F>
__device__ __forceinline__ int64_t lb_rows(const GraphView& g, const int32_t* list, const int64_t* offs, int64_t cnt,
                                           F f) {
  return lb_rows_aux(g, list, offs, cnt, NoAux{},
                     [&](int64_t i, int32_t x, int32_t y, uint32_t) { f(i, x, y); });
}

__device__ __forceinline__ int64_t row_positions(const GraphView& g, int32_t x) {
  return (g.nindex[x + 1] - g.nindex[x]) + (g.aoff[x + 1] - g.aoff[x]);
}

// Element k of row(x) (base positions first, then added), or -1 if tombstoned.
__device__ __forceinline__ int32_t row_elem(const GraphView& g, int32_t x, int64_t k, int64_t nb) {
  if (k < nb) {
    const int64_t gk = g.nindex[x] + k;
    if (g.dead[x] != 0 && !live_at(g.live, gk)) return -1;
    return g.nlist[gk];
  }
  return g.aadj[g.aoff[x] + (k - nb)];
}

// As lb_rows, with the row position j of y passed too; positions start at
// `skip` (offs counts the positions from `skip` on).  f(i, x, y, j).
template <class F>
__device__ __forceinline__ void lb_rows_pos(const GraphView& g, const int32_t* list, const int64_t* offs, int64_t cnt,
                                            int64_t skip, F f) {
  constexpr int64_t kChunk = 256;
  const int64_t total = offs[cnt];
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kChunk; base < total;
       base += nwarps * kChunk) {
    int64_t i = 0;
    if (lane == 0) {
      int64_t lo = 0, hi = cnt;
      while (hi - lo > 1) {
        const int64_t mid = (lo + hi) >> 1;
        if (offs[mid] <= base) lo = mid; else hi = mid;
      }
      i = lo;
    }
    i = __shfl_sync(0xffffffffu, i, 0);
    const int64_t end = base + kChunk < total ? base + kChunk : total;
    int64_t cur = -1, next_off = 0, row_off = 0, nb = 0;
    int32_t x = 0;
    for (int64_t e = base + lane; e < end; e += 32) {
      if (cur < 0 || e >= next_off) {
        while (offs[i + 1] <= e) ++i;
        cur = i;
        x = list[i];
        row_off = offs[i];
        next_off = offs[i + 1];
        nb = g.nindex[x + 1] - g.nindex[x];
      }
      const int64_t j = e - row_off + skip;
      const int32_t y = row_elem(g, x, j, nb);
      if (y >= 0) f(i, x, y, j);
    }
  }
}

// ---- primitives (mf_prims.cu) -----------------------------------------------

struct Scratch;  // workspace for primitives

// out[i] = sum_{j<i} in[j] for i in [0, n]; out has n+1 entries (out[n] = total).
void scan_exclusive_i64(const int64_t* in, int64_t* out, int64_t n, Scratch& ws, cudaStream_t s);
void scan_exclusive_i32(const int32_t* in, int64_t* out, int64_t n, Scratch& ws, cudaStream_t s);
void scan_exclusive_u8(const uint8_t* in, int64_t* out, int64_t n, Scratch& ws, cudaStream_t s);
// Packed scan of the hop-1 marks: high 32 bits count marked vertices, low 32
// bits marked vertices that are not seed rows (v2i < 0).

// Stable LSD radix sort of (key, value) on key bits [0, bits); result in keys/vals.
void radix_sort_pairs(uint64_t* keys, uint32_t* vals, int64_t n, int bits, Scratch& ws, cudaStream_t s);

struct Scratch {
  DBuf<int64_t> block_sums;
  DBuf<int64_t> block_sums2;
  DBuf<int32_t> hist;
  DBuf<int64_t> hist_scan;
  DBuf<uint64_t> keys_alt;
  DBuf<uint32_t> vals_alt;
  DBuf<unsigned long long> scan_status;   // look-back scan: 3 words per tile, tagged with scan_seq
  unsigned long long scan_seq = 0;
  void release() {
    scan_status.release();
    block_sums.release();
    block_sums2.release();
    hist.release();
    hist_scan.release();
    keys_alt.release();
    vals_alt.release();
  }
};

int bits_for(int64_t v);  // number of bits to hold values in [0, v]

}  // namespace mf

// ---- the context --------------------------------------------------------------

struct SubBatchTrace {
  int64_t hdr[10];
  std::vector<int32_t> seeds, cands, cid_after, order;
  std::vector<uint8_t> mis_after;
  std::vector<int64_t> row_len;
};

// Buffers of one sub-batch's "front": its hop-1 set, candidate list and
// packed-size bound.  They depend only on the batch's graph and the planned
// seed list, so the front of the next sub-batch is computed on a second
// stream while the current one clusters and repairs (two sets, alternating).
namespace mf {
struct Front {
  mf::DBuf<uint32_t> bits;                  // hop-1 bitmap, then the seed bitmap
  mf::DBuf<int64_t> bits_sums;              // per-block counts of the bitmap scan
  mf::DBuf<unsigned long long> uacc;        // per-seed sums of the size bound
  mf::DBuf<int32_t> hlist, cands;           // swapped into the context when its sub-batch runs
  mf::DBuf<int64_t> lb_offs;                // row offsets of the seeds
  mf::DBuf<int64_t> cnt;                    // [0] (hop-1 << 32 | candidates), [1] size bound
  mf::Scratch ws;
};
}  // namespace mf

struct mf_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int32_t n = 0;
  int64_t nnz = 0;
  uint64_t header_edges = 0;
  bool rows_sorted = true;
  bool symmetric = false;   // every base entry has its reverse (then every overlay row too)

  mf::DBuf<int64_t> nindex;
  mf::DBuf<int32_t> nlist;
  mf::DBuf<uint32_t> live;
  mf::DBuf<int32_t> dead, rcnt, deg;
  mf::DBuf<int64_t> aoff, aoff_alt;
  mf::DBuf<int32_t> aadj, aown, aadj_alt, aown_alt;
  int64_t a_total = 0;

  mf::DBuf<uint8_t> mis;
  mf::DBuf<int32_t> cid, v2i;
  mf::DBuf<uint32_t> bval, wval;
  mf::DBuf<int32_t> f1;
  uint32_t epoch = 0;

  // batch-sized buffers
  mf::DBuf<int32_t> bu, bv;
  mf::DBuf<uint8_t> bins;
  mf::DBuf<uint64_t> keys;
  mf::DBuf<uint32_t> vals;
  mf::DBuf<int32_t> prev;       // previous edge index per endpoint slot
  mf::DBuf<int64_t> i64a, i64b; // scans
  mf::DBuf<int32_t> i32a, i32b, i32c;
  mf::DBuf<uint8_t> u8a;
  // overlay rebuild
  mf::DBuf<int32_t> acnt_new;
  mf::DBuf<uint8_t> akill;
  mf::DBuf<uint64_t> app_keys;
  mf::DBuf<uint32_t> app_vals;
  // sub-batch buffers
  mf::DBuf<int32_t> seeds, cands, hlist, touched;
  mf::DBuf<int32_t> rowcid;
  mf::DBuf<uint8_t> creates;
  mf::DBuf<int64_t> rowlens;
  // speculative repair
  mf::DBuf<int32_t> rp_w0, rp_w1, rp_n0, rp_n1;
  mf::DBuf<uint64_t> rp_keys, rp_keys2;
  mf::DBuf<uint32_t> rp_vals, rp_vals2;
  mf::DBuf<uint8_t> rp_u8;
  mf::DBuf<int64_t> rp_pos;
  mf::DBuf<int64_t> big_pos, big_off, big_nr, big_chunks, big_pre;
  mf::DBuf<int32_t> big_r;
  mf::DBuf<unsigned long long> big_best;
  int big_grid = 0;
  mf::DBuf<uint32_t> bitmaps;   // per-CTA vertex bitmaps for exact 2-hop sizes
  int64_t bitmap_words = 0;
  int bitmap_ctas = 0;
  mf::DBuf<int32_t> heavy_slot, heavy_list;
  mf::DBuf<uint32_t> heavy_bits;
  int64_t heavy_cap = 0, heavy_used = 0;
  mf::DBuf<uint32_t> dense_bits;      // per dense seed bitmaps (exact sizes)
  mf::DBuf<int64_t> dense_light;      // per dense seed light volume (size bound)
  mf::DBuf<int32_t> pull_long;        // vertices with long rows for the warp pull pass
  mf::DBuf<uint32_t> ncbits;          // non-skipped candidate bits for the pull pass
  // exact 2-hop sizes by row passes: seed masks per vertex and their filter
  // bits, the huge rows' chunk ORs, neighbourhood volumes, chunk tasks, the
  // seed groups, huge-row slots, counters
  mf::DBuf<uint32_t> p2_mask, p2_filt, p2_racc;
  mf::DBuf<int64_t> p2_vol, p2_tasks;
  mf::DBuf<int32_t> p2_grp, p2_huge;
  mf::DBuf<unsigned long long> p2_cnt;
  // sub-batch plan of the current batch: cuts, estimates, seed lists
  mf::DBuf<int64_t> plan_cuts, plan_ests, plan_send, plan_pos;
  mf::DBuf<uint8_t> plan_flags;
  mf::DBuf<int32_t> seeds_all;
  // first-hit chunk queue (rows) and the need seeds' chunk queue
  mf::DBuf<int32_t> rq_idx, rq_v, mq_idx, mq_v;
  mf::DBuf<int64_t> mq_base;
  mf::DBuf<uint8_t> xst, xleave;      // exact-MIS mode: completion states, leave flags
  // batched form (mf_batched.cu): per-vertex engine scratch kept between
  // batches (clustering-write tags, row map = -1, three zero bitmaps), its
  // tag epoch, and the per-batch scratch of one engine item
  mf::DBuf<uint8_t> cta_vert, cta_ws;
  uint32_t cta_epoch = 0;
  bool exact = false;                  // exact-MIS mode on
  mf::Front front[2];                 // current and next sub-batch fronts
  cudaStream_t stream_b = nullptr;    // the fronts of later sub-batches run here
  cudaEvent_t ev_a = nullptr, ev_b = nullptr;
  mf::DBuf<int64_t> n2cache;           // exact 2-hop sizes of this batch's rows
  mf::DBuf<uint32_t> n2stamp;          // batch stamp of each cached size
  mf::DBuf<int64_t> n2bound;           // tighter upper bounds of this batch's 2-hop sizes
  mf::DBuf<uint32_t> n2bstamp;         // batch stamp of each cached bound
  uint32_t n2batch = 0;
  mf::DBuf<int32_t> dense_idx, dense_hl, pair_d, pair_h, todo;
  // per-pass capacities of the push form's dense seeds and light pairs, when
  // lower than the memory-derived ones (MISFIT_GB_EXACT_CAPS=dense,pairs at
  // context creation; 0 = not lowered): small graphs then take the retry path
  int64_t exact_cap_dense = 0, exact_cap_pairs = 0;
  // outcomes of the tighter size bound (bit 0 = last: it settled the
  // sub-batch), how often it ran, and the sub-batches it was skipped on
  uint32_t bound_hist = 0;
  int64_t bound_tries = 0, bound_skips = 0;
  // the candidates' cluster ids, pull or push per sub-batch (tuning
  // cand_push 0): row entries the pull read per vertex in the last batch
  // that pulled on a graph of 2^20 vertices or more (1 before any), and the
  // pull sub-batches of the current batch
  double pull_visit_ratio = 1.0;
  int64_t pull_runs = 0;
  mf::DBuf<unsigned long long> fpos;   // first-hit positions
  mf::DBuf<int32_t> un_idx, un_v, need, needv, live_i, live_v, nlist_need;
  mf::DBuf<uint32_t> nmark;            // epoch marks: neighbours of seeds needing their hop-2 part
  mf::DBuf<int64_t> un_cnt;
  mf::DBuf<int64_t> counters;   // device counters
  int64_t* h_counters = nullptr;  // pinned mirror
  mf::Scratch ws;

  int64_t max_csr = 0;
  mf_batch_stats stats{};
  bool trace = false;
  std::vector<SubBatchTrace> traces;

  // optional per-stage CUDA-event profiling
  int profile = 0;                     // 0 off, 1 all stages, 2 the push_hop and pull stages only
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<std::pair<int, size_t>> ev_marks;
  double stage_ms[mf::kStCount] = {};
  int64_t stage_calls[mf::kStCount] = {};
  // device counters of algorithmic work (elements, rows) per stage
  mf::DBuf<unsigned long long> work;   // 2 * kStCount entries
  double stage_bytes[mf::kStCount] = {};
  mf::DBuf<int64_t> lb_offs;           // row-position prefix for lb_rows
  mf::DBuf<uint32_t> cidbits;          // bit y <=> cid[y] != -1, during the clustering read
  int64_t touched_total = 0;
  int64_t dbg_first[5] = {};           // debug: first-hit calls, rows, warp-level rows, chunk rows, chunks

  // pinned staging for host-input batches
  uint8_t* h_stage = nullptr;
  int64_t h_stage_cap = 0;
  // the pipelined engine: batches enqueued by mf_apply_batch_async run in
  // order on this context's worker thread (made on first use); `pending`
  // counts the ones not yet collected
  mf::AsyncQueue* aq = nullptr;
  bool pending = false;
  // load-balancing settings (mf_set_tuning); they move work between kernels,
  // never a result
  mf_tuning tune = mf_tuning{2048, 2048, 64, 256, 0, 1};

  mf::GraphView view() const {
    return mf::GraphView{n, nindex.p, nlist.p, live.p, dead.p, aoff.p, aadj.p};
  }
};

namespace mf {
// Records a start/end event pair around a stage when profiling is on.
// Calls f(buf) for every device buffer a context owns (graph state,
// per-batch and per-sub-batch scratch, primitive workspace).
template <class F>
void for_each_buffer(mf_ctx* c, F&& f) {
  f(c->nindex); f(c->aoff); f(c->aoff_alt); f(c->i64a); f(c->i64b); f(c->rowlens); f(c->rp_pos);
  f(c->big_pos); f(c->big_off); f(c->big_nr); f(c->big_chunks); f(c->big_pre); f(c->dense_light);
  f(c->plan_cuts); f(c->plan_ests); f(c->plan_send); f(c->plan_pos); f(c->mq_base);
  f(c->n2cache); f(c->n2bound); f(c->un_cnt); f(c->counters); f(c->lb_offs);
  f(c->nlist); f(c->dead); f(c->rcnt); f(c->deg); f(c->aadj); f(c->aown); f(c->aadj_alt); f(c->aown_alt);
  f(c->cid); f(c->v2i); f(c->f1); f(c->bu); f(c->bv); f(c->prev); f(c->i32a); f(c->i32b); f(c->i32c);
  f(c->acnt_new); f(c->seeds); f(c->cands); f(c->hlist); f(c->touched); f(c->rowcid);
  f(c->rp_w0); f(c->rp_w1); f(c->rp_n0); f(c->rp_n1); f(c->big_r); f(c->heavy_slot); f(c->heavy_list);
  f(c->pull_long); f(c->seeds_all); f(c->rq_idx); f(c->rq_v); f(c->mq_idx); f(c->mq_v);
  f(c->dense_idx); f(c->dense_hl); f(c->pair_d); f(c->pair_h); f(c->todo);
  f(c->un_idx); f(c->un_v); f(c->need); f(c->needv); f(c->live_i); f(c->live_v); f(c->nlist_need);
  f(c->live); f(c->bval); f(c->wval); f(c->vals); f(c->app_vals); f(c->rp_vals); f(c->rp_vals2);
  f(c->bitmaps); f(c->heavy_bits); f(c->dense_bits); f(c->ncbits); f(c->n2stamp);
  f(c->n2bstamp); f(c->nmark); f(c->cidbits);
  f(c->mis); f(c->bins); f(c->u8a); f(c->akill); f(c->creates); f(c->rp_u8); f(c->plan_flags);
  f(c->xst); f(c->xleave); f(c->cta_vert); f(c->cta_ws);
  f(c->keys); f(c->app_keys); f(c->rp_keys); f(c->rp_keys2);
  f(c->big_best); f(c->fpos); f(c->work);
  f(c->p2_mask); f(c->p2_filt); f(c->p2_racc); f(c->p2_vol); f(c->p2_tasks); f(c->p2_grp); f(c->p2_huge);
  f(c->p2_cnt);
  f(c->ws.block_sums); f(c->ws.block_sums2); f(c->ws.hist); f(c->ws.hist_scan); f(c->ws.keys_alt);
  f(c->ws.vals_alt); f(c->ws.scan_status);
  for (auto& fr : c->front) {
    f(fr.bits); f(fr.bits_sums); f(fr.uacc); f(fr.hlist); f(fr.cands); f(fr.lb_offs); f(fr.cnt);
    f(fr.ws.block_sums); f(fr.ws.block_sums2); f(fr.ws.hist); f(fr.ws.hist_scan); f(fr.ws.keys_alt);
    f(fr.ws.vals_alt); f(fr.ws.scan_status);
  }
}

// Device bytes a context holds now.
inline int64_t ctx_device_bytes(mf_ctx* c) {
  int64_t total = 0;
  for_each_buffer(c, [&](auto& b) { total += b.cap * (int64_t)sizeof(*b.p); });
  return total;
}

// Frees every device buffer (the stream, events and pinned counters stay) and
// resets the state that lives in them, so that the next use re-creates it.
inline void release_device_state(mf_ctx* c) {
  for_each_buffer(c, [](auto& b) { b.release(); });
  c->bitmap_ctas = 0;
  c->bitmap_words = 0;
  c->heavy_cap = 0;
  c->heavy_used = 0;
  c->epoch = 0;
  c->n2batch = 0;
}

// Frees the per-batch and per-sub-batch scratch but keeps the graph state
// and the n-sized vertex scratch (what a context needs between batches).
inline void release_batch_scratch(mf_ctx* c) {
  const void* keep[] = {&c->nindex, &c->nlist, &c->live, &c->dead, &c->rcnt, &c->deg, &c->aoff, &c->aadj,
                        &c->aown, &c->mis, &c->cid, &c->v2i, &c->bval, &c->wval, &c->f1, &c->nmark,
                        &c->nlist_need, &c->touched, &c->hlist, &c->acnt_new, &c->aoff_alt, &c->counters,
                        &c->cta_vert};
  for_each_buffer(c, [&](auto& b) {
    for (const void* k : keep)
      if (k == static_cast<const void*>(&b)) return;
    b.release();
  });
  c->bitmap_ctas = 0;
  c->bitmap_words = 0;
  c->heavy_cap = 0;
  c->heavy_used = 0;
  c->n2batch = 0;
}

// Pinned host copy of a graph's state (see mf_pool.cu).
struct PinnedSnapshot {
  uint8_t* host = nullptr;
  size_t cap = 0, used = 0;
  std::vector<std::pair<size_t, size_t>> parts;  // (offset, bytes) per saved buffer
};

int64_t snapshot_bytes(const mf_ctx* c);
void evict(mf_ctx* c, PinnedSnapshot& snap);        // device -> pinned host, then frees the device buffers
void restore(mf_ctx* c, const PinnedSnapshot& snap);
void alloc_vertex_scratch(mf_ctx* c);              // n-sized scratch with its initial values (mf_overlay.cu)
void bind_device(const mf_ctx* c);                 // cudaSetDevice(c->device)
double now_ms_host();

struct StageScope {
  mf_ctx* c;
  int stage;
  size_t first = 0;
  bool on;
  StageScope(mf_ctx* ctx, int st)
      : c(ctx), stage(st),
        on((ctx->profile & 3) == 1 || ((ctx->profile & 3) == 2 && (st == kStPushHop || st == kStPull))) {
    if (!on) return;
    if (c->ev_used + 2 > c->ev_pool.size()) {
      for (int k = 0; k < 64; ++k) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) { on = false; return; }
        c->ev_pool.push_back(e);
      }
    }
    first = c->ev_used;
    c->ev_used += 2;
    cudaEventRecord(c->ev_pool[first], c->stream);
  }
  ~StageScope() {
    if (!on) return;
    cudaEventRecord(c->ev_pool[first + 1], c->stream);
    c->ev_marks.emplace_back(stage, first);
  }
};

// mf_overlay.cu
void upload_base(mf_ctx* c, int32_t n, const int64_t* nindex, const int32_t* nlist, int64_t nnz);
void apply_overlay(mf_ctx* c, int64_t m);          // uses c->bu/bv/bins
void flag_updates(mf_ctx* c, int64_t m);           // c->bu/bv -> c->bins
// host u/v -> host ins_out through a fixed device array; m <= MF_NOALLOC_MAX_UPDATES
void flag_updates_noalloc(mf_ctx* c, const int32_t* u, const int32_t* v, int64_t m, uint8_t* ins_out);
void noalloc_refresh(int device);   // scratch address of the no-allocation flags, looked up again
void compact_graph(mf_ctx* c, std::vector<int64_t>& nindex_out, std::vector<int32_t>& nlist_out);
void rebase(mf_ctx* c);
void greedy_mis(mf_ctx* c, uint8_t* d_out);
void check_mis(mf_ctx* c, int64_t* viol, int64_t* uncovered);
void exact_fixup(mf_ctx* c);                       // exact-MIS mode after a batch
// mf_parse.cu: batch file -> c->bu / c->bv (valid lines, file order); returns the count
int64_t parse_batch_file_device(mf_ctx* c, const char* path);
// mf_repair.cu
void process_batch(mf_ctx* c, int64_t m);          // everything after the overlay apply
int64_t initial_max_csr(int32_t n, uint64_t edges);
}  // namespace mf
