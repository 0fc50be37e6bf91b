// mf_scan.cuh -- the library's exclusive scan, as a template over the item
// loader, so that a caller can scan values it computes on the fly (the row
// counts of the load-balanced traversals) without writing them first.
// Included by mf_prims.cu (the plain-array scans) and mf_repair.cu.
#pragma once

#include "mf_internal.cuh"

namespace mf {
namespace scan_detail {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;

template <typename T>
struct Loader {
  const T* p;
  __device__ __forceinline__ int64_t operator()(int64_t i) const { return (int64_t)p[i]; }
};

__device__ __forceinline__ int64_t block_sum(int64_t v, int64_t* smem_warp) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) smem_warp[w] = v;
  __syncthreads();
  int64_t t = 0;
  if (threadIdx.x < 32) {
    t = threadIdx.x < (blockDim.x >> 5) ? smem_warp[threadIdx.x] : 0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  return t;  // valid in thread 0
}

// Exclusive scan across the block of one value per thread; returns the
// thread's prefix and writes the block total to *total.
__device__ __forceinline__ int64_t block_exclusive(int64_t v, int64_t* smem_warp, int64_t* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int64_t inc = v;
  for (int o = 1; o < 32; o <<= 1) {
    int64_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) smem_warp[w] = inc;
  __syncthreads();
  if (threadIdx.x < 32) {
    const int nw = blockDim.x >> 5;
    int64_t x = threadIdx.x < nw ? smem_warp[threadIdx.x] : 0;
    int64_t xi = x;
    for (int o = 1; o < 32; o <<= 1) {
      int64_t t = __shfl_up_sync(0xffffffffu, xi, o);
      if (threadIdx.x >= o) xi += t;
    }
    if (threadIdx.x < nw) smem_warp[threadIdx.x] = xi - x;
    if (threadIdx.x == nw - 1) smem_warp[32] = xi;
  }
  __syncthreads();
  const int64_t r = smem_warp[w] + inc - v;
  *total = smem_warp[32];
  __syncthreads();
  return r;
}

// One block scans the whole (small) input tile by tile with a carry.
template <typename L>
__global__ void k_scan_single(L load, int64_t n, int64_t* out) {
  pdl_wait();
  pdl_trigger();
  __shared__ int64_t sw[33];
  int64_t carry = 0;
  for (int64_t base = 0; base < n; base += kTile) {
    int64_t v[kItems];
    int64_t local = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
      const int64_t i = base + (int64_t)threadIdx.x * kItems + k;
      v[k] = i < n ? load(i) : 0;
    }
#pragma unroll
    for (int k = 0; k < kItems; ++k) local += v[k];
    int64_t tot;
    int64_t pre = block_exclusive(local, sw, &tot) + carry;
    for (int k = 0; k < kItems; ++k) {
      const int64_t i = base + (int64_t)threadIdx.x * kItems + k;
      if (i < n) out[i] = pre;
      pre += v[k];
    }
    carry += tot;
  }
  if (threadIdx.x == 0) out[n] = carry;
}

// Single-pass scan with decoupled look-back (Merrill and Garland, "Single-pass
// Parallel Prefix Scan with Decoupled Look-back", 2016): one launch, one
// tile of kTile items per block.  Tile t publishes its aggregate, then looks
// back over its predecessors, adding aggregates until it meets an inclusive
// prefix, and publishes its own inclusive prefix.  Each tile has three
// status words: aggregate, inclusive prefix, and a tag (seq << 2 | flag,
// flag 1 = aggregate ready, 2 = inclusive ready), the value slots written
// before the tag.  `seq` is new for every call, so the words are never reset
// (a stale tag never matches).  Blocks are dispatched in index order, so a
// tile's predecessors are running or done; still, a wait on one gives up
// after kLookbackSpin reads, and the tile then sums its predecessors' inputs
// itself, so the result is right and the wait ends either way.
constexpr int64_t kLookbackSpin = (int64_t)1 << 22;

template <typename L>
__global__ void __launch_bounds__(kThreads) k_scan_lookback(L load, int64_t n, int64_t* out,
                                                            unsigned long long* st, unsigned long long seq) {
  pdl_wait();
  pdl_trigger();
  __shared__ int64_t tile[kTile];
  __shared__ int64_t sw[33];
  __shared__ int64_t s_excl;
  __shared__ int s_fallback;
  const int64_t t = blockIdx.x;
  const int64_t base = t * kTile;
  // all of the thread's items are loaded before any is stored: a loader's
  // generic loads may not pass a store to shared memory, so interleaved they
  // would run one dependent chain (list entry -> row bounds) at a time
  int64_t v[kItems];
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    const int64_t i = base + k * kThreads + threadIdx.x;
    v[k] = i < n ? load(i) : 0;
  }
#pragma unroll
  for (int k = 0; k < kItems; ++k) tile[k * kThreads + threadIdx.x] = v[k];
  __syncthreads();
  int64_t local = 0;
  for (int k = 0; k < kItems; ++k) local += tile[threadIdx.x * kItems + k];
  int64_t tot;
  int64_t pre = block_exclusive(local, sw, &tot);
  unsigned long long* my = st + 3 * t;
  if (threadIdx.x == 0) {
    int64_t excl = 0;
    int fb = 0;
    if (t > 0) {
      *(volatile unsigned long long*)(my + 0) = (unsigned long long)tot;
      __threadfence();
      atomicExch(my + 2, (seq << 2) | 1ull);
      for (int64_t q = t - 1; q >= 0;) {
        unsigned long long tag = 0;
        int64_t spins = 0;
        do {
          tag = *(volatile const unsigned long long*)(st + 3 * q + 2);
        } while ((tag >> 2) != seq && ++spins < kLookbackSpin);
        if ((tag >> 2) != seq) {
          fb = 1;
          break;
        }
        __threadfence();
        if ((tag & 3ull) == 2ull) {
          excl += (int64_t)*(volatile const unsigned long long*)(st + 3 * q + 1);
          break;
        }
        excl += (int64_t)*(volatile const unsigned long long*)(st + 3 * q + 0);
        --q;
      }
    }
    s_excl = excl;
    s_fallback = fb;
  }
  __syncthreads();
  if (s_fallback) {
    int64_t acc = 0;
    for (int64_t i = threadIdx.x; i < base; i += blockDim.x) acc += load(i);
    const int64_t sum = block_sum(acc, sw);
    if (threadIdx.x == 0) s_excl = sum;
    __syncthreads();
  }
  const int64_t excl = s_excl;
  if (threadIdx.x == 0) {
    *(volatile unsigned long long*)(my + 1) = (unsigned long long)(excl + tot);
    __threadfence();
    atomicExch(my + 2, (seq << 2) | 2ull);
  }
  pre += excl;
  for (int k = 0; k < kItems; ++k) {
    const int idx = threadIdx.x * kItems + k;
    const int64_t v = tile[idx];
    tile[idx] = pre;
    pre += v;
  }
  __syncthreads();
  for (int k = 0; k < kItems; ++k) {
    const int idx = k * kThreads + threadIdx.x;
    const int64_t i = base + idx;
    if (i < n) out[i] = tile[idx];
  }
  if (t == (int64_t)gridDim.x - 1 && threadIdx.x == 0) out[n] = excl + tot;
}

// Inputs up to two tiles go to one block; larger ones to the look-back scan.
constexpr int64_t kSingleScanMax = 2 * kTile;

template <typename L>
void scan_exclusive(L load, int64_t* out, int64_t n, Scratch& ws, cudaStream_t s) {
  if (n <= 0) {
    MF_CUDA(cudaMemsetAsync(out, 0, sizeof(int64_t), s));
    return;
  }
  if (n <= kSingleScanMax) {
    MF_K(launch_pdl(k_scan_single<L>, 1, kThreads, 0, s, load, n, out));
    MF_CUDA(cudaGetLastError());
    return;
  }
  const int64_t nb = (n + kTile - 1) / kTile;
  if (ws.scan_status.cap < 3 * nb) {
    ws.scan_status.reserve(3 * nb);
    // fresh memory may hold anything: no tag may match a later sequence number
    MF_CUDA(cudaMemsetAsync(ws.scan_status.p, 0, sizeof(unsigned long long) * (size_t)ws.scan_status.cap, s));
  }
  const unsigned long long seq = ++ws.scan_seq;
  MF_K(launch_pdl(k_scan_lookback<L>, (unsigned)nb, kThreads, 0, s, load, n, out, ws.scan_status.p, seq));
  MF_CUDA(cudaGetLastError());
}

}  // namespace scan_detail

// out[i] = sum_{j<i} load(j) for i in [0, n]; one launch.
template <typename L>
void scan_exclusive_with(L load, int64_t* out, int64_t n, Scratch& ws, cudaStream_t s) {
  scan_detail::scan_exclusive(load, out, n, ws, s);
}

}  // namespace mf
