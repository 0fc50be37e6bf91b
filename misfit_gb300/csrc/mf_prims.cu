// mf_prims.cu -- device scans and a stable LSD radix sort.
//
// Scans: one launch.  Small inputs in one block; larger ones with the
// single-pass decoupled look-back scan (k_scan_lookback).  Tiles are 256
// threads x 8 items, loaded striped for coalescing and scanned per thread out
// of shared memory.
// Radix sort: 8-bit digits, per-tile digit histograms, a scan over the
// digit-major histogram and a stable scatter that ranks items inside a tile
// with __match_any_sync.  Stability is what the callers rely on: equal keys
// keep their input (value) order.
#include "mf_internal.cuh"

namespace mf {

namespace {

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
  __shared__ int64_t sw[33];
  int64_t carry = 0;
  for (int64_t base = 0; base < n; base += kTile) {
    int64_t v[kItems];
    int64_t local = 0;
    for (int k = 0; k < kItems; ++k) {
      const int64_t i = base + (int64_t)threadIdx.x * kItems + k;
      v[k] = i < n ? load(i) : 0;
      local += v[k];
    }
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
  __shared__ int64_t tile[kTile];
  __shared__ int64_t sw[33];
  __shared__ int64_t s_excl;
  __shared__ int s_fallback;
  const int64_t t = blockIdx.x;
  const int64_t base = t * kTile;
  for (int k = 0; k < kItems; ++k) {
    const int idx = k * kThreads + threadIdx.x;
    const int64_t i = base + idx;
    tile[idx] = i < n ? load(i) : 0;
  }
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
    MF_K(k_scan_single<<<1, kThreads, 0, s>>>(load, n, out));
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
  MF_K(k_scan_lookback<<<(unsigned)nb, kThreads, 0, s>>>(load, n, out, ws.scan_status.p, seq));
  MF_CUDA(cudaGetLastError());
}

// ---- radix sort --------------------------------------------------------------

__global__ void k_radix_hist(const uint64_t* keys, int64_t n, int shift, int32_t* hist, int nblocks) {
  __shared__ int32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kTile;
  for (int k = 0; k < kItems; ++k) {
    const int64_t i = base + (int64_t)k * kThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1);
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

__global__ void k_radix_scatter(const uint64_t* keys, const uint32_t* vals, int64_t n, int shift,
                                const int64_t* offs, int nblocks, uint64_t* okeys, uint32_t* ovals) {
  __shared__ int32_t wcnt[kThreads / 32][256];
  __shared__ int32_t running[256];
  __shared__ int32_t itotal[256];
  __shared__ int64_t base_off[256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  base_off[threadIdx.x] = offs[(int64_t)threadIdx.x * nblocks + blockIdx.x];
  running[threadIdx.x] = 0;
  const unsigned lt = (1u << lane) - 1u;
  const int64_t base = (int64_t)blockIdx.x * kTile;
  for (int k = 0; k < kItems; ++k) {
    for (int j = 0; j < kThreads / 32; ++j) wcnt[j][threadIdx.x] = 0;
    __syncthreads();
    const int64_t i = base + (int64_t)k * kThreads + threadIdx.x;
    const bool valid = i < n;
    uint64_t key = 0;
    uint32_t val = 0;
    int d = 256;
    if (valid) {
      key = keys[i];
      val = vals[i];
      d = (int)((key >> shift) & 255u);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & lt);
    if (valid && rank == 0) wcnt[w][d] = __popc(peers);
    __syncthreads();
    {
      int acc = 0;
      for (int j = 0; j < kThreads / 32; ++j) {
        const int t = wcnt[j][threadIdx.x];
        wcnt[j][threadIdx.x] = acc;
        acc += t;
      }
      itotal[threadIdx.x] = acc;
    }
    __syncthreads();
    if (valid) {
      const int64_t pos = base_off[d] + running[d] + wcnt[w][d] + rank;
      okeys[pos] = key;
      ovals[pos] = val;
    }
    __syncthreads();
    running[threadIdx.x] += itotal[threadIdx.x];
    __syncthreads();
  }
}

// Whole stable LSD sort of up to kSmallSort pairs in one block: every 8-bit
// pass ranks the items with per-warp match_any counts, in shared memory.
constexpr int kSmallSort = 1024;

__global__ void __launch_bounds__(kThreads) k_radix_small(uint64_t* keys, uint32_t* vals, int n, int bits) {
  __shared__ uint64_t sk[2][kSmallSort];
  __shared__ uint32_t sv[2][kSmallSort];
  __shared__ int32_t wcnt[kThreads / 32][256];
  __shared__ int32_t dbase[256];
  __shared__ int32_t itotal[256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  for (int i = threadIdx.x; i < n; i += kThreads) {
    sk[0][i] = keys[i];
    sv[0][i] = vals[i];
  }
  __syncthreads();
  int cur = 0;
  for (int shift = 0; shift < bits; shift += 8) {
    // digit histogram -> exclusive digit bases
    dbase[threadIdx.x] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += kThreads) atomicAdd(&dbase[(sk[cur][i] >> shift) & 255u], 1);
    __syncthreads();
    if (threadIdx.x == 0) {
      int acc = 0;
      for (int d = 0; d < 256; ++d) { const int t = dbase[d]; dbase[d] = acc; acc += t; }
    }
    __syncthreads();
    for (int base = 0; base < n; base += kThreads) {
      for (int j = 0; j < kThreads / 32; ++j) wcnt[j][threadIdx.x] = 0;
      __syncthreads();
      const int i = base + threadIdx.x;
      const bool valid = i < n;
      int d = 256;
      if (valid) d = (int)((sk[cur][i] >> shift) & 255u);
      const unsigned peers = __match_any_sync(0xffffffffu, d);
      const int rank = __popc(peers & lt);
      if (valid && rank == 0) wcnt[w][d] = __popc(peers);
      __syncthreads();
      {
        int acc = 0;
        for (int j = 0; j < kThreads / 32; ++j) {
          const int t = wcnt[j][threadIdx.x];
          wcnt[j][threadIdx.x] = acc;
          acc += t;
        }
        itotal[threadIdx.x] = acc;
      }
      __syncthreads();
      if (valid) {
        const int pos = dbase[d] + wcnt[w][d] + rank;
        sk[cur ^ 1][pos] = sk[cur][i];
        sv[cur ^ 1][pos] = sv[cur][i];
      }
      __syncthreads();
      dbase[threadIdx.x] += itotal[threadIdx.x];
      __syncthreads();
    }
    cur ^= 1;
  }
  for (int i = threadIdx.x; i < n; i += kThreads) {
    keys[i] = sk[cur][i];
    vals[i] = sv[cur][i];
  }
}

}  // namespace

int bits_for(int64_t v) {
  int b = 1;
  while (b < 63 && (v >> b) != 0) ++b;
  return b;
}

void scan_exclusive_i64(const int64_t* in, int64_t* out, int64_t n, Scratch& ws, cudaStream_t s) {
  scan_exclusive(Loader<int64_t>{in}, out, n, ws, s);
}
void scan_exclusive_i32(const int32_t* in, int64_t* out, int64_t n, Scratch& ws, cudaStream_t s) {
  scan_exclusive(Loader<int32_t>{in}, out, n, ws, s);
}
void scan_exclusive_u8(const uint8_t* in, int64_t* out, int64_t n, Scratch& ws, cudaStream_t s) {
  scan_exclusive(Loader<uint8_t>{in}, out, n, ws, s);
}

void radix_sort_pairs(uint64_t* keys, uint32_t* vals, int64_t n, int bits, Scratch& ws, cudaStream_t s) {
  if (n <= 1) return;
  if (n <= kSmallSort) {
    MF_K(k_radix_small<<<1, kThreads, 0, s>>>(keys, vals, (int)n, bits));
    MF_CUDA(cudaGetLastError());
    return;
  }
  const int nblocks = (int)((n + kTile - 1) / kTile);
  ws.keys_alt.reserve(n);
  ws.vals_alt.reserve(n);
  ws.hist.reserve((int64_t)256 * nblocks);
  ws.hist_scan.reserve((int64_t)256 * nblocks + 1);
  uint64_t* ka = keys;
  uint32_t* va = vals;
  uint64_t* kb = ws.keys_alt.p;
  uint32_t* vb = ws.vals_alt.p;
  const int passes = (bits + 7) / 8;
  for (int pass = 0; pass < passes; ++pass) {
    const int shift = pass * 8;
    MF_K(k_radix_hist<<<nblocks, kThreads, 0, s>>>(ka, n, shift, ws.hist.p, nblocks));
    scan_exclusive_i32(ws.hist.p, ws.hist_scan.p, (int64_t)256 * nblocks, ws, s);
    MF_K(k_radix_scatter<<<nblocks, kThreads, 0, s>>>(ka, va, n, shift, ws.hist_scan.p, nblocks, kb, vb));
    MF_CUDA(cudaGetLastError());
    uint64_t* tk = ka; ka = kb; kb = tk;
    uint32_t* tv = va; va = vb; vb = tv;
  }
  if (ka != keys) {
    MF_CUDA(cudaMemcpyAsync(keys, ka, sizeof(uint64_t) * n, cudaMemcpyDeviceToDevice, s));
    MF_CUDA(cudaMemcpyAsync(vals, va, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s));
  }
}

}  // namespace mf
