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
#include "mf_scan.cuh"

namespace mf {

namespace {

using namespace scan_detail;

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
