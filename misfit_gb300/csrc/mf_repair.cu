// mf_repair.cu -- the per-sub-batch path on the device.
//
// Reference: GPUVertexClusteringGraph::processBatchWithVertexClustering
// (src/misfit/misfit.cu:468-692) with its host stages (split :490-521,
// 2-hop lists :527-558, row packing :560-599) and kernels (:211-358).
//
// The reference materialises every seed's exact 2-hop list on the host and
// ships it to the GPU.  Nothing here materialises a 2-hop list: a seed row is
// the virtual sequence  [s] ++ row(s) ++ row(h1) ++ row(h2) ++ ...  (h over
// row(s) in order).  The first element with a property is the same in the
// virtual sequence and in the de-duplicated BFS list, and set-valued queries
// do not care about repeats, so clustering and repair read rows straight out
// of the HBM CSR + overlay.  Only the split rule needs exact list lengths
// (MAX_CSR_ELEMENTS grows when the packed lists overflow it); those are
// counted exactly, and only when an upper bound says growth is possible.
//
// Canonical schedule for the racy kernels (the same the oracle uses):
//   clustering bulk-synchronous (pre-kernel reads, new ids by ascending row,
//   highest row writes last); assignment by ascending sub-batch index (lists
//   walked descending); clusters processed in ascending id.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <optional>
#include <unordered_map>

#include "mf_internal.cuh"
#include "mf_scan.cuh"

namespace mf {

int64_t initial_max_csr(int32_t n, uint64_t edges) {
  // src/misfit/misfit.cu:768-772
  double avg = n > 0 ? (double)edges / n : 1.0;
  int64_t est = (int64_t)(kMaxBatchEdges * 2.0 * avg * avg);
  int64_t v = est > 0 ? std::min<int64_t>(800000000LL, est) : 50000000LL;
  return std::max<int64_t>(v, 1000000LL);
}

namespace {

constexpr int kTB = 256;
static_assert(kTB == kLbThreads, "lb_rows kernels run kLbThreads-thread blocks");
constexpr int32_t kSkip = -2;
// host counter slots [kFrontSlot + 2f, +1]: front f's counts, copied on the
// stream that computed it
constexpr int kFrontSlot = 10;

inline unsigned grid_for(int64_t n, int per = kTB) {
  int64_t g = (n + per - 1) / per;
  if (g < 1) g = 1;
  return (unsigned)std::min<int64_t>(g, (int64_t)1 << 30);
}
inline unsigned warps_grid(int64_t items) { return grid_for(items * 32); }

__device__ __forceinline__ int64_t warp_id() {
  return ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
}

// ---- split ------------------------------------------------------------------

__global__ void k_slot_keys(const int32_t* u, const int32_t* v, int64_t m, int sbits, uint64_t* keys, uint32_t* vals) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 2 * m) return;
  const int32_t x = (i & 1) ? v[i >> 1] : u[i >> 1];
  keys[i] = ((uint64_t)x << sbits) | (uint64_t)i;
  vals[i] = (uint32_t)i;
}

__global__ void k_prev(const uint64_t* keys, const uint32_t* vals, int64_t cnt, int sbits, int32_t* prev) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= cnt) return;
  const uint32_t slot = vals[j];
  int32_t pe = -1;
  if (j > 0 && (keys[j - 1] >> sbits) == (keys[j] >> sbits)) pe = (int32_t)(vals[j - 1] >> 1);
  prev[slot] = pe;
}

// ---- sub-batch plan ---------------------------------------------------------------
// The split and the seed lists depend only on the batch, the degrees and
// MAX_CSR_ELEMENTS, not on the clustering or repair of earlier sub-batches,
// so they are planned for the whole batch (from p0) at once.

// Cuts of all sub-batches from p0 (src/misfit/misfit.cu:494-523): each edge
// adds deg * 1000 for every endpoint not seen yet in its sub-batch
// (:501-507), and the sub-batch ends before the first edge t >= 1 whose
// running estimate reaches MAX_CSR_ELEMENTS (:509-511).  One CTA:
// per sub-batch the estimates of a window of 1024 edges are scanned in shared
// memory; the cut is the first t >= 1 whose running estimate reaches maxcsr,
// else the length (min(m - p, MAX_BATCH_SIZE)).  cuts[k] = end of sub-batch
// k, ests[k] = estimate of the edges before the cut.
constexpr int kCutThreads = 1024;

__global__ void __launch_bounds__(kCutThreads) k_cuts(const int32_t* u, const int32_t* v, const int32_t* prev,
                                                      const int32_t* deg, int64_t m, int64_t p0, int64_t maxcsr,
                                                      int64_t* cuts, int64_t* ests, unsigned long long* count) {
  __shared__ int64_t s_warp[kCutThreads / 32];
  __shared__ int64_t s_total;
  __shared__ int64_t s_cut, s_est;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  int64_t p = p0, k = 0;
  while (p < m) {
    const int64_t len = min(m - p, kMaxBatchEdges);
    int64_t acc = 0;
    if (tid == 0) { s_cut = len; s_est = -1; }
    __syncthreads();
    for (int64_t t0 = 0; t0 < len; t0 += kCutThreads) {
      const int64_t t = t0 + tid;
      int64_t c = 0;
      if (t < len) {
        const int64_t j = p + t;
        if (prev[2 * j] < p) c += (int64_t)deg[u[j]] * kEstimateWeight;
        if (prev[2 * j + 1] < p) c += (int64_t)deg[v[j]] * kEstimateWeight;
      }
      int64_t inc = c;
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
      }
      if (lane == 31) s_warp[wid] = inc;
      __syncthreads();
      if (tid == 0) {
        int64_t run = 0;
        for (int w = 0; w < kCutThreads / 32; ++w) { const int64_t y = s_warp[w]; s_warp[w] = run; run += y; }
        s_total = run;
      }
      __syncthreads();
      const int64_t incl = acc + s_warp[wid] + inc;  // estimate of edges 0..t
      if (t >= 1 && t < len && incl >= maxcsr) atomicMin((unsigned long long*)&s_cut, (unsigned long long)t);
      __syncthreads();
      if (t == s_cut) s_est = incl - c;
      acc += s_total;
      __syncthreads();
      if (s_cut < len) break;
    }
    const int64_t cut = s_cut;
    if (tid == 0) {
      cuts[k] = p + cut;
      ests[k] = s_est >= 0 ? s_est : acc;
    }
    __syncthreads();
    p += cut;
    ++k;
  }
  if (tid == 0) *count = (unsigned long long)k;
}

// Seed flag of every endpoint slot from 2*p0: first appearance within its own
// sub-batch (the sub-batch of edge j starts at the last cut <= j).
__global__ void k_plan_seed_flags(const int32_t* prev, const int64_t* cuts, const unsigned long long* count, int64_t m,
                                  int64_t p0, uint8_t* flags) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 2 * (m - p0)) return;
  const int64_t slot = 2 * p0 + i;
  const int64_t j = slot >> 1;
  int64_t lo = 0, hi = (int64_t)*count;  // first k with cuts[k] > j
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (cuts[mid] <= j) lo = mid + 1; else hi = mid;
  }
  const int64_t start = lo == 0 ? p0 : cuts[lo - 1];
  flags[i] = prev[slot] < start ? 1 : 0;
}

__global__ void k_plan_seed_compact(const int32_t* u, const int32_t* v, const uint8_t* flags, const int64_t* pos,
                                    int64_t m, int64_t p0, int32_t* seeds_all) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 2 * (m - p0) || !flags[i]) return;
  const int64_t slot = 2 * p0 + i;
  seeds_all[pos[i]] = (slot & 1) ? v[slot >> 1] : u[slot >> 1];
}

// seed_end[k] = number of seeds of sub-batches 0..k.
__global__ void k_plan_seed_ends(const int64_t* cuts, const unsigned long long* count, const int64_t* pos, int64_t p0,
                                 int64_t* seed_end) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < (int64_t)*count) seed_end[k] = pos[2 * (cuts[k] - p0)];
}

// Seeds of one sub-batch into their rows: seeds[i], v2i[seeds[i]] = i.
__global__ void k_seed_rows(const int32_t* seeds_all, int64_t ns, int32_t* seeds, int32_t* v2i) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ns) return;
  const int32_t x = seeds_all[i];
  seeds[i] = x;
  v2i[x] = (int32_t)i;
}

// ---- hop-1 set and candidates ---------------------------------------------------

// Row-position counts for lb_rows; rows that must not be visited count 0.
// kCntMarked: the rows i with marks[i] >= 0 (marks passed as rowcid).
enum CountKind : int { kCntAll = 0, kCntSeedRows, kCntCandRows, kCntSeedPushers, kCntHopPushers, kCntMarked };

// The count of row i is computed inside the scan's tile load (RowCounts is
// the scan's loader), so the prefix needs one launch and no count array.
struct RowCounts {
  GraphView g;
  const int32_t* list;
  int kind;
  const int32_t* rowcid;
  int64_t ns;
  const uint32_t* bval;
  uint32_t epoch;
  const int32_t* v2i;
  __device__ __forceinline__ int64_t operator()(int64_t i) const {
    const int32_t x = list[i];
    bool use = true;
    if (kind == kCntSeedRows) {
      use = rowcid[i] != kSkip;
    } else if (kind == kCntCandRows) {
      use = rowcid[ns + i] != kSkip;
    } else if (kind == kCntSeedPushers) {
      use = (bval[x] >> kRowBits) == epoch;
    } else if (kind == kCntMarked) {
      use = rowcid[i] >= 0;
    } else if (kind == kCntHopPushers) {
      use = (bval[x] >> kRowBits) == epoch;
      const int32_t vi = v2i[x];
      // seeds push in their own pass; a candidate row that writes its own tag
      // over row(x) dominates bval[x] there (candidate tags are the larger)
      if (vi >= 0 && ((int64_t)vi < ns || rowcid[vi] != kSkip)) use = false;
    }
    return use ? row_positions(g, x) : 0;
  }
};

__device__ __forceinline__ void add_work(unsigned long long* work, int64_t visited) {
  for (int o = 16; o > 0; o >>= 1) visited += __shfl_down_sync(0xffffffffu, visited, o);
  if ((threadIdx.x & 31) == 0 && visited) atomicAdd(work, (unsigned long long)visited);
}

// ---- hop-1 set as a bitmap ----------------------------------------------------------
// The hop-1 marks of a sub-batch go into a bitmap (hbits) and the seeds into
// another (sbits); a two-level popcount scan over the words gives, per word,
// the offsets of its marked vertices in hlist and of its marked non-seeds in
// the candidate list, so both lists come out in ascending vertex id without
// touching n-sized arrays.  Counts are packed as (hop-1 << 32) | candidates.
constexpr int kBitsThreads = 256;
constexpr int kBitsPerThread = 1;                               // words per thread
constexpr int kBitsWords = kBitsThreads * kBitsPerThread;       // words per block

// One pass over the seed rows: the hop-1 bit of every element, and per seed
// the sum of len(h) over row(s) for the packed-size upper bound (uacc).
// deg[y] (DeltaOverlay::degree) is at least the overlay row length of y (a
// tombstone removes at least one base entry), so the sums stay upper bounds.
__global__ void __launch_bounds__(kLbThreads, MF_LB_MIN_BLOCKS) k_lb_hop1_bound(GraphView g, const int32_t* deg, const int32_t* seeds,
                                                              const int64_t* offs, int64_t ns, uint32_t* hbits,
                                                              unsigned long long* uacc, unsigned long long* work) {
  pdl_wait();
  pdl_trigger();
  int64_t cur = -1;
  unsigned long long acc = 0;
  const int64_t vis = lb_rows(g, seeds, offs, ns, [&](int64_t i, int32_t, int32_t y) {
    const uint32_t bit = 1u << (y & 31);
    if (!(hbits[y >> 5] & bit)) atomicOr(hbits + (y >> 5), bit);
    if (i != cur) {
      if (cur >= 0 && acc) atomicAdd(uacc + cur, acc);
      cur = i;
      acc = 0;
    }
    acc += (unsigned long long)__ldg(deg + y);
  });
  if (cur >= 0 && acc) atomicAdd(uacc + cur, acc);
  add_work(work, vis);
}

__global__ void k_seed_bits(const int32_t* seeds, int64_t ns, uint32_t* sbits) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ns) atomicOr(sbits + (seeds[i] >> 5), 1u << (seeds[i] & 31));
}

__device__ __forceinline__ int64_t bits_count4(const uint32_t* hbits, const uint32_t* sbits, int64_t w0,
                                               int64_t words) {
  int64_t h = 0, c = 0;
  for (int j = 0; j < kBitsPerThread; ++j) {
    const int64_t w = w0 + j;
    if (w < words) {
      const uint32_t m = hbits[w];
      h += __popc(m);
      c += __popc(m & ~sbits[w]);
    }
  }
  return (h << 32) | c;
}

// Block-wide exclusive scan of one int64 per thread (kBitsThreads threads).
__device__ __forceinline__ int64_t bits_block_scan(int64_t x, int64_t* s_warp, int64_t* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int64_t inc = x;
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) s_warp[wid] = inc;
  __syncthreads();
  if (threadIdx.x == 0) {
    int64_t run = 0;
    for (int w = 0; w < kBitsThreads / 32; ++w) { const int64_t y = s_warp[w]; s_warp[w] = run; run += y; }
    s_warp[kBitsThreads / 32] = run;
  }
  __syncthreads();
  const int64_t r = s_warp[wid] + inc - x;
  *total = s_warp[kBitsThreads / 32];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kBitsThreads) k_bits_reduce(const uint32_t* hbits, const uint32_t* sbits,
                                                              int64_t words, int64_t* block_sums) {
  pdl_wait();
  pdl_trigger();
  __shared__ int64_t s_warp[kBitsThreads / 32 + 1];
  const int64_t w0 = (int64_t)blockIdx.x * kBitsWords + (int64_t)threadIdx.x * kBitsPerThread;
  int64_t total = 0;
  bits_block_scan(bits_count4(hbits, sbits, w0, words), s_warp, &total);
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// Exclusive scan of the block sums in place (one block; loops for any count);
// the grand total goes to *total.
__global__ void __launch_bounds__(kBitsThreads) k_bits_scan_sums(int64_t* block_sums, int64_t nblocks,
                                                                 int64_t* total) {
  pdl_wait();
  pdl_trigger();
  __shared__ int64_t s_warp[kBitsThreads / 32 + 1];
  int64_t carry = 0;
  for (int64_t b0 = 0; b0 < nblocks; b0 += kBitsThreads) {
    const int64_t b = b0 + threadIdx.x;
    const int64_t x = b < nblocks ? block_sums[b] : 0;
    int64_t t = 0;
    const int64_t e = bits_block_scan(x, s_warp, &t);
    if (b < nblocks) block_sums[b] = carry + e;
    carry += t;
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(kBitsThreads) k_bits_compact(const uint32_t* hbits, const uint32_t* sbits,
                                                               int64_t words, const int64_t* block_offs, int64_t cap,
                                                               int64_t ns, int32_t* hlist, int32_t* cands,
                                                               int32_t* v2i) {
  pdl_wait();
  pdl_trigger();
  __shared__ int64_t s_warp[kBitsThreads / 32 + 1];
  const int64_t w0 = (int64_t)blockIdx.x * kBitsWords + (int64_t)threadIdx.x * kBitsPerThread;
  int64_t total = 0;
  const int64_t off = block_offs[blockIdx.x] + bits_block_scan(bits_count4(hbits, sbits, w0, words), s_warp, &total);
  int64_t ph = off >> 32, pc = off & 0xffffffffll;
  for (int j = 0; j < kBitsPerThread; ++j) {
    const int64_t w = w0 + j;
    if (w >= words) break;
    uint32_t m = hbits[w];
    const uint32_t sm = sbits[w];
    while (m) {
      const int b = __ffs(m) - 1;
      m &= m - 1;
      const int32_t x = (int32_t)(w * 32 + b);
      hlist[ph++] = x;
      if (!((sm >> b) & 1u)) {
        if (pc < cap) {
          cands[pc] = x;
          if (v2i) v2i[x] = (int32_t)(ns + pc);
        }
        ++pc;
      }
    }
  }
}

// Row map of the candidates (rows ns .. ns + nct - 1), once the previous
// sub-batch has cleared its rows.
__global__ void k_cand_v2i(const int32_t* cands, int64_t nct, int64_t ns, int32_t* v2i) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nct) v2i[cands[i]] = (int32_t)(ns + i);
}

// ---- packed sizes ---------------------------------------------------------------

// Upper bound of the packed element count: per seed 1 + len(s) + sum of
// len(h) over row(s), capped by n (the sums come from k_lb_hop1_bound); plus
// the candidate row lengths.
// The candidate count comes from the hop-1 compaction on the device (low 32
// bits of *hop_counts, capped at capc), so the bound needs no host round trip
// after the hop-1 stage.  Grid-stride over the ns + nct rows.
__global__ void k_bound_finish(GraphView g, const int32_t* seeds, int64_t ns, const int32_t* cands,
                               const int64_t* hop_counts, int64_t capc, const unsigned long long* uacc,
                               const int64_t* n2cache, const uint32_t* n2stamp, const int64_t* n2bound,
                               const uint32_t* n2bstamp, uint32_t stamp, unsigned long long* out) {
  pdl_wait();
  pdl_trigger();
  const int64_t nct = min((int64_t)(*hop_counts & 0xffffffffll), capc);
  const int64_t rows = ns + nct;
  unsigned long long b = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x) {
    if (i < ns) {
      const int32_t s = seeds[i];
      if (n2stamp[s] == stamp) {
        b += (unsigned long long)n2cache[s];   // exact size known from an earlier sub-batch
      } else if (n2bstamp[s] == stamp) {
        b += (unsigned long long)n2bound[s];   // tighter bound known from an earlier sub-batch
      } else {
        unsigned long long e = 1ull + (unsigned long long)row_len(g, s) + uacc[i];
        if (e > (unsigned long long)g.n) e = (unsigned long long)g.n;
        b += e;
      }
    } else {
      b += (unsigned long long)row_len(g, cands[i - ns]);
    }
  }
  for (int o = 16; o > 0; o >>= 1) b += __shfl_down_sync(0xffffffffu, b, o);
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(out, b);
}

// Seeds whose exact size is cached for this batch take it; the others are
// listed for computation.
// With bounds (the tighter-bound pass), a cached bound also counts as known.
__global__ void k_exact_todo(const int32_t* seeds, int64_t ns, const int64_t* n2cache, const uint32_t* n2stamp,
                             const int64_t* n2bound, const uint32_t* n2bstamp, bool bounds, uint32_t stamp,
                             int64_t* lens, int32_t* todo, unsigned long long* cnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ns) return;
  const int32_t s = seeds[i];
  if (n2stamp[s] == stamp) lens[i] = n2cache[s];
  else if (bounds && n2bstamp[s] == stamp) lens[i] = n2bound[s];
  else todo[atomicAdd(cnt, 1ull)] = (int32_t)i;
}

__global__ void k_exact_store(const int32_t* seeds, const int32_t* list, int64_t cnt, const int64_t* lens,
                              int64_t* n2cache, uint32_t* n2stamp, uint32_t stamp) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= cnt) return;
  const int64_t i = list[k];
  const int32_t s = seeds[i];
  n2cache[s] = lens[i];
  n2stamp[s] = stamp;
}

// ---- exact 2-hop list sizes ------------------------------------------------------
// |2-hop list of s| = |union over h in N[s] of N[h]|, N[x] = {x} u row(x).
// Heavy vertices (row length >= threshold) get a bitmap of N[h] built once per
// batch (rows do not change between the sub-batches of a batch).  A seed with
// heavy members ORs their bitmaps word-parallel into its CTA's private
// bitmap, sets the bits of the light members' N[h] with atomics, and counts
// with popcount; a seed with only light members and little volume sets bits
// and counts newly set ones, then clears the words it touched.

constexpr int kMaxHeavyPerSeed = 2048;

__global__ void k_heavy_collect(GraphView g, const int32_t* seeds, const int64_t* offs, int64_t ns, int64_t thr,
                                int32_t* slot, int32_t* list, unsigned long long* count) {
  auto consider = [&](int32_t h) {
    if (row_len(g, h) >= thr && slot[h] == -1 && atomicCAS(slot + h, -1, -2) == -1)
      list[atomicAdd(count, 1ull)] = h;
  };
  lb_rows(g, seeds, offs, ns, [&](int64_t, int32_t, int32_t y) { consider(y); });
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += (int64_t)gridDim.x * blockDim.x)
    consider(seeds[i]);
}

__global__ void k_heavy_assign(const int32_t* list, int64_t from, int64_t to, int64_t cap, int32_t* slot) {
  const int64_t k = from + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < to) slot[list[k]] = k < cap ? (int32_t)k : -3;
}

__global__ void k_heavy_reset(const int32_t* list, int64_t cnt, int32_t* slot) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < cnt) slot[list[k]] = -1;
}

// Bits of N[h] for the heavy vertices list[0..cnt) (their bitmaps are slots
// from..from+cnt, zeroed before).
__global__ void k_heavy_build(GraphView g, const int32_t* list, const int64_t* offs, int64_t cnt, int64_t from,
                              int64_t words, uint32_t* bits) {
  lb_rows(g, list, offs, cnt, [&](int64_t i, int32_t, int32_t y) {
    atomicOr(bits + (from + i) * words + (y >> 5), 1u << (y & 31));
  });
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t h = list[i];
    atomicOr(bits + (from + i) * words + (h >> 5), 1u << (h & 31));
  }
}

// Classification pass, one CTA per seed: heavy members (cached bitmaps) and
// the light volume of N[s].  Seeds with little light volume and no heavy
// member are counted right here in the CTA's private bitmap (set bits,
// count newly set ones, clear what was touched).  The others are "dense":
// each gets a global bitmap (at most dmax of them per pass; the rest are
// marked -2 for the next pass), its heavy slots and its light members go
// to lists that the grid-wide passes below consume.
struct DenseOut {
  unsigned long long* ndense;     // dense seeds accepted
  int32_t* dseed;                 // dense index -> seed index
  int32_t* dhoff;                 // dense index -> offset in hlist
  int32_t* dnh;                   // dense index -> heavy count
  int32_t* hlist;                 // heavy slots of all dense seeds
  unsigned long long* hused;
  int32_t* pair_d;                // light members: dense index
  int32_t* pair_h;                // light members: vertex
  unsigned long long* npairs;
  int64_t* dlight;                // dense index -> light volume (sum of |N[h]| over light members)
  int64_t dmax, hcap, pcap;
};

__global__ void __launch_bounds__(512) k_exact_classify(GraphView g, const int32_t* seeds, const int32_t* todo,
                                                        int64_t ntodo, const int32_t* slot, int64_t words,
                                                        uint32_t* privbm, int64_t dense_min, int64_t* lens,
                                                        DenseOut o) {
  uint32_t* P = privbm + (int64_t)blockIdx.x * words;
  __shared__ int32_t s_h[kMaxHeavyPerSeed];
  __shared__ int s_nh, s_over, s_d;
  __shared__ unsigned long long s_light, s_lcount, s_acount, s_cnt, s_pbase, s_pfill;
  __shared__ int s_hoff;
  const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t t = blockIdx.x; t < ntodo; t += gridDim.x) {
    const int64_t i = todo[t];
    const int32_t s = seeds[i];
    if (threadIdx.x == 0) { s_nh = 0; s_over = 0; s_light = 0; s_lcount = 0; s_acount = 0; s_cnt = 0; s_pfill = 0; }
    __syncthreads();
    const int64_t nb = g.nindex[s + 1] - g.nindex[s];
    const int64_t total = nb + (g.aoff[s + 1] - g.aoff[s]);
    {
      unsigned long long lsum = 0, lcnt = 0, acnt = 0;
      for (int64_t k = (int64_t)threadIdx.x - 1; k < total; k += blockDim.x) {
        const int32_t h = k < 0 ? s : row_elem(g, s, k, nb);
        if (h < 0) continue;
        ++acnt;
        const int32_t sl = slot[h];
        if (sl >= 0) {
          const int idx = atomicAdd(&s_nh, 1);
          if (idx < kMaxHeavyPerSeed) s_h[idx] = sl; else s_over = 1;
        } else {
          lsum += (unsigned long long)(row_len(g, h) + 1);
          lcnt += 1;
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
        lcnt += __shfl_xor_sync(0xffffffffu, lcnt, o);
        acnt += __shfl_xor_sync(0xffffffffu, acnt, o);
      }
      if ((threadIdx.x & 31) == 0) {
        if (lcnt) {
          atomicAdd(&s_light, lsum);
          atomicAdd(&s_lcount, lcnt);
        }
        if (acnt) atomicAdd(&s_acount, acnt);
      }
    }
    __syncthreads();
    const bool over = s_over != 0;
    const bool dense = over || s_nh > 0 || (int64_t)s_light > dense_min;
    if (!dense) {
      unsigned long long local = 0;
      auto setbit = [&](int32_t y) {
        const uint32_t bit = 1u << (y & 31);
        if (!(atomicOr(P + (y >> 5), bit) & bit)) ++local;
      };
      if (threadIdx.x == 0) setbit(s);
      for (int64_t k = threadIdx.x; k < total; k += blockDim.x) {
        const int32_t h = row_elem(g, s, k, nb);
        if (h >= 0) setbit(h);
      }
      for (int64_t k = wid; k < total; k += nw) {
        const int32_t h = row_elem(g, s, k, nb);
        if (h >= 0) warp_row_each(g, h, setbit);
      }
      atomicAdd(&s_cnt, local);
      __syncthreads();
      auto clr = [&](int32_t y) { P[y >> 5] = 0u; };
      if (threadIdx.x == 0) clr(s);
      for (int64_t k = threadIdx.x; k < total; k += blockDim.x) {
        const int32_t h = row_elem(g, s, k, nb);
        if (h >= 0) clr(h);
      }
      for (int64_t k = wid; k < total; k += nw) {
        const int32_t h = row_elem(g, s, k, nb);
        if (h >= 0) warp_row_each(g, h, clr);
      }
      __syncthreads();
      if (threadIdx.x == 0) lens[i] = (int64_t)s_cnt;
    } else {
      const int nh = over ? 0 : s_nh;
      // pair slots: one per member written below (all live members when the
      // heavy list overflowed, else the light ones)
      const unsigned long long lc = over ? s_acount : s_lcount;
      if (threadIdx.x == 0) {
        s_d = -1;
        const unsigned long long d = atomicAdd(o.ndense, 1ull);
        const unsigned long long hoff = atomicAdd(o.hused, (unsigned long long)nh);
        const unsigned long long pb = atomicAdd(o.npairs, lc);
        s_pbase = pb;
        if ((int64_t)d < o.dmax && (int64_t)(hoff + nh) <= o.hcap && (int64_t)(pb + lc) <= o.pcap) {
          s_d = (int)d;
          s_hoff = (int)hoff;
          o.dseed[d] = (int32_t)i;
          o.dhoff[d] = (int32_t)hoff;
          o.dnh[d] = nh;
          o.dlight[d] = over ? (int64_t)g.n : (int64_t)s_light;
          lens[i] = 0;
        } else {
          if ((int64_t)d < o.dmax) o.dseed[d] = -1;   // index taken but unused
          lens[i] = -2;                                  // retried in the next pass
        }
      }
      __syncthreads();
      const int d = s_d;
      if (d < 0) {
        // retried in the next pass: the pair slots this seed reserved are
        // marked unused (k_dense_light and its row prefix skip them)
        const unsigned long long q1 = min(s_pbase + lc, (unsigned long long)o.pcap);
        for (unsigned long long q = s_pbase + threadIdx.x; q < q1; q += blockDim.x) {
          o.pair_d[q] = -1;
          o.pair_h[q] = s;
        }
      }
      if (d >= 0) {
        for (int j = threadIdx.x; j < nh; j += blockDim.x) o.hlist[s_hoff + j] = s_h[j];
        // one shared atomic per warp and round: the lanes with a light member
        // take consecutive slots
        const int lane = threadIdx.x & 31;
        for (int64_t k0 = -1; k0 < total; k0 += blockDim.x) {
          const int64_t k = k0 + threadIdx.x;
          int32_t h = -1;
          if (k < total) {
            h = k < 0 ? s : row_elem(g, s, k, nb);
            if (h >= 0 && !over && slot[h] >= 0) h = -1;
          }
          const unsigned m = __ballot_sync(0xffffffffu, h >= 0);
          if (m == 0) continue;
          unsigned long long base = 0;
          if (lane == 0) base = atomicAdd(&s_pfill, (unsigned long long)__popc(m));
          base = __shfl_sync(0xffffffffu, base, 0);
          if (h >= 0) {
            const unsigned long long q = s_pbase + base + __popc(m & ((1u << lane) - 1u));
            o.pair_d[q] = d;
            o.pair_h[q] = h;
          }
        }
      }
    }
    __syncthreads();
  }
}

// Dense bitmaps: P_d = OR of the heavy members' cached bitmaps.  Grid
// (dense seeds, word tiles) with the seed index fastest, so that the seeds
// sharing a heavy member read its tile while it is still in L2.
constexpr int kDenseTile = 2048;  // words per block (256 threads x 8)

__global__ void k_dense_or(int64_t nd, const int32_t* dseed, const int32_t* dhoff, const int32_t* dnh,
                           const int32_t* hlist, const uint32_t* hbits, int64_t words, uint32_t* dbits) {
  const int64_t d = blockIdx.x;
  if (d >= nd) return;
  const int32_t nh = dseed[d] >= 0 ? dnh[d] : 0;
  const int32_t* hl = hlist + dhoff[d];
  const int64_t w0 = (int64_t)blockIdx.y * kDenseTile;
  const int64_t w1 = min(words, w0 + kDenseTile);
  for (int64_t w = w0 + threadIdx.x; w < w1; w += blockDim.x) {
    uint32_t v = 0;
    for (int j = 0; j < nh; ++j) v |= __ldg(hbits + (int64_t)hl[j] * words + w);
    dbits[d * words + w] = v;
  }
}

// Dense bitmaps: bits of N[h] for every light member h (load-balanced).
__global__ void k_dense_light(GraphView g, const int32_t* pair_d, const int32_t* pair_h, const int64_t* offs,
                              int64_t np, int64_t words, uint32_t* dbits) {
  lb_rows(g, pair_h, offs, np, [&](int64_t k, int32_t, int32_t y) {
    atomicOr(dbits + (int64_t)pair_d[k] * words + (y >> 5), 1u << (y & 31));
  });
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < np; k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t h = pair_h[k];
    if (pair_d[k] >= 0) atomicOr(dbits + (int64_t)pair_d[k] * words + (h >> 5), 1u << (h & 31));
  }
}

__global__ void k_dense_pop(int64_t nd, const int32_t* dseed, int64_t words, const uint32_t* dbits, int64_t* lens) {
  const int64_t d = blockIdx.x;
  if (d >= nd || dseed[d] < 0) return;
  const int64_t w0 = (int64_t)blockIdx.y * kDenseTile;
  const int64_t w1 = min(words, w0 + kDenseTile);
  unsigned long long c = 0;
  for (int64_t w = w0 + threadIdx.x; w < w1; w += blockDim.x) c += __popc(dbits[d * words + w]);
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(reinterpret_cast<unsigned long long*>(lens + dseed[d]), c);
}

// Upper bound of a dense seed's 2-hop size without the light members' bits:
// |union of the heavy N[h]| + sum of |N[h]| over the light members, at most n.
__global__ void k_dense_bound(int64_t nd, const int32_t* dseed, const int64_t* dlight, int32_t n, int64_t* lens) {
  const int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nd || dseed[d] < 0) return;
  int64_t* l = lens + dseed[d];
  *l = min((int64_t)n, *l + dlight[d]);
}

__global__ void k_todo_retry(const int64_t* lens, const int32_t* todo, int64_t ntodo, int32_t* out,
                             unsigned long long* cnt) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < ntodo && lens[todo[t]] == -2) out[atomicAdd(cnt, 1ull)] = todo[t];
}

// ---- exact 2-hop sizes, pull form (symmetric graphs) ----------------------------
// For a group of up to 32*SW seeds s_j: mask[u] bit j <=> u in N[s_j].  On a
// symmetric overlay graph, v is in the 2-hop list of s_j iff the OR of mask
// over {v} u row(v) has bit j:
//   v in N[s_j]                          <=> mask[v] bit j;
//   v in row(y) for some y in row(s_j)   <=> y in row(v), and mask[y] bit j;
// and u = s_j in row(v) means v in row(s_j).  One pass over every row
// therefore sizes the whole group: it reads each live entry once and gathers
// one mask per entry, a cost set by the graph, where the push form pays one
// atomic per element of every member's row (tens of millions per seed next to
// R-MAT hubs).
constexpr int kP2MaxWords = 8;          // mask words per vertex: up to 256 seeds per pass
constexpr int64_t kP2Short = 32;        // rows of up to this many positions: one thread each
constexpr int64_t kP2Huge = 1024;       // rows longer than this: chunks spread over many warps
constexpr int64_t kP2Chunk = 2048;      // positions per chunk of a huge row
constexpr int64_t kP2Grab = 128;        // vertices per block a warp takes
constexpr double kP2PassVolume = 0.5;   // cost of a pass, in push-form volume per position

template <int SW>
__device__ __forceinline__ void p2_or(uint32_t (&m)[SW], const uint32_t* mask, int32_t u) {
  const uint32_t* p = mask + (int64_t)u * SW;
  if constexpr (SW >= 4) {
#pragma unroll
    for (int h = 0; h < SW / 4; ++h) {
      const uint4 a = __ldg(reinterpret_cast<const uint4*>(p) + h);
      m[4 * h] |= a.x;
      m[4 * h + 1] |= a.y;
      m[4 * h + 2] |= a.z;
      m[4 * h + 3] |= a.w;
    }
  } else if constexpr (SW == 2) {
    const uint2 a = __ldg(reinterpret_cast<const uint2*>(p));
    m[0] |= a.x;
    m[1] |= a.y;
  } else {
    m[0] |= __ldg(p);
  }
}

// Bit u of the group's filter: u is in some N[s_j] (mask[u] is not zero).
// n bits stay in L2 while the masks (up to 32 bytes per vertex) do not, so
// the pass reads a mask from DRAM only where the filter says it is not zero.
__device__ __forceinline__ bool p2_in(const uint32_t* filt, int32_t u) {
  return (__ldg(filt + (u >> 5)) >> (u & 31)) & 1u;
}

// OR of mask over positions [lo, hi) of row(x), every lane a share (lanes
// disagree until p2_warp_or).
template <int SW>
__device__ __forceinline__ void p2_warp_span(const GraphView& g, const uint32_t* mask, const uint32_t* filt,
                                             int32_t x, int64_t lo, int64_t hi, uint32_t (&m)[SW]) {
  const int lane = threadIdx.x & 31;
  const int64_t b = g.nindex[x], nb = g.nindex[x + 1] - b;
  const bool dead = g.dead[x] != 0;
  const int64_t ab = g.aoff[x];
  for (int64_t k0 = lo + lane; k0 < hi; k0 += 128) {
    int32_t y[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t k = k0 + 32 * q;
      y[q] = -1;
      if (k < hi) {
        if (k < nb) {
          if (!dead || live_at(g.live, b + k)) y[q] = __ldg(g.nlist + b + k);
        } else {
          y[q] = g.aadj[ab + (k - nb)];
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (y[q] >= 0 && !p2_in(filt, y[q])) y[q] = -1;
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (y[q] >= 0) p2_or(m, mask, y[q]);
  }
}

template <int SW>
__device__ __forceinline__ void p2_warp_or(uint32_t (&m)[SW]) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int w = 0; w < SW; ++w) m[w] |= __shfl_xor_sync(0xffffffffu, m[w], o);
}

// acc[w] of lane l += number of lanes whose m[w] has bit l (all lanes call).
template <int SW>
__device__ __forceinline__ void p2_count_lanes(const uint32_t (&m)[SW], uint32_t (&acc)[SW]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int w = 0; w < SW; ++w) {
    if (!__any_sync(0xffffffffu, m[w] != 0u)) continue;
#pragma unroll 8
    for (int bit = 0; bit < 32; ++bit) {
      const unsigned bal = __ballot_sync(0xffffffffu, (m[w] >> bit) & 1u);
      if (lane == bit) acc[w] += (uint32_t)__popc(bal);
    }
  }
}

// Per-lane counts into the group's counters (through shared memory).
template <int SW>
__device__ __forceinline__ void p2_flush(const uint32_t (&acc)[SW], unsigned long long* s_cnt,
                                         unsigned long long* counts) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int w = 0; w < SW; ++w)
    if (acc[w]) atomicAdd(s_cnt + w * 32 + lane, (unsigned long long)acc[w]);
  __syncthreads();
  for (int i = threadIdx.x; i < 32 * SW; i += blockDim.x)
    if (s_cnt[i]) atomicAdd(counts + i, s_cnt[i]);
}

// Neighbourhood volume of each seed to size: sum over h in N[s] of
// (deg(h) + 1).  Grid (seeds, 4 slices of the row); vol pre-zeroed.
__global__ void k_p2_volume(GraphView g, const int32_t* deg, const int32_t* seeds, const int32_t* todo, int64_t ntodo,
                            int64_t* vol) {
  const int64_t t = blockIdx.x;
  if (t >= ntodo) return;
  const int32_t s = seeds[todo[t]];
  const int64_t nb = g.nindex[s + 1] - g.nindex[s];
  const int64_t total = nb + (g.aoff[s + 1] - g.aoff[s]);
  unsigned long long sum = 0;
  for (int64_t k = (int64_t)blockIdx.y * blockDim.x + threadIdx.x - 1; k < total;
       k += (int64_t)gridDim.y * blockDim.x) {
    const int32_t h = k < 0 ? s : row_elem(g, s, k, nb);
    if (h >= 0) sum += (unsigned long long)__ldg(deg + h) + 1ull;
  }
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if ((threadIdx.x & 31) == 0 && sum) atomicAdd(reinterpret_cast<unsigned long long*>(vol + t), sum);
}

// mask[u] bit j for u in N[s_j], j < k.  Grid (k, slices of the row).
template <int SW>
__global__ void k_p2_mark(GraphView g, const int32_t* seeds, const int32_t* grp, int k, uint32_t* mask,
                          uint32_t* filt) {
  const int j = blockIdx.x;
  if (j >= k) return;
  const int32_t s = seeds[grp[j]];
  const int64_t nb = g.nindex[s + 1] - g.nindex[s];
  const int64_t total = nb + (g.aoff[s + 1] - g.aoff[s]);
  const uint32_t bit = 1u << (j & 31);
  uint32_t* col = mask + (j >> 5);
  for (int64_t t = (int64_t)blockIdx.y * blockDim.x + threadIdx.x - 1; t < total;
       t += (int64_t)gridDim.y * blockDim.x) {
    const int32_t h = t < 0 ? s : row_elem(g, s, t, nb);
    if (h < 0) continue;
    uint32_t* p = col + (int64_t)h * SW;
    if (!(*p & bit)) atomicOr(p, bit);   // a stale read only costs an atomic
    uint32_t* f = filt + (h >> 5);
    const uint32_t fb = 1u << (h & 31);
    if (!(*f & fb)) atomicOr(f, fb);
  }
}

// The pass over every vertex.  Warps take blocks of kP2Grab consecutive
// vertices from a counter (the work of a block varies by orders of
// magnitude on power-law graphs; static assignment left most SMs idle
// while a few walked the heavy blocks).  In a block, 32 vertices at a time:
// rows of up to kP2Short positions one thread each, rows up to kP2Huge by
// the whole warp one after another; longer rows get a slot in `huge` and one
// task per kP2Chunk positions for k_p2_huge.  counts[j] += vertices whose OR
// has bit j.
struct P2Work {
  unsigned long long* next;      // vertex counter of the block grabs
  int32_t* huge;                 // slot -> vertex
  unsigned long long* nhuge;
  int64_t hcap;
  int64_t* tasks;                // (slot << 32) | chunk
  unsigned long long* ntasks;
  int64_t tcap;
};

template <int SW>
__global__ void __launch_bounds__(256) k_p2_rows(GraphView g, const uint32_t* mask, const uint32_t* filt,
                                                 unsigned long long* counts, P2Work wk) {
  __shared__ unsigned long long s_cnt[32 * SW];
  for (int i = threadIdx.x; i < 32 * SW; i += blockDim.x) s_cnt[i] = 0;
  __syncthreads();
  uint32_t acc[SW];
#pragma unroll
  for (int w = 0; w < SW; ++w) acc[w] = 0;
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long grab = 0;
    if (lane == 0) grab = atomicAdd(wk.next, (unsigned long long)kP2Grab);
    const int64_t first = (int64_t)__shfl_sync(0xffffffffu, grab, 0);
    if (first >= g.n) break;
    const int64_t last = min((int64_t)g.n, first + kP2Grab);
    for (int64_t base = first; base < last; base += 32) {
      const int64_t vi = base + lane;
      uint32_t m[SW];
#pragma unroll
      for (int w = 0; w < SW; ++w) m[w] = 0;
      bool warp_row = false;
      int64_t nch = 0;
      if (vi < last) {
        const int32_t v = (int32_t)vi;
        const int64_t b = g.nindex[v], e = g.nindex[v + 1];
        const int64_t ab = g.aoff[v], ae = g.aoff[v + 1];
        const int64_t tot = (e - b) + (ae - ab);
        if (tot > kP2Huge) {
          nch = (tot + kP2Chunk - 1) / kP2Chunk;
        } else {
          if (p2_in(filt, v)) p2_or(m, mask, v);
          if (tot > kP2Short) {
            warp_row = true;
          } else {
            // four positions per step: their ids, then their filter bits,
            // then the masks of those that pass, all loads of a step in flight
            const bool dead = g.dead[v] != 0;
            const int64_t nb = e - b;
            for (int64_t k0 = 0; k0 < tot; k0 += 4) {
              int32_t y[4];
#pragma unroll
              for (int q = 0; q < 4; ++q) {
                const int64_t k = k0 + q;
                y[q] = -1;
                if (k < nb) {
                  if (!dead || live_at(g.live, b + k)) y[q] = __ldg(g.nlist + b + k);
                } else if (k < tot) {
                  y[q] = g.aadj[ab + (k - nb)];
                }
              }
#pragma unroll
              for (int q = 0; q < 4; ++q)
                if (y[q] >= 0 && !p2_in(filt, y[q])) y[q] = -1;
#pragma unroll
              for (int q = 0; q < 4; ++q)
                if (y[q] >= 0) p2_or(m, mask, y[q]);
            }
          }
        }
      }
      // huge rows of these 32 vertices: one slot each and their chunk
      // tasks, one atomic per warp for each
      const unsigned hm = __ballot_sync(0xffffffffu, nch > 0);
      if (hm) {
        int64_t incl = nch;
        for (int o = 1; o < 32; o <<= 1) {
          const int64_t t = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += t;
        }
        const int64_t wtot = __shfl_sync(0xffffffffu, incl, 31);
        unsigned long long sbase = 0, tbase = 0;
        if (lane == 0) {
          sbase = atomicAdd(wk.nhuge, (unsigned long long)__popc(hm));
          tbase = atomicAdd(wk.ntasks, (unsigned long long)wtot);
        }
        sbase = __shfl_sync(0xffffffffu, sbase, 0);
        tbase = __shfl_sync(0xffffffffu, tbase, 0);
        if (nch > 0) {
          const int64_t slot = (int64_t)sbase + __popc(hm & ((1u << lane) - 1u));
          const int64_t t0 = (int64_t)tbase + incl - nch;
          if (slot < wk.hcap) {
            wk.huge[slot] = (int32_t)vi;
            for (int64_t c = 0; c < nch; ++c)
              if (t0 + c < wk.tcap) wk.tasks[t0 + c] = (slot << 32) | c;
          }
        }
      }
      unsigned wl = __ballot_sync(0xffffffffu, warp_row);
      while (wl) {
        const int src = __ffs(wl) - 1;
        wl &= wl - 1;
        const int32_t x = (int32_t)(base + src);
        const int64_t tot = (g.nindex[x + 1] - g.nindex[x]) + (g.aoff[x + 1] - g.aoff[x]);
        uint32_t r[SW];
#pragma unroll
        for (int w = 0; w < SW; ++w) r[w] = 0;
        p2_warp_span(g, mask, filt, x, 0, tot, r);
        p2_warp_or(r);
        if (lane == src)
#pragma unroll
          for (int w = 0; w < SW; ++w) m[w] |= r[w];
      }
      p2_count_lanes(m, acc);
    }
  }
  p2_flush(acc, s_cnt, counts);
}

// ---- bulk staging of row spans (cp.async.bulk, completion on an mbarrier) ----
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// One thread: bytes expected on bar, then the copy global -> shared that
// completes them.  dst, src and bytes are multiples of 16 (callers check).
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
// Wait for the phase of bar with parity `parity`; false after `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int64_t limit) {
  for (int64_t it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

constexpr int kP2Sub = 512;                  // positions per staged span of a chunk task
constexpr int kP2SubBuf = kP2Sub + 8;        // room for the 16-byte rounding at both ends
constexpr int64_t kBulkPolls = (int64_t)1 << 22;

// A staged span: positions [p0, p1) of row x; the base entries in
// [p0, min(p1, nb)) sit in the buffer from entry `lead` on (copied from the
// 16-byte boundary at or below their address), the rest are added entries.
struct P2Span {
  int64_t slot, p0, p1, b, nb, ab;
  int32_t x, lead;
  bool dead, copied, valid;
};

// Chunk tasks of the huge rows, one warp each, split into spans of kP2Sub
// positions; the chunk's OR goes to racc of its row's slot.  With `bulk`,
// the base-row ids of the warp's next span are copied into shared memory by
// the bulk-copy engine while the current span is processed (two buffers,
// one mbarrier each); every copy starts on a 16-byte boundary of the row
// array (rounded down, its length rounded up; the array carries 16 bytes of
// padding).  Without it the ids are read with plain loads.  (At R-MAT scale
// 26 both take the same time: the span's filter and mask loads, which
// depend on the ids, bound the pass.)  A wait that runs out sets *err and
// the warp stops, after a bounded wait for its copy still in flight.
template <int SW>
__global__ void __launch_bounds__(256) k_p2_huge(GraphView g, const uint32_t* mask, const uint32_t* filt, P2Work wk,
                                                 uint32_t* racc, bool bulk, unsigned long long* err) {
  extern __shared__ __align__(16) unsigned char p2_smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nwb = blockDim.x >> 5;
  int32_t* bufs = reinterpret_cast<int32_t*>(p2_smem) + (int64_t)wib * 2 * kP2SubBuf;
  uint64_t* bars = reinterpret_cast<uint64_t*>(p2_smem + (size_t)nwb * 2 * kP2SubBuf * 4) + wib * 2;
  if (lane == 0) {
    mbar_init(bars, 1);
    mbar_init(bars + 1, 1);
    mbar_init_fence();
  }
  __syncwarp();
  uint32_t parity[2] = {0u, 0u};
  const int64_t total = min((int64_t)*wk.ntasks, wk.tcap);
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  // span after (t, sub) in this warp's sequence: next sub of the task, else
  // the first of the warp's next task
  auto describe = [&](int64_t t, int64_t sub) {
    P2Span sp{};
    sp.valid = false;
    if (t >= total) return sp;
    const int64_t task = wk.tasks[t];
    const int64_t i = task >> 32, c = task & 0xffffffffll;
    if (i >= wk.hcap) return sp;   // never: hcap bounds the rows over kP2Huge positions
    const int32_t x = wk.huge[i];
    const int64_t b = g.nindex[x], nb = g.nindex[x + 1] - b;
    const int64_t ab = g.aoff[x], tot = nb + (g.aoff[x + 1] - ab);
    const int64_t c0 = c * kP2Chunk, c1 = min(tot, c0 + kP2Chunk);
    sp.p0 = c0 + sub * kP2Sub;
    if (sp.p0 >= c1) return sp;
    sp.p1 = min(c1, sp.p0 + kP2Sub);
    sp.slot = i;
    sp.x = x;
    sp.b = b;
    sp.nb = nb;
    sp.ab = ab;
    sp.dead = g.dead[x] != 0;
    sp.valid = true;
    return sp;
  };
  auto issue = [&](P2Span& sp, int buf) {
    sp.copied = false;
    sp.lead = 0;
    const int64_t e = min(sp.p1, sp.nb);
    if (!bulk || sp.p0 >= e) return;
    const uintptr_t a = reinterpret_cast<uintptr_t>(g.nlist + sp.b + sp.p0);
    const uintptr_t a0 = a & ~(uintptr_t)15;
    const uint32_t bytes = (uint32_t)(((a + 4 * (uintptr_t)(e - sp.p0) - a0) + 15) & ~(uintptr_t)15);
    int32_t* dst = bufs + buf * kP2SubBuf;
    if ((reinterpret_cast<uintptr_t>(dst) & 15) != 0 || bytes > 4u * kP2SubBuf) return;   // never: plain loads then
    sp.lead = (int32_t)((a - a0) >> 2);
    sp.copied = true;
    if (lane == 0) bulk_load(dst, reinterpret_cast<const void*>(a0), bytes, bars + buf);
  };
  int64_t t = warp_id(), sub = 0;
  P2Span cur = describe(t, sub);
  int slot = 0;
  if (cur.valid) issue(cur, slot);
  uint32_t r[SW];
#pragma unroll
  for (int w = 0; w < SW; ++w) r[w] = 0;
  bool failed = false;
  while (cur.valid) {
    int64_t nt = t, ns = sub + 1;
    P2Span nxt = describe(nt, ns);
    if (!nxt.valid) {
      nt = t + nw;
      ns = 0;
      nxt = describe(nt, ns);
    }
    if (nxt.valid) issue(nxt, slot ^ 1);
    if (cur.copied) {
      if (!mbar_wait(bars + slot, parity[slot], kBulkPolls)) {
        failed = true;
        if (lane == 0) atomicExch(err, 1ull);
        break;
      }
      parity[slot] ^= 1u;
    }
    const int32_t* sb = bufs + slot * kP2SubBuf + cur.lead;
    const int64_t e = min(cur.p1, cur.nb);
    for (int64_t k0 = cur.p0 + lane; k0 < cur.p1; k0 += 128) {
      int32_t y[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int64_t k = k0 + 32 * q;
        y[q] = -1;
        if (k < cur.p1) {
          if (k < e) {
            if (!cur.dead || live_at(g.live, cur.b + k))
              y[q] = cur.copied ? sb[k - cur.p0] : __ldg(g.nlist + cur.b + k);
          } else {
            y[q] = g.aadj[cur.ab + (k - cur.nb)];
          }
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (y[q] >= 0 && !p2_in(filt, y[q])) y[q] = -1;
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (y[q] >= 0) p2_or(r, mask, y[q]);
    }
    __syncwarp();
    // the task's OR goes out after its last span
    if (!nxt.valid || nt != t) {
      p2_warp_or(r);
#pragma unroll
      for (int w = 0; w < SW; ++w) {
        if (lane == w && r[w]) atomicOr(racc + cur.slot * SW + w, r[w]);
        r[w] = 0;
      }
    }
    cur = nxt;
    t = nt;
    sub = ns;
    slot ^= 1;
  }
  if (failed && cur.valid) {
    // the copy of the span after the one that ran out may still be in flight
    int64_t nt = t, ns = sub + 1;
    P2Span nxt = describe(nt, ns);
    if (!nxt.valid) nxt = describe(t + nw, 0);
    if (nxt.valid && nxt.p0 < min(nxt.p1, nxt.nb)) mbar_wait(bars + (slot ^ 1), parity[slot ^ 1], kBulkPolls);
  }
}

// The huge rows' own masks plus their chunks' ORs, counted.
template <int SW>
__global__ void __launch_bounds__(256) k_p2_huge_count(const uint32_t* mask, const int32_t* huge,
                                                       const unsigned long long* nhuge, int64_t hcap,
                                                       const uint32_t* racc, unsigned long long* counts) {
  __shared__ unsigned long long s_cnt[32 * SW];
  for (int i = threadIdx.x; i < 32 * SW; i += blockDim.x) s_cnt[i] = 0;
  __syncthreads();
  uint32_t acc[SW];
#pragma unroll
  for (int w = 0; w < SW; ++w) acc[w] = 0;
  const int64_t nh = min((int64_t)*nhuge, hcap);
  const int64_t step = ((int64_t)gridDim.x * blockDim.x);
  for (int64_t base = warp_id() * 32; base < nh; base += step) {
    const int64_t i = base + (threadIdx.x & 31);
    uint32_t m[SW];
#pragma unroll
    for (int w = 0; w < SW; ++w) m[w] = 0;
    if (i < nh) {
      p2_or(m, mask, huge[i]);
#pragma unroll
      for (int w = 0; w < SW; ++w) m[w] |= racc[i * SW + w];
    }
    p2_count_lanes(m, acc);
  }
  p2_flush(acc, s_cnt, counts);
}

__global__ void k_p2_store(const unsigned long long* counts, const int32_t* grp, int k, int64_t* lens) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < k) lens[grp[j]] = (int64_t)counts[j];
}


__global__ void k_cand_lens(GraphView g, const int32_t* cands, int64_t nct, int64_t* lens) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nct) lens[k] = row_len(g, cands[k]);
}

// Growth of MAX_CSR_ELEMENTS while packing rows in order
// (src/misfit/misfit.cu:565-568): whenever a row's end offset reaches the
// limit, the limit becomes 1.5x that end offset.  io[0] = limit in/out,
// io[1] = packed total out.
// Algorithmic accounting of one sub-batch (profiler bit 4): the packed
// volume (sum of the exact row lengths) and the degrees of the mapped rows.
__global__ void k_acct(const int64_t* lens, int64_t rows, const int32_t* seeds, int64_t ns, const int32_t* cands,
                       const int32_t* deg, unsigned long long* acc) {
  unsigned long long a = 0, d = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x) {
    a += (unsigned long long)lens[i];
    d += (unsigned long long)deg[i < ns ? seeds[i] : cands[i - ns]];
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    d += __shfl_down_sync(0xffffffffu, d, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (a) atomicAdd(acc, a);
    if (d) atomicAdd(acc + 1, d);
  }
}

__global__ void k_growth(const int64_t* pex, int64_t rows, int64_t* io) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int64_t cur = io[0];
  int64_t start = 0;
  while (start < rows) {
    int64_t lo = start, hi = rows;  // first i >= start with pex[i+1] >= cur
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (pex[mid + 1] >= cur) hi = mid; else lo = mid + 1;
    }
    if (lo >= rows) break;
    const int64_t end = pex[lo + 1];
    cur = (int64_t)((double)(uint64_t)end * 1.5);
    start = lo + 1;
  }
  io[0] = cur;
  io[1] = pex[rows];
}

// ---- clustering ------------------------------------------------------------------

// ---- first-hit row searches --------------------------------------------------------
// First position j of row(x) (in order) whose element y satisfies a predicate,
// for every x of a list.  A warp scans the first `bound` positions; rows
// still unresolved are finished by a load-balanced pass that keeps the
// minimum hit position per row (atomicMin), so hub rows are spread over the
// GPU while short rows stop at their first hit.

constexpr unsigned long long kNoPos = ~0ull;

// The element already carries a cluster id, tested on a bitmap (bit y set
// <=> cid[y] != -1) built before the clustering read, while the ids do not
// change: the first-hit searches read 1 bit per element from an array 32x
// smaller than the ids, which stays in L1, instead of a 4-byte id from L2.
struct HasCidBit {
  const uint32_t* bits;
  __device__ __forceinline__ bool operator()(int32_t y) const { return (__ldg(bits + (y >> 5)) >> (y & 31)) & 1u; }
};

// One warp per 1,024 vertices (32 bitmap words): eight coalesced 16-byte
// loads per lane, four ids each; the eight lanes that share a word OR their
// nibbles together, and lane L stores the warp's word L.
constexpr int64_t kCidBitsPerWarp = 1024;

__global__ void k_cid_bits(const int32_t* cid, int32_t n, uint32_t* bits) {
  pdl_wait();
  pdl_trigger();
  const int lane = threadIdx.x & 31;
  const int64_t v0 = warp_id() * kCidBitsPerWarp;
  if (v0 >= n) return;   // the whole warp
  uint32_t mine = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int64_t v = v0 + k * 128 + lane * 4;
    uint32_t nib = 0;
    if (v + 3 < n) {
      const int4 x = *reinterpret_cast<const int4*>(cid + v);
      nib = (uint32_t)(x.x != -1) | (uint32_t)(x.y != -1) << 1 | (uint32_t)(x.z != -1) << 2 |
            (uint32_t)(x.w != -1) << 3;
    } else {
      for (int t = 0; t < 4; ++t)
        if (v + t < n && cid[v + t] != -1) nib |= 1u << t;
    }
    // word k * 4 + lane / 8 of the warp's span, nibble lane % 8
    uint32_t part = nib << ((lane & 7) * 4);
    part |= __shfl_xor_sync(0xffffffffu, part, 1);
    part |= __shfl_xor_sync(0xffffffffu, part, 2);
    part |= __shfl_xor_sync(0xffffffffu, part, 4);
    const uint32_t word = __shfl_sync(0xffffffffu, part, (lane & 3) * 8);
    if ((lane >> 2) == k) mine = word;
  }
  const int64_t wi = (v0 >> 5) + lane;
  if (wi < ((int64_t)n + 31) / 32) bits[wi] = mine;
}

// ---- first-hit searches with device-side counts ---------------------------------
// Three levels, none of which needs the host to know a count:
//   1. one thread per row probes the first kProbe positions, eight at a time
//      (their loads, then their tests);
//   2. rows still open go to a queue; a fixed grid of warps scans positions
//      kProbe .. bound of each (a tuning setting, 256 by default);
//   3. rows still open get chunks of kFirstChunk positions from one packed
//      64-bit counter ((rows << 40) | chunks), so that the chunk bases grow
//      with the row slots; a fixed grid of warps takes chunks, finds the row
//      by binary search over the bases and keeps the minimum hit position.
// The same chunk queue drives the marking of the need seeds' neighbours.
constexpr int kProbe = 32;
constexpr int64_t kFirstChunk = 256;
constexpr int kChunkShift = 40;
constexpr unsigned long long kChunkMask = (1ull << kChunkShift) - 1;

struct ChunkQueue {
  int32_t* idx;                    // caller's row index
  int32_t* v;                      // row vertex
  int64_t* base;                   // first chunk of the row
  unsigned long long* packed;      // (rows << 40) | chunks
};

__device__ __forceinline__ void cq_push(const ChunkQueue& q, int32_t idx, int32_t v, int64_t chunks) {
  const unsigned long long old = atomicAdd(q.packed, (1ull << kChunkShift) | (unsigned long long)chunks);
  const int64_t slot = (int64_t)(old >> kChunkShift);
  q.idx[slot] = idx;
  q.v[slot] = v;
  q.base[slot] = (int64_t)(old & kChunkMask);
}

// Slot of chunk c: the last slot whose base is <= c (bases grow with slots).
// Warp-cooperative (all lanes call it with the same c): a 32-way search, so
// the dependent loads are log32(rows) rounds instead of log2(rows).
__device__ __forceinline__ int64_t cq_slot(const ChunkQueue& q, int64_t rows, int64_t c) {
  const int lane = threadIdx.x & 31;
  int64_t lo = 0, hi = rows;
  while (hi - lo > 1) {
    const int64_t step = (hi - lo + 31) >> 5;
    const int64_t idx = lo + (int64_t)lane * step;
    const unsigned m = __ballot_sync(0xffffffffu, idx < hi && q.base[idx] <= c);
    lo += (int64_t)(31 - __clz(m)) * step;
    const int64_t nh = lo + step;
    hi = nh < hi ? nh : hi;
  }
  return lo;
}

// Warp-cooperative: first position k in [k0, k1) of row(x) (nb base
// positions, then the added entries) whose element is live and satisfies
// pred, or -1.  Steps of one, two, then four 32-position windows: the
// windows of a step are loaded before any is tested, so each lane has up to
// four element loads (then four predicate loads) in flight; the answer is
// the lowest hit of the first window that has one.
template <class P>
__device__ __forceinline__ int64_t warp_first_range(const GraphView& g, int32_t x, int64_t nb, int64_t k0, int64_t k1,
                                                    P pred) {
  const int lane = threadIdx.x & 31;
  const int64_t b0 = g.nindex[x];
  const int64_t a0 = g.aoff[x];
  const bool filt = g.dead[x] != 0;
  int nwin = 1;   // windows per step: 1, 2, then 4 (a hit is often early)
  for (int64_t base = k0; base < k1; base += 32 * nwin, nwin = nwin < 4 ? 2 * nwin : 4) {
    int32_t y[4];
    bool live[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t k = base + 32 * q + lane;
      y[q] = -1;
      live[q] = false;
      if (q < nwin && k < k1) {
        if (k < nb) {
          y[q] = __ldg(g.nlist + b0 + k);
          live[q] = !filt || live_at(g.live, b0 + k);
        } else {
          y[q] = g.aadj[a0 + (k - nb)];
          live[q] = true;
        }
      }
    }
    bool ok[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) ok[q] = live[q] && pred(y[q]);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const unsigned m = __ballot_sync(0xffffffffu, ok[q]);
      if (m) return base + 32 * q + (__ffs(m) - 1);
    }
  }
  return -1;
}

struct FirstQueues {
  int32_t* mid_idx;
  int32_t* mid_v;
  unsigned long long* mid_count;
  ChunkQueue rest;
  int64_t bound;    // positions the warp level covers (kProbe .. bound); a tuning setting
};

template <class P>
__global__ void k_first_probe(GraphView g, const int32_t* list, const unsigned long long* dcnt, P pred,
                              unsigned long long* firstpos, FirstQueues q) {
  pdl_wait();
  pdl_trigger();
  const int64_t cnt = (int64_t)*dcnt;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t x = list[i];
    const int64_t nb = g.nindex[x + 1] - g.nindex[x];
    const int64_t np = nb + (g.aoff[x + 1] - g.aoff[x]);
    const int64_t lim = np < kProbe ? np : kProbe;
    const int64_t b0 = g.nindex[x];
    const int64_t a0 = g.aoff[x];
    const bool filt = g.dead[x] != 0;
    unsigned long long fp = kNoPos;
    for (int64_t k0 = 0; k0 < lim && fp == kNoPos; k0 += 8) {
      int32_t y[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int64_t k = k0 + t;
        y[t] = -1;
        if (k < lim) {
          if (k < nb) {
            if (!filt || live_at(g.live, b0 + k)) y[t] = __ldg(g.nlist + b0 + k);
          } else {
            y[t] = g.aadj[a0 + (k - nb)];
          }
        }
      }
      bool ok[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) ok[t] = y[t] >= 0 && pred(y[t]);
#pragma unroll
      for (int t = 7; t >= 0; --t)
        if (ok[t]) fp = (unsigned long long)(k0 + t);
    }
    firstpos[i] = fp;
    if (fp == kNoPos && np > kProbe) {
      const unsigned long long u = atomicAdd(q.mid_count, 1ull);
      q.mid_idx[u] = (int32_t)i;
      q.mid_v[u] = x;
    }
  }
}

template <class P>
__global__ void k_first_warp(GraphView g, P pred, unsigned long long* firstpos, FirstQueues q) {
  pdl_wait();
  pdl_trigger();
  const int lane = threadIdx.x & 31;
  const int64_t nmid = (int64_t)*q.mid_count;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = warp_id(); w < nmid; w += nw) {
    const int32_t i = q.mid_idx[w];
    const int32_t x = q.mid_v[w];
    const int64_t nb = g.nindex[x + 1] - g.nindex[x];
    const int64_t np = nb + (g.aoff[x + 1] - g.aoff[x]);
    const int64_t lim = np < q.bound ? np : q.bound;
    const int64_t hit = warp_first_range(g, x, nb, kProbe, lim, pred);
    if (hit >= 0) {
      if (lane == 0) firstpos[i] = (unsigned long long)hit;
    } else if (np > q.bound && lane == 0) {
      cq_push(q.rest, i, x, (np - q.bound + kFirstChunk - 1) / kFirstChunk);
    }
  }
}

template <class P>
__global__ void k_first_chunks(GraphView g, P pred, unsigned long long* firstpos, FirstQueues q) {
  pdl_wait();
  pdl_trigger();
  const int lane = threadIdx.x & 31;
  const unsigned long long pk = *q.rest.packed;
  const int64_t rows = (int64_t)(pk >> kChunkShift), chunks = (int64_t)(pk & kChunkMask);
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c = warp_id(); c < chunks; c += nw) {
    const int64_t slot = cq_slot(q.rest, rows, c);
    const int32_t i = q.rest.idx[slot];
    const int32_t x = q.rest.v[slot];
    const int64_t p0 = q.bound + (c - q.rest.base[slot]) * kFirstChunk;
    // skip when an earlier position already hit; one lane reads, so that the
    // whole warp takes the same branch while other warps lower the value
    unsigned long long fp = 0;
    if (lane == 0) fp = *(volatile const unsigned long long*)(firstpos + i);
    fp = __shfl_sync(0xffffffffu, fp, 0);
    if (fp <= (unsigned long long)p0) continue;
    const int64_t nb = g.nindex[x + 1] - g.nindex[x];
    const int64_t np = nb + (g.aoff[x + 1] - g.aoff[x]);
    const int64_t end = min(p0 + kFirstChunk, np);
    const int64_t hit = warp_first_range(g, x, nb, p0, end, pred);
    if (hit >= 0 && lane == 0) atomicMin(firstpos + i, (unsigned long long)hit);
  }
}

// Per row: early return when the row's own vertex already has an id
// (src/misfit/misfit.cu:224); the other rows are listed (row index and
// vertex) for the first-existing-id searches.
__global__ void k_row_skip(const int32_t* seeds, int64_t ns, const int32_t* cands, int64_t nct, const int32_t* cid,
                           int32_t* rowcid, uint8_t* creates, int32_t* live_i, int32_t* live_v,
                           unsigned long long* nlive) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ns + nct) return;
  const int32_t x = i < ns ? seeds[i] : cands[i - ns];
  if (cid[x] != -1) {
    rowcid[i] = kSkip;
    creates[i] = 0;
    return;
  }
  const unsigned long long k = atomicAdd(nlive, 1ull);
  live_i[k] = (int32_t)i;
  live_v[k] = x;
}

// The first existing id of row(x) in order, if any; seeds without one go on
// to their hop-2 part (`need`), everything else without one creates a cluster.
__global__ void k_live_decide(GraphView g, const int32_t* live_i, const int32_t* live_v,
                              const unsigned long long* dcnt, int64_t ns, const unsigned long long* firstpos,
                              const int32_t* cid, int32_t* rowcid, uint8_t* creates, const int32_t* seeds,
                              int32_t* need, int32_t* needv, unsigned long long* nneed, ChunkQueue mq) {
  pdl_wait();
  pdl_trigger();
  const int64_t cnt = (int64_t)*dcnt;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t i = live_i[k];
    const int32_t x = live_v[k];
    const unsigned long long fp = firstpos[k];
    if (fp != kNoPos) {
      rowcid[i] = cid[row_elem(g, x, (int64_t)fp, g.nindex[x + 1] - g.nindex[x])];
      creates[i] = 0;
      continue;
    }
    rowcid[i] = -1;
    creates[i] = 1;
    if (i < ns) {
      const unsigned long long u = atomicAdd(nneed, 1ull);
      need[u] = i;
      const int32_t s = seeds[i];
      needv[u] = s;
      const int64_t np = row_positions(g, s);
      if (np > 0) cq_push(mq, (int32_t)u, s, (np + kFirstChunk - 1) / kFirstChunk);
    }
  }
}

// A seed row is [s] ++ row(s) ++ row(h1) ++ row(h2) ++ ... (h over row(s) in
// order): after row(s), its first existing id is f1(h) of the first h of
// row(s) that has one, f1(h) being the id of the first element of row(h)
// with an id.  f1 is computed for the neighbours of the seeds that need it.
__global__ void k_mark_need(GraphView g, ChunkQueue mq, uint32_t epoch, uint32_t* nmark, int32_t* list,
                            unsigned long long* count) {
  pdl_wait();
  pdl_trigger();
  const int lane = threadIdx.x & 31;
  const unsigned long long pk = *mq.packed;
  const int64_t rows = (int64_t)(pk >> kChunkShift), chunks = (int64_t)(pk & kChunkMask);
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c = warp_id(); c < chunks; c += nw) {
    const int64_t slot = cq_slot(mq, rows, c);
    const int32_t x = mq.v[slot];
    const int64_t p0 = (c - mq.base[slot]) * kFirstChunk;
    const int64_t nb = g.nindex[x + 1] - g.nindex[x];
    const int64_t end = min(p0 + kFirstChunk, nb + (g.aoff[x + 1] - g.aoff[x]));
    for (int64_t k = p0 + lane; k < end; k += 32) {
      const int32_t y = row_elem(g, x, k, nb);
      if (y >= 0 && nmark[y] != epoch && atomicExch(nmark + y, epoch) != epoch) list[atomicAdd(count, 1ull)] = y;
    }
  }
}

__global__ void k_f1_finish(GraphView g, const int32_t* list, const unsigned long long* dcnt,
                            const unsigned long long* firstpos, const int32_t* cid, int32_t* f1) {
  pdl_wait();
  pdl_trigger();
  const int64_t cnt = (int64_t)*dcnt;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t x = list[i];
    const unsigned long long fp = firstpos[i];
    f1[x] = fp == kNoPos ? -1 : cid[row_elem(g, x, (int64_t)fp, g.nindex[x + 1] - g.nindex[x])];
  }
}

struct HasF1 {    // the element's own row holds an element with a cluster id
  const int32_t* f1;
  __device__ __forceinline__ bool operator()(int32_t y) const { return f1[y] != -1; }
};

__global__ void k_need_decide(GraphView g, const int32_t* need, const int32_t* needv, const unsigned long long* dcnt,
                              const unsigned long long* firstpos, const int32_t* f1, int32_t* rowcid,
                              uint8_t* creates) {
  pdl_wait();
  pdl_trigger();
  const int64_t cnt = (int64_t)*dcnt;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long fp = firstpos[k];
    if (fp == kNoPos) continue;
    const int32_t s = needv[k];
    const int32_t h = row_elem(g, s, (int64_t)fp, g.nindex[s + 1] - g.nindex[s]);
    rowcid[need[k]] = f1[h];
    creates[need[k]] = 0;
  }
}

// New cluster ids by ascending row index; the seed rows that write (not
// skipped) also take phase 1 of the clustering write here: bval[s] = max tag
// of those rows with s = their own vertex (the rest of phase 1 is
// k_lb_push_seed).  A skipped row stays skipped whatever its id.
__global__ void k_new_ids(int64_t rows, const int64_t* pos, int32_t* rowcid, const int32_t* seeds, int64_t ns,
                          uint32_t epoch, uint32_t* bval) {
  pdl_wait();
  pdl_trigger();
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows) return;
  const int32_t rc = rowcid[i];
  if (rc == -1) rowcid[i] = (int32_t)pos[i];
  if (i < ns && rc != kSkip) atomicMax(bval + seeds[i], (epoch << kRowBits) | (uint32_t)i);
}

// The pushes are reductions whose results are not read back, so they issue
// as fire-and-forget RED operations.  Within one launch a tag word only
// grows, so a plain read that already shows the pushed tag (or a larger one)
// proves the push cannot change it and it is skipped: rows of R-MAT
// sub-batches share their hub neighbours, and without the filter every
// hop-1 row's push to a hub serialises on that one address.
__device__ __forceinline__ void push_w(uint32_t* wval, int32_t y, uint32_t tag) {
  if (wval[y] < tag) atomicMax(wval + y, tag);
}

// Phase 1: bval[y] = max tag of the non-skipped seed rows with y in {s} u
// row(s): the seeds themselves in k_new_ids, their rows here.

__global__ void k_lb_push_seed(GraphView g, const int32_t* seeds, const int64_t* offs, int64_t ns, uint32_t epoch,
                               uint32_t* bval, unsigned long long* work) {
  pdl_wait();
  pdl_trigger();
  const int64_t vis = lb_rows(g, seeds, offs, ns, [&](int64_t i, int32_t, int32_t y) {
    push_w(bval, y, (epoch << kRowBits) | (uint32_t)i);
  });
  add_work(work, vis);
}



// Phase 2: wval[y] = max over x with y in {x} u row(x) of bval[x] (the 2-hop
// reach of the seed rows), and the candidate rows' own tags over row(c).
// Every vertex of list a (cnt_a) and list b (cnt_b) pushes its own phase-1
// tag, when it has one of this epoch, to itself (one launch for the seeds
// and the hop-1 vertices).
__global__ void k_self_push(const int32_t* a, int64_t cnt_a, const int32_t* b, int64_t cnt_b, uint32_t epoch,
                            const uint32_t* bval, uint32_t* wval) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt_a + cnt_b) return;
  const int32_t x = i < cnt_a ? a[i] : b[i - cnt_a];
  const uint32_t t = bval[x];
  if ((t >> kRowBits) == epoch) push_w(wval, x, t);
}

__global__ void __launch_bounds__(kLbThreads, MF_LB_MIN_BLOCKS) k_lb_push_hop(GraphView g, const int32_t* list, const int64_t* offs,
                                                            int64_t cnt, uint32_t epoch, const uint32_t* bval,
                                                            uint32_t* wval, unsigned long long* work) {
  pdl_wait();
  pdl_trigger();
  // the row's tag is staged once per row with the row's metadata
  const int64_t vis = lb_rows_aux(
      g, list, offs, cnt, [&](int64_t, int32_t x) { return bval[x]; },
      [&](int64_t, int32_t, int32_t y, uint32_t t) { push_w(wval, y, t); });
  add_work(work, vis);
}

__global__ void k_lb_push_cand(GraphView g, const int32_t* cands, const int64_t* offs, int64_t nct, int64_t ns,
                               uint32_t epoch, uint32_t* wval, unsigned long long* work) {
  pdl_wait();
  pdl_trigger();
  const int64_t vis = lb_rows(g, cands, offs, nct, [&](int64_t i, int32_t, int32_t y) {
    push_w(wval, y, (epoch << kRowBits) | (uint32_t)(ns + i));
  });
  add_work(work, vis);
}

// Pull form of the candidate writes (symmetric graphs with sorted base rows).
// The candidate rows that write are the non-skipped ones, and their tags
// grow with the candidate's vertex id (candidates are packed in ascending
// id), so the last writer of y among them is its largest-id non-skipped
// candidate neighbour: the added part of row(y) is scanned, then the base
// part from its end until the first such neighbour.  That tag dominates every
// seed-row tag; without one, the pushed seed-row tag (wval) decides.
// One thread per vertex; rows longer than a.pull_long positions (a tuning
// setting, 2048 by default) go to a list that k_pull_cand_long finishes with
// one warp per row.

struct PullArgs {
  GraphView g;
  const int32_t* v2i;
  const int32_t* rowcid;
  const uint32_t* ncbits;         // bit c set <=> c is a non-skipped candidate
  int64_t ns;
  const uint32_t* wval;
  uint32_t epoch;
  int32_t* cid;
  int32_t* longv;                 // rows left for the warp pass
  unsigned long long* nlong;
  unsigned long long* work;
  int64_t pull_long;              // rows longer than this go to the warp pass
};

__device__ __forceinline__ bool pull_nonskip(const PullArgs& a, int32_t c) {
  return (__ldg(a.ncbits + (c >> 5)) >> (c & 31)) & 1u;
}

// Bits of the non-skipped candidates (rows ns .. ns+nct-1) for the pull pass.
__global__ void k_cand_bits(const int32_t* cands, int64_t nct, int64_t ns, const int32_t* rowcid, uint32_t* bits) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nct || rowcid[ns + i] == kSkip) return;
  const int32_t c = cands[i];
  atomicOr(bits + (c >> 5), 1u << (c & 31));
}

__device__ __forceinline__ void pull_finish(const PullArgs& a, int32_t y, int32_t best) {
  if (best >= 0) {
    a.cid[y] = a.rowcid[a.v2i[best]];
  } else {
    const uint32_t t = a.wval[y];
    if ((t >> kRowBits) == a.epoch) a.cid[y] = a.rowcid[t & kRowMask];
  }
}

__global__ void k_pull_cand(PullArgs a) {
  pdl_wait();
  pdl_trigger();
  const GraphView& g = a.g;
  const int64_t yi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t visited = 0;
  if (yi < g.n) {
    const int32_t y = (int32_t)yi;
    const int64_t b = g.nindex[y], e = g.nindex[y + 1];
    const int64_t ab = g.aoff[y], ae = g.aoff[y + 1];
    if ((e - b) + (ae - ab) > a.pull_long) {
      a.longv[atomicAdd(a.nlong, 1ull)] = y;
    } else {
      int32_t best = -1;
      for (int64_t k = ab; k < ae; ++k) {
        const int32_t c = g.aadj[k];
        ++visited;
        if (c > best && pull_nonskip(a, c)) best = c;
      }
      const bool filt = g.dead[y] != 0;
      for (int64_t k = e - 1; k >= b; --k) {
        const int32_t c = __ldg(g.nlist + k);
        ++visited;
        if (c <= best) break;
        if (filt && !live_at(g.live, k)) continue;
        if (pull_nonskip(a, c)) {
          best = c;
          break;
        }
      }
      pull_finish(a, y, best);
    }
  }
  add_work(a.work, visited);
}

// The long rows: the warp takes the maximum over the added part, then walks
// the sorted base part from its end 32 positions at a time.  Scanning from
// the end, the positions with c > best form a prefix of the lanes; the
// first of them (lowest lane) that is live and non-skipped is the answer,
// and a prefix shorter than 32 lanes ends the walk.
__global__ void k_pull_cand_long(PullArgs a) {
  pdl_wait();
  pdl_trigger();
  const GraphView& g = a.g;
  const int lane = threadIdx.x & 31;
  const int64_t nl = (int64_t)*a.nlong;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int64_t visited = 0;
  for (int64_t w = warp_id(); w < nl; w += nw) {
    const int32_t y = a.longv[w];
    const int64_t b = g.nindex[y], e = g.nindex[y + 1];
    const int64_t ab = g.aoff[y], ae = g.aoff[y + 1];
    int32_t best = -1;
    for (int64_t k = ab + lane; k < ae; k += 32) {
      const int32_t c = g.aadj[k];
      ++visited;
      if (c > best && pull_nonskip(a, c)) best = c;
    }
    for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
    const bool filt = g.dead[y] != 0;
    for (int64_t k0 = e - 1; k0 >= b; k0 -= 32) {
      const int64_t k = k0 - lane;
      int32_t c = -1;
      bool above = false, hit = false;
      if (k >= b) {
        c = __ldg(g.nlist + k);
        ++visited;
        above = c > best;
        hit = above && (!filt || live_at(g.live, k)) && pull_nonskip(a, c);
      }
      const unsigned hm = __ballot_sync(0xffffffffu, hit);
      if (hm) {
        best = __shfl_sync(0xffffffffu, c, __ffs(hm) - 1);
        break;
      }
      if (__ballot_sync(0xffffffffu, above) != 0xffffffffu) break;  // the rest is <= best
    }
    if (lane == 0) pull_finish(a, y, best);
  }
  add_work(a.work, visited);
}

// cid[y] = id of the row that wrote y last, for every y tagged this epoch.
__global__ void k_finalize_all(const uint32_t* wval, int32_t n, uint32_t epoch, const int32_t* rowcid, int32_t* cid) {
  pdl_wait();
  pdl_trigger();
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t x0 = q * 4;
  if (x0 >= n) return;
  if (x0 + 4 <= n) {
    const uint4 t = reinterpret_cast<const uint4*>(wval)[q];
    if ((t.x >> kRowBits) == epoch) cid[x0 + 0] = rowcid[t.x & kRowMask];
    if ((t.y >> kRowBits) == epoch) cid[x0 + 1] = rowcid[t.y & kRowMask];
    if ((t.z >> kRowBits) == epoch) cid[x0 + 2] = rowcid[t.z & kRowMask];
    if ((t.w >> kRowBits) == epoch) cid[x0 + 3] = rowcid[t.w & kRowMask];
  } else {
    for (int64_t x = x0; x < n; ++x) {
      const uint32_t t = wval[x];
      if ((t >> kRowBits) == epoch) cid[x] = rowcid[t & kRowMask];
    }
  }
}

// ---- assignment and order ------------------------------------------------------------

// The cluster count (*ccp, the new-id scan total) comes from the device; ids
// at or beyond min(cluster_count, MAX_BATCH_SIZE) are dropped.
__global__ void k_assign(const int32_t* u, const int32_t* v, int64_t p, int64_t len, const int32_t* cid,
                         const int64_t* ccp, uint64_t* keys, uint32_t* vals, unsigned long long* count) {
  pdl_wait();
  pdl_trigger();
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= len) return;
  const int64_t limit = min(*ccp, kMaxBatchEdges);
  const int64_t j = p + t;
  int32_t c = cid[u[j]];
  if (c == -1) c = cid[v[j]];
  if (c < 0 || (int64_t)c >= limit) return;
  const unsigned long long k = atomicAdd(count, 1ull);
  keys[k] = ((uint64_t)c << kRowBits) | (uint64_t)(kRowMask - (uint32_t)t);
  vals[k] = (uint32_t)t;
}

// ---- repair -------------------------------------------------------------------------------

struct RepairArgs {
  GraphView g;
  const int32_t* u;
  const int32_t* v;
  const uint8_t* ins;
  int64_t p;
  const uint32_t* order;
  int64_t cnt;
  int64_t ns;
  const int32_t* v2i;
  uint8_t* mis;
};

__device__ __forceinline__ bool is_seed_row(const RepairArgs& a, int32_t x) {
  const int32_t i = a.v2i[x];
  return i >= 0 && (int64_t)i < a.ns;
}

// any z in row-of(x) with mis[z] and z != except, one thread.
__device__ bool thread_any_member(const RepairArgs& a, int32_t x, int32_t except) {
  const GraphView& g = a.g;
  const uint8_t* mis = a.mis;
  auto hit = [&](int32_t z) { return z != except && mis[z] != 0; };
  if (!is_seed_row(a, x)) return thread_row_until(g, x, hit);
  if (hit(x)) return true;
  if (thread_row_until(g, x, hit)) return true;
  return thread_row_until(g, x, [&](int32_t h) { return thread_row_until(g, h, hit); });
}

// Q(w) of the insertion rule (src/misfit/misfit.cu:300-313).
__device__ bool eligible(const RepairArgs& a, int32_t w) {
  if (a.mis[w]) return false;
  if (a.v2i[w] < 0) return false;
  return !thread_any_member(a, w, -1);
}

// Single CTA walks the repair order; per chunk of 1024 edges it finds the next
// edge whose endpoint states call for work, evaluates it with the whole block,
// and repeats.  Exact sequential semantics of the canonical schedule.
// Shared flags are read into registers between two barriers so that every
// thread takes the same branch; warp loops exit on warp-uniform votes.
__global__ void __launch_bounds__(1024) k_repair_sequential(RepairArgs a) {
  __shared__ int s_first;
  __shared__ int s_act;        // 1 insert, 2 delete
  __shared__ int32_t s_x, s_keep;
  __shared__ unsigned long long s_best;
  __shared__ int s_flag;
  const GraphView& g = a.g;
  uint8_t* mis = a.mis;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  for (int64_t base = 0; base < a.cnt; base += blockDim.x) {
    const int64_t idx = base + tid;
    int32_t eu = 0, ev = 0;
    bool eins = false;
    const bool valid = idx < a.cnt;
    if (valid) {
      const int64_t j = a.p + a.order[idx];
      eu = a.u[j];
      ev = a.v[j];
      eins = a.ins[j] != 0;
    }
    int start = 0;
    while (true) {
      if (tid == 0) s_first = 1 << 30;
      __syncthreads();
      if (valid && tid >= start) {
        const bool mu = mis[eu] != 0, mv = mis[ev] != 0;
        if (eins ? (mu && mv) : (mu != mv)) atomicMin(&s_first, tid);
      }
      __syncthreads();
      const int first = s_first;
      if (first >= (int)blockDim.x) break;
      if (tid == first) {
        const bool mu = mis[eu] != 0;
        if (eins) {
          const int32_t r = eu > ev ? eu : ev;
          mis[r] = 0;
          s_act = 1;
          s_x = r;
        } else {
          s_act = 2;
          s_x = mu ? ev : eu;     // the endpoint that may join
          s_keep = mu ? eu : ev;  // the endpoint in the set
        }
        s_best = ~0ull;
        s_flag = 0;
      }
      __syncthreads();
      const int act = s_act;
      const int32_t x = s_x, keep = s_keep;
      if (act == 1 && a.v2i[x] >= 0) {
        // Insertion rule: first eligible w of row-of(r) in order.  Position
        // keys: 0 = r itself, 1 + k = row(r)[k], hop-2 = 2^62 + (k << 32) + j.
        const int32_t r = x;
        const bool seed = is_seed_row(a, r);
        if (tid == 0 && seed && eligible(a, r)) atomicMin(&s_best, 0ull);
        const int64_t nb = g.nindex[r + 1] - g.nindex[r];
        const int64_t nr = nb + (g.aoff[r + 1] - g.aoff[r]);
        for (int64_t k = tid; k < nr; k += blockDim.x) {
          const int32_t w = row_elem(g, r, k, nb);
          if (w >= 0 && eligible(a, w)) atomicMin(&s_best, 1ull + (unsigned long long)k);
        }
        __syncthreads();
        bool done = s_best != ~0ull;
        __syncthreads();
        if (!done && seed) {
          for (int64_t k0 = 0; k0 < nr; k0 += nw) {
            const int64_t k = k0 + wid;
            const int32_t h = k < nr ? row_elem(g, r, k, nb) : -1;
            if (h >= 0) {
              const int64_t hb = g.nindex[h + 1] - g.nindex[h];
              const int64_t hn = hb + (g.aoff[h + 1] - g.aoff[h]);
              for (int64_t j0 = 0; j0 < hn; j0 += 32) {
                const int64_t jj = j0 + lane;
                bool ok = false;
                if (jj < hn) {
                  const int32_t w = row_elem(g, h, jj, hb);
                  ok = w >= 0 && eligible(a, w);
                }
                const unsigned msk = __ballot_sync(0xffffffffu, ok);
                if (msk) {
                  if (lane == 0)
                    atomicMin(&s_best, (1ull << 62) + ((unsigned long long)k << 32) +
                                           (unsigned long long)(j0 + __ffs(msk) - 1));
                  break;
                }
              }
            }
            __syncthreads();
            done = s_best != ~0ull;
            __syncthreads();
            if (done) break;
          }
        }
        if (tid == 0 && s_best != ~0ull) {
          const unsigned long long key = s_best;
          int32_t w;
          if (key == 0) {
            w = r;
          } else if (key < (1ull << 62)) {
            w = row_elem(g, r, (int64_t)(key - 1), nb);
          } else {
            const int64_t k = (int64_t)((key - (1ull << 62)) >> 32);
            const int64_t jj = (int64_t)(key & 0xffffffffull);
            const int32_t h = row_elem(g, r, k, nb);
            w = row_elem(g, h, jj, g.nindex[h + 1] - g.nindex[h]);
          }
          mis[w] = 1;
        }
      } else if (act == 2) {
        // Deletion rule: y joins unless row-of(y) holds a member other than keep.
        const int32_t y = x;
        if (a.v2i[y] < 0) {
          if (tid == 0) mis[y] = 1;
        } else {
          const bool seed = is_seed_row(a, y);
          auto hit = [&](int32_t z) { return z != keep && mis[z] != 0; };
          bool found = tid == 0 && seed && hit(y);
          const int64_t nb = g.nindex[y + 1] - g.nindex[y];
          const int64_t ny = nb + (g.aoff[y + 1] - g.aoff[y]);
          for (int64_t k = tid; k < ny && !found; k += blockDim.x) {
            const int32_t z = row_elem(g, y, k, nb);
            if (z >= 0 && hit(z)) found = true;
          }
          if (found) s_flag = 1;
          __syncthreads();
          const bool done = s_flag != 0;
          __syncthreads();
          if (!done && seed) {
            for (int64_t k = wid; k < ny; k += nw) {
              const int32_t h = row_elem(g, y, k, nb);
              bool f = false;
              if (h >= 0) {
                const int64_t hb = g.nindex[h + 1] - g.nindex[h];
                const int64_t hn = hb + (g.aoff[h + 1] - g.aoff[h]);
                for (int64_t j0 = 0; j0 < hn; j0 += 32) {
                  const int64_t jj = j0 + lane;
                  bool ok = false;
                  if (jj < hn) {
                    const int32_t z = row_elem(g, h, jj, hb);
                    ok = z >= 0 && hit(z);
                  }
                  if (__any_sync(0xffffffffu, ok)) { f = true; break; }
                  if (__any_sync(0xffffffffu, *(volatile int*)&s_flag != 0)) break;
                }
              }
              if (f && lane == 0) s_flag = 1;
              if (__any_sync(0xffffffffu, f || *(volatile int*)&s_flag != 0)) break;
            }
          }
          __syncthreads();
          if (tid == 0 && !s_flag) mis[y] = 1;
        }
      }
      __syncthreads();
      start = first + 1;
    }
  }
}

// ---- speculative repair ---------------------------------------------------------------------
// The repair order is a total order of edges; the result must equal walking
// it one edge at a time.  Each round evaluates every pending edge (one warp
// per edge) against a view: the committed membership plus the writes that the
// previous round's evaluations made at earlier positions.  The first position
// whose writes changed since the previous round is final together with
// everything before it (each of those saw exactly the writes of its
// predecessors), so that prefix is committed and the next round starts after
// it.  Independent edges settle in the same round; a chain of k dependent
// edges needs k rounds.  After kMaxRounds rounds the remainder is walked by
// the sequential kernel.

constexpr int kMaxRounds = 48;
constexpr int kRoundsPerSync = 2;   // small rounds queued per host read-back

struct View {
  const uint8_t* m;     // bit 0: committed membership; bit 1: pending writes exist
  const uint64_t* keys; // pending writes sorted by (vertex << 32 | position)
  const uint32_t* vals;
  int64_t nkeys;
};

__device__ __forceinline__ int view_get(const View& V, int32_t x, uint32_t t) {
  const uint8_t b = V.m[x];
  if (!(b & 2)) return b & 1;
  const uint64_t q = ((uint64_t)(uint32_t)x << 32) | t;
  int64_t lo = 0, hi = V.nkeys;  // first key >= q
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (V.keys[mid] < q) lo = mid + 1; else hi = mid;
  }
  if (lo > 0 && (uint32_t)(V.keys[lo - 1] >> 32) == (uint32_t)x) return (int)V.vals[lo - 1];
  return b & 1;
}

struct SpecArgs {
  GraphView g;
  const int32_t* u;
  const int32_t* v;
  const uint8_t* ins;
  int64_t p;
  const uint32_t* order;
  int64_t p0, cnt, ns;
  const int32_t* v2i;
  View view;
  int32_t* out0;   // vertex written first (removal for an insert, join for a delete) or -1
  int32_t* out1;   // vertex that joins after an insert's removal, or -1
  // deferral of long hop-2 searches to the grid-wide kernel
  int64_t big_threshold;
  unsigned long long* big_count;
  int64_t* big_pos;       // repair position of each deferred edge
  int32_t* big_r;         // its removed vertex r
  int64_t* big_off;       // offset of its prefix array in `pre`
  int64_t* big_nr;        // entries of row(r)
  int64_t* pre;           // prefix sums of len(h) over row(r), nr + 1 entries per deferred edge
  unsigned long long* pre_used;
  int64_t pre_cap;
  // rounds queued without a host read-back: [0] first pending position,
  // [1] entries of the view, [2] 1 once no position changed, [3] rounds run
  // (k_spec_round keeps them); p0 and view.nkeys above are then ignored
  int64_t* dyn = nullptr;
};

// A queued round's start and view from the device; false once the repair
// is done (the round then does nothing).
__device__ __forceinline__ bool spec_dyn_load(SpecArgs& a) {
  if (a.dyn == nullptr) return true;
  if (a.dyn[2] != 0) return false;
  a.p0 = a.dyn[0];
  a.view.nkeys = a.dyn[1];
  return true;
}

constexpr int32_t kDeferred = -2;

// Membership seen by the edge at position t (its own removal of `self0` applied).
struct Member {
  const View* V;
  uint32_t t;
  int32_t self0;
  __device__ __forceinline__ int operator()(int32_t x) const { return x == self0 ? 0 : view_get(*V, x, t); }
};

__device__ __forceinline__ bool spec_seed(const SpecArgs& a, int32_t x) {
  const int32_t i = a.v2i[x];
  return i >= 0 && (int64_t)i < a.ns;
}

// Thread: does row(x) hold a member other than `except`?  1 yes, 0 no, -1
// when `left` ran out first (it is decremented by the live elements read).
// Eight positions at a time: their ids, then their membership bytes, all
// loads of a group in flight before any is tested; the rare pending-write
// lookups (bit 1 of the byte) go through the view.  A group may read past
// the budget or past the first member; only the answer is defined.
__device__ __forceinline__ int t_row_any(const GraphView& g, int32_t x, const Member& mem, int32_t except, int& left) {
  const uint8_t* m = mem.V->m;
  auto group = [&](const int32_t (&y)[8]) {
    uint8_t mb[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) mb[q] = y[q] >= 0 ? m[y[q]] : 0;
    bool hit = false;
    int cnt = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      if (y[q] < 0) continue;
      ++cnt;
      if (y[q] == except || y[q] == mem.self0) continue;
      hit |= (mb[q] & 2) ? mem(y[q]) != 0 : (mb[q] & 1) != 0;
    }
    left -= cnt;
    return hit;
  };
  const int64_t b = g.nindex[x], e = g.nindex[x + 1];
  const bool filt = g.dead[x] != 0;
  for (int64_t k0 = b; k0 < e; k0 += 8) {
    if (left <= 0) return -1;
    int32_t y[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int64_t k = k0 + q;
      y[q] = -1;
      if (k < e && (!filt || live_at(g.live, k))) y[q] = __ldg(g.nlist + k);
    }
    if (group(y)) return 1;
  }
  const int64_t ab = g.aoff[x], ae = g.aoff[x + 1];
  for (int64_t k0 = ab; k0 < ae; k0 += 8) {
    if (left <= 0) return -1;
    int32_t y[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) y[q] = k0 + q < ae ? g.aadj[k0 + q] : -1;
    if (group(y)) return 1;
  }
  return 0;
}

// Warp: does row(x) hold a member other than `except`?  Steps of one, two,
// then four 32-position windows, the ids and then the membership bytes of a
// step loaded before any is tested.
__device__ bool w_row_any(const GraphView& g, int32_t x, const Member& mem, int32_t except) {
  const int lane = threadIdx.x & 31;
  const uint8_t* m = mem.V->m;
  const int64_t b = g.nindex[x], nb = g.nindex[x + 1] - b;
  const int64_t ab = g.aoff[x];
  const int64_t np = nb + (g.aoff[x + 1] - ab);
  const bool filt = g.dead[x] != 0;
  int nwin = 1;
  for (int64_t base = 0; base < np; base += 32 * nwin, nwin = nwin < 4 ? 2 * nwin : 4) {
    int32_t y[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t k = base + 32 * q + lane;
      y[q] = -1;
      if (q < nwin && k < np) {
        if (k < nb) {
          if (!filt || live_at(g.live, b + k)) y[q] = __ldg(g.nlist + b + k);
        } else {
          y[q] = g.aadj[ab + (k - nb)];
        }
      }
    }
    uint8_t mb[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) mb[q] = y[q] >= 0 ? m[y[q]] : 0;
    bool hit = false;
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (y[q] >= 0 && y[q] != except && y[q] != mem.self0) hit |= (mb[q] & 2) ? mem(y[q]) != 0 : (mb[q] & 1) != 0;
    if (__any_sync(0xffffffffu, hit)) return true;
  }
  return false;
}

// Warp: does row-of(x) hold a member other than `except`?
__device__ bool w_any(const SpecArgs& a, const Member& mem, int32_t x, int32_t except) {
  const GraphView& g = a.g;
  const int lane = threadIdx.x & 31;
  const bool seed = spec_seed(a, x);
  if (seed && x != except && mem(x) != 0) return true;
  if (w_row_any(g, x, mem, except)) return true;
  if (!seed) return false;
  const int64_t nb = g.nindex[x + 1] - g.nindex[x];
  const int64_t nr = nb + (g.aoff[x + 1] - g.aoff[x]);
  for (int64_t k0 = 0; k0 < nr; k0 += 32) {
    const int64_t k = k0 + lane;
    const int32_t h = k < nr ? row_elem(g, x, k, nb) : -1;
    bool found = false, longrow = false;
    if (h >= 0) {
      if (row_len(g, h) <= 64) {
        int unbounded = 1 << 30;
        found = t_row_any(g, h, mem, except, unbounded) > 0;
      } else {
        longrow = true;
      }
    }
    if (__any_sync(0xffffffffu, found)) return true;
    unsigned lm = __ballot_sync(0xffffffffu, longrow);
    while (lm) {
      const int src = __ffs(lm) - 1;
      lm &= lm - 1;
      const int32_t hh = __shfl_sync(0xffffffffu, h, src);
      if (w_row_any(g, hh, mem, except)) return true;
    }
  }
  return false;
}

// Thread: 1 if row-of(x) holds a member (other than `except`), 0 if it holds
// none, -1 if about `budget` elements were read without an answer (up to
// seven more: the row scans read eight at a time).
__device__ int t_any_bounded(const SpecArgs& a, const Member& mem, int32_t x, int32_t except, int budget) {
  int left = budget;
  if (!spec_seed(a, x)) return t_row_any(a.g, x, mem, except, left);
  if (x != except && mem(x)) return 1;
  const int r = t_row_any(a.g, x, mem, except, left);
  if (r != 0) return r;
  int res = 0;
  thread_row_until(a.g, x, [&](int32_t h) {
    res = t_row_any(a.g, h, mem, except, left);
    return res != 0;
  });
  return res;
}

// Warp: first eligible element of row(x) in row order, or -1.  Every lane
// checks its element with a short serial scan; the elements left undecided
// (a long row without an early member) are settled by the whole warp, in
// position order, so a hub element does not keep one lane scanning alone.
__device__ int32_t w_first_eligible_row(const SpecArgs& a, const Member& mem, int32_t x) {
  const GraphView& g = a.g;
  const int lane = threadIdx.x & 31;
  const int64_t nb = g.nindex[x + 1] - g.nindex[x];
  const int64_t np = nb + (g.aoff[x + 1] - g.aoff[x]);
  for (int64_t k0 = 0; k0 < np; k0 += 32) {
    const int64_t k = k0 + lane;
    const int32_t w = k < np ? row_elem(g, x, k, nb) : -1;
    int state = 0;  // 0 not eligible, 1 eligible, 2 undecided
    if (w >= 0 && !mem(w) && a.v2i[w] >= 0) {
      const int r = t_any_bounded(a, mem, w, -1, 64);
      state = r == 0 ? 1 : (r < 0 ? 2 : 0);
    }
    unsigned m = __ballot_sync(0xffffffffu, state != 0);
    while (m) {
      const int src = __ffs(m) - 1;
      m &= m - 1;
      const int32_t ww = __shfl_sync(0xffffffffu, w, src);
      const int st = __shfl_sync(0xffffffffu, state, src);
      if (st == 1 || !w_any(a, mem, ww, -1)) return ww;
    }
  }
  return -1;
}

// Warp: first eligible w of row-of(r) in order (src/misfit/misfit.cu:300-314), or -1.
__device__ int32_t w_first_eligible(const SpecArgs& a, const Member& mem, int32_t r) {
  const GraphView& g = a.g;
  const int lane = threadIdx.x & 31;
  const bool seed = spec_seed(a, r);
  if (seed && !mem(r) && a.v2i[r] >= 0 && !w_any(a, mem, r, -1)) return r;
  int32_t w = w_first_eligible_row(a, mem, r);
  if (w >= 0) return w;
  if (!seed) return -1;
  const int64_t nb = g.nindex[r + 1] - g.nindex[r];
  const int64_t nr = nb + (g.aoff[r + 1] - g.aoff[r]);
  // Volume of the hop-2 part; long ones go to the grid-wide search.  Four
  // windows of row(r) per step, their ids and then their row lengths loaded
  // before any is summed.
  int64_t vol = 0;
  for (int64_t k0 = lane; k0 < nr; k0 += 128) {
    int32_t hq[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) hq[q] = k0 + 32 * q < nr ? row_elem(g, r, k0 + 32 * q, nb) : -1;
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (hq[q] >= 0) vol += row_positions(g, hq[q]);   // positions, tombstoned ones included
  }
  for (int o = 16; o > 0; o >>= 1) vol += __shfl_xor_sync(0xffffffffu, vol, o);
  if (vol > a.big_threshold) {
    unsigned long long off = 0;
    if (lane == 0) off = atomicAdd(a.pre_used, (unsigned long long)(nr + 1));
    off = __shfl_sync(0xffffffffu, off, 0);
    if ((int64_t)(off + nr + 1) <= a.pre_cap) {
      int64_t carry = 0;
      for (int64_t k0 = 0; k0 < nr; k0 += 128) {
        // four windows: every row length loaded before any prefix is stored
        int64_t len[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int64_t k = k0 + 32 * q + lane;
          const int32_t h = k < nr ? row_elem(g, r, k, nb) : -1;
          len[q] = h >= 0 ? row_positions(g, h) : 0;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int64_t k = k0 + 32 * q + lane;
          int64_t inc = len[q];
          for (int o = 1; o < 32; o <<= 1) {
            const int64_t t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
          }
          if (k < nr) a.pre[off + k] = carry + inc - len[q];
          carry += __shfl_sync(0xffffffffu, inc, 31);
        }
      }
      if (lane == 0) {
        a.pre[off + nr] = carry;
        const unsigned long long b = atomicAdd(a.big_count, 1ull);
        a.big_pos[b] = (int64_t)mem.t;
        a.big_r[b] = r;
        a.big_off[b] = (int64_t)off;
        a.big_nr[b] = nr;
      }
      return kDeferred;
    }
  }
  for (int64_t k = 0; k < nr; ++k) {
    const int32_t h = row_elem(g, r, k, nb);
    if (h < 0) continue;
    w = w_first_eligible_row(a, mem, h);
    if (w >= 0) return w;
  }
  return -1;
}

constexpr int kBigChunk = 256;  // positions per chunk = threads per block of k_big_scan

// Chunk prefix over the deferred edges (one block, any size up to 1024
// threads): chunk_pre[i] = first chunk of deferred edge i, chunk_pre[nbig] =
// total; best[i] = none; the chunk queue restarts.
__device__ void big_prep_block(const SpecArgs& a, int64_t* chunk_pre, unsigned long long* best,
                               unsigned long long* queue) {
  const int64_t nbig = (int64_t)*(volatile unsigned long long*)a.big_count;
  __shared__ int64_t s_carry;
  if (threadIdx.x == 0) { s_carry = 0; queue[0] = 0; queue[1] = 0; }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __shared__ int64_t s_w[32];
  for (int64_t base = 0; base < nbig; base += blockDim.x) {
    const int64_t i = base + threadIdx.x;
    int64_t cnt = 0;
    if (i < nbig) {
      const int64_t vol = a.pre[a.big_off[i] + a.big_nr[i]];
      cnt = (vol + kBigChunk - 1) / kBigChunk;
      best[i] = ~0ull;
    }
    int64_t inc = cnt;
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) s_w[wid] = inc;
    __syncthreads();
    if (threadIdx.x == 0) {
      int64_t acc = 0;
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { const int64_t t = s_w[k]; s_w[k] = acc; acc += t; }
    }
    __syncthreads();
    if (i < nbig) chunk_pre[i] = s_carry + s_w[wid] + inc - cnt;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) s_carry += s_w[wid] + inc;
    __syncthreads();
  }
  if (threadIdx.x == 0) chunk_pre[nbig] = s_carry;
}

// One warp per pending edge.  The last block to finish also prepares the
// grid-wide hop-2 search (big_prep_block): every block fences its deferral
// records before it counts itself done.
__global__ void k_spec_eval(SpecArgs a, int64_t* chunk_pre, unsigned long long* best, unsigned long long* queue,
                            unsigned int* done) {
  pdl_wait();
  pdl_trigger();
  if (!spec_dyn_load(a)) return;
  const int64_t wi = warp_id();
  if (wi < a.cnt - a.p0) {
    const int lane = threadIdx.x & 31;
    const int64_t pos = a.p0 + wi;
    const int64_t j = a.p + a.order[pos];
    const int32_t x = a.u[j], y = a.v[j];
    const bool ins = a.ins[j] != 0;
    Member mem{&a.view, (uint32_t)pos, -1};
    const int mx = mem(x), my = mem(y);
    int32_t o0 = -1, o1 = -1;
    if (ins) {
      if (mx && my) {
        const int32_t r = x > y ? x : y;
        o0 = r;
        mem.self0 = r;
        if (a.v2i[r] >= 0) o1 = w_first_eligible(a, mem, r);
      }
    } else if (mx != my) {
      const int32_t yy = mx ? y : x, keep = mx ? x : y;
      if (a.v2i[yy] < 0 || !w_any(a, mem, yy, keep)) o0 = yy;
    }
    if (lane == 0) {
      a.out0[pos] = o0;
      a.out1[pos] = o1;
    }
  }
  __shared__ bool s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (s_last) {
    __threadfence();
    big_prep_block(a, chunk_pre, best, queue);
  }
}

// Grid-wide first-eligible search over the flattened hop-2 sequences of the
// deferred edges; chunks of kBigChunk positions (one per thread) are handed
// out in increasing position order.  The row index of each position comes
// from a binary search in a shared copy of the prefix entries that cover the
// chunk (one global search per chunk).  Each thread checks its element with a
// bounded serial scan (64 reads); elements that scan leaves undecided (a long
// row-of without an early member) are settled afterwards by whole warps, so
// that no single thread walks a hub row alone.  The chunk's answer is the
// smallest eligible position.
__global__ void __launch_bounds__(kBigChunk, 4) k_big_scan(SpecArgs a, const int64_t* chunk_pre,
                                                        unsigned long long* best, unsigned long long* queue) {
  pdl_wait();
  pdl_trigger();
  if (!spec_dyn_load(a)) return;
  const GraphView& g = a.g;
  const int64_t nbig = (int64_t)*a.big_count;
  const int64_t total = chunk_pre[nbig];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __shared__ unsigned long long s_chunk;
  __shared__ unsigned long long s_best;
  __shared__ int s_live, s_nu;
  __shared__ int64_t s_k0;
  __shared__ int64_t s_pre[kBigChunk + 1];
  __shared__ int64_t s_uq[kBigChunk];
  __shared__ int32_t s_uz[kBigChunk];
  while (true) {
    if (threadIdx.x == 0) s_chunk = atomicAdd(queue, 1ull);
    __syncthreads();
    const int64_t chunk = (int64_t)s_chunk;
    if (chunk >= total) break;
    int64_t lo = 0, hi = nbig;  // last i with chunk_pre[i] <= chunk
    while (hi - lo > 1) {
      const int64_t mid = (lo + hi) >> 1;
      if (chunk_pre[mid] <= chunk) lo = mid; else hi = mid;
    }
    const int64_t i = lo;
    const int64_t p0 = (chunk - chunk_pre[i]) * kBigChunk;
    const int64_t* pre = a.pre + a.big_off[i];
    const int64_t nr = a.big_nr[i];
    const int64_t vol = pre[nr];
    const int32_t r = a.big_r[i];
    if (wid == 0) {
      // warp 0: skip test, then the last k with pre[k] <= p0 by a 32-way
      // search (each step samples 32 prefix entries and keeps the interval
      // around the boundary, so a hub row of 10^6 entries takes 4 steps)
      int live = 0;
      if (lane == 0) {
        live = (unsigned long long)p0 < best[i] ? 1 : 0;  // an earlier chunk may have answered
        // chunks are handed out in increasing position order, so once edge i
        // has an answer before this chunk, no later chunk of edge i can beat
        // it: move the queue head to the next edge's first chunk
        if (!live) atomicMax(queue, (unsigned long long)chunk_pre[i + 1]);
      }
      live = __shfl_sync(0xffffffffu, live, 0);
      int64_t lo = 0, hi = nr;  // pre[lo] <= p0 < pre[hi]
      while (live && hi - lo > 1) {
        const int64_t step = (hi - lo + 31) / 32;
        const int64_t idx = lo + (int64_t)lane * step;
        const unsigned m = __ballot_sync(0xffffffffu, idx < hi && pre[idx] <= p0);
        const int top = 31 - __clz(m);
        const int64_t nlo = lo + (int64_t)top * step;
        hi = min(nlo + step, hi);
        lo = nlo;
      }
      if (lane == 0) {
        s_best = ~0ull;
        s_nu = 0;
        s_live = live;
        s_k0 = lo;
        if (live) atomicAdd(queue + 1, 1ull);  // chunks scanned (the rest were skipped)
      }
    }
    __syncthreads();
    if (s_live) {
      // prefix entries k0 .. k0 + kBigChunk (clamped to nr); the positions of
      // the chunk lie in rows k0 .. k0 + kBigChunk - 1 unless rows are empty
      const int64_t k0 = s_k0;
      const int64_t kn = min((int64_t)kBigChunk, nr - k0);
      for (int64_t t = threadIdx.x; t <= kn; t += blockDim.x) s_pre[t] = pre[k0 + t];
      __syncthreads();
      const int64_t q = p0 + threadIdx.x;
      if (q < vol) {
        int64_t k;
        if (q < s_pre[kn]) {
          int lo2 = 0, hi2 = (int)kn;  // last t with s_pre[t] <= q
          while (hi2 - lo2 > 1) {
            const int mid = (lo2 + hi2) >> 1;
            if (s_pre[mid] <= q) lo2 = mid; else hi2 = mid;
          }
          k = k0 + lo2;
        } else {
          int64_t klo = k0 + kn, khi = nr;  // beyond the shared window (empty rows): global search
          while (khi - klo > 1) {
            const int64_t mid = (klo + khi) >> 1;
            if (pre[mid] <= q) klo = mid; else khi = mid;
          }
          k = klo;
        }
        Member mem{&a.view, (uint32_t)a.big_pos[i], r};
        const int32_t h = row_elem(g, r, k, g.nindex[r + 1] - g.nindex[r]);
        if (h >= 0) {
          const int32_t z = row_elem(g, h, q - pre[k], g.nindex[h + 1] - g.nindex[h]);
          if (z >= 0 && !mem(z) && a.v2i[z] >= 0) {
            const int res = t_any_bounded(a, mem, z, -1, 64);
            if (res == 0) {
              atomicMin(&s_best, (unsigned long long)q);
            } else if (res < 0) {
              const int u = atomicAdd(&s_nu, 1);  // at most one entry per thread
              s_uq[u] = q;
              s_uz[u] = z;
            }
          }
        }
      }
      __syncthreads();
      const int nu = s_nu;
      Member mem{&a.view, (uint32_t)a.big_pos[i], r};
      for (int u = wid; u < nu; u += nw) {
        const unsigned long long qq = (unsigned long long)s_uq[u];
        unsigned long long cur = 0;
        if (lane == 0) cur = atomicAdd(&s_best, 0ull);
        cur = __shfl_sync(0xffffffffu, cur, 0);
        if (qq >= cur) continue;  // a smaller eligible position is known
        if (!w_any(a, mem, s_uz[u], -1) && lane == 0) atomicMin(&s_best, qq);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_best != ~0ull) {
      atomicMin(best + i, s_best);
      atomicMax(queue, (unsigned long long)chunk_pre[i + 1]);   // edge i's later chunks cannot win
    }
    __syncthreads();
  }
}

// The answer of deferred edge i: the vertex at its smallest eligible
// position, or -1.
__device__ void big_finalize_one(const SpecArgs& a, const unsigned long long* best, int64_t i) {
  const GraphView& g = a.g;
  int32_t w = -1;
  if (best[i] != ~0ull) {
    const int64_t q = (int64_t)best[i];
    const int64_t* pre = a.pre + a.big_off[i];
    const int64_t nr = a.big_nr[i];
    const int32_t r = a.big_r[i];
    int64_t klo = 0, khi = nr;
    while (khi - klo > 1) {
      const int64_t mid = (klo + khi) >> 1;
      if (pre[mid] <= q) klo = mid; else khi = mid;
    }
    const int32_t h = row_elem(g, r, klo, g.nindex[r + 1] - g.nindex[r]);
    w = row_elem(g, h, q - pre[klo], g.nindex[h + 1] - g.nindex[h]);
  }
  a.out1[a.big_pos[i]] = w;
}

__global__ void k_big_finalize(SpecArgs a, const unsigned long long* best) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < (int64_t)*a.big_count) big_finalize_one(a, best, i);
}

__global__ void k_spec_first_change(const int32_t* n0, const int32_t* n1, const int32_t* r0, const int32_t* r1,
                                    int64_t p0, int64_t cnt, unsigned long long* out) {
  const int64_t pos = p0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pos < cnt && (n0[pos] != r0[pos] || n1[pos] != r1[pos])) atomicMin(out, (unsigned long long)pos);
}

__global__ void k_spec_count(const int32_t* n0, const int32_t* n1, int64_t p0, int64_t cnt, uint8_t* c) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p0 + i < cnt) c[i] = (uint8_t)((n0[p0 + i] >= 0) + (n1[p0 + i] >= 0));
}

__global__ void k_spec_fill(const int32_t* n0, const int32_t* n1, const int64_t* pos_out, int64_t p0, int64_t cnt,
                            const int32_t* u, const int32_t* v, const uint8_t* ins, int64_t p, const uint32_t* order,
                            uint64_t* keys, uint32_t* vals) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p0 + i >= cnt) return;
  const int64_t pos = p0 + i;
  int64_t k = pos_out[i];
  const int32_t a = n0[pos], b = n1[pos];
  if (a >= 0) {
    keys[k] = ((uint64_t)(uint32_t)a << 32) | (uint64_t)pos;
    vals[k] = ins[p + order[pos]] ? 0u : 1u;
    ++k;
  }
  if (b >= 0) {
    keys[k] = ((uint64_t)(uint32_t)b << 32) | (uint64_t)pos;
    vals[k] = 1u;
  }
}

__global__ void k_spec_clear_flags(const uint64_t* keys, int64_t nk, uint8_t* m) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nk) m[keys[k] >> 32] &= 1;
}

// Commit every write at a position <= f that is the last such write to its vertex.
__global__ void k_spec_commit(const uint64_t* keys, const uint32_t* vals, int64_t nk, uint64_t f, uint8_t* m) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nk) return;
  const uint64_t key = keys[k];
  if ((key & 0xffffffffull) > f) return;
  if (k + 1 < nk) {
    const uint64_t nx = keys[k + 1];
    if ((nx >> 32) == (key >> 32) && (nx & 0xffffffffull) <= f) return;
  }
  m[key >> 32] = (uint8_t)vals[k];
}

__global__ void k_spec_keep_flags(const uint64_t* keys, int64_t nk, uint64_t f, uint8_t* m, uint8_t* keep) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nk) return;
  const bool later = (keys[k] & 0xffffffffull) > f;
  keep[k] = later ? 1 : 0;
  if (later) m[keys[k] >> 32] |= 2;
}

__global__ void k_spec_compact(const uint64_t* keys, const uint32_t* vals, const uint8_t* keep, const int64_t* pos,
                               int64_t nk, uint64_t* okeys, uint32_t* ovals) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nk || !keep[k]) return;
  okeys[pos[k]] = keys[k];
  ovals[pos[k]] = vals[k];
}

// One CTA finishes a round whose pending positions fit kRoundCap (the common
// case: a sub-batch has tens of processed edges).  It does, in order, what
// k_spec_first_change, k_spec_count + scan + k_spec_fill, the sort,
// k_spec_clear_flags, k_spec_commit, k_spec_keep_flags and k_spec_compact
// do for larger rounds, with the writes in shared memory.  out[0] = first
// changed position (cnt when none), out[1] = entries of the new view.
constexpr int kRoundThreads = 1024;
constexpr int kRoundCap = kRoundThreads;          // pending positions
constexpr int kRoundWrites = 2 * kRoundCap;       // at most two writes per position

// Exclusive block scan of one int per thread (blockDim.x == kRoundThreads).
__device__ __forceinline__ int round_scan(int x, int* s_warp, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int inc = x;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) s_warp[wid] = inc;
  __syncthreads();
  if (threadIdx.x < 32) {
    const int w = s_warp[threadIdx.x];
    int wi = w;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, wi, o);
      if (threadIdx.x >= o) wi += y;
    }
    s_warp[threadIdx.x] = wi - w;
    if (threadIdx.x == 31) s_warp[32] = wi;
  }
  __syncthreads();
  const int r = s_warp[wid] + inc - x;
  *total = s_warp[32];
  __syncthreads();
  return r;
}

// Start of a queued repair: both result pairs' first buffers to "no
// write", the round words and the deferral counters to zero, in one launch.
__global__ void k_repair_init(int32_t* w0, int32_t* w1, int64_t cnt, int64_t* dyn, int64_t* counts) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cnt) {
    w0[i] = -1;
    w1[i] = -1;
  }
  if (i < 4) dyn[i] = 0;
  if (i < 6) counts[i] = 0;
}

__global__ void __launch_bounds__(kRoundThreads) k_spec_round(const int32_t* n0, const int32_t* n1, const int32_t* r0,
                                                              const int32_t* r1, int64_t p0, int64_t cnt,
                                                              const uint8_t* ins, int64_t p, const uint32_t* order,
                                                              uint64_t* view_keys, uint32_t* view_vals,
                                                              int64_t nview_old, uint8_t* m,
                                                              unsigned long long* out, SpecArgs sa,
                                                              const unsigned long long* best) {
  pdl_wait();
  pdl_trigger();
  if (!spec_dyn_load(sa)) return;
  if (sa.dyn != nullptr) {
    p0 = sa.p0;
    nview_old = sa.view.nkeys;
  }
  __shared__ uint64_t s_keys[kRoundWrites];
  __shared__ uint32_t s_vals[kRoundWrites];
  __shared__ int s_warp[33];
  __shared__ unsigned long long s_f;
  const int tid = threadIdx.x;
  // answers of the edges whose hop-2 search ran grid-wide (k_big_scan)
  const int64_t nbig = (int64_t)*sa.big_count;
  for (int64_t i = tid; i < nbig; i += kRoundThreads) big_finalize_one(sa, best, i);
  __syncthreads();
  const int64_t pending = cnt - p0;
  if (tid == 0) s_f = (unsigned long long)cnt;
  __syncthreads();
  // first changed position; this round's writes into shared memory
  int32_t a = -1, b = -1;
  const int64_t pos = p0 + tid;
  if (tid < pending) {
    a = n0[pos];
    b = n1[pos];
    if (a != r0[pos] || b != r1[pos]) atomicMin(&s_f, (unsigned long long)pos);
  }
  int nk = 0;
  const int off = round_scan((a >= 0) + (b >= 0), s_warp, &nk);
  if (tid < pending) {
    int k = off;
    if (a >= 0) {
      s_keys[k] = ((uint64_t)(uint32_t)a << 32) | (uint64_t)pos;
      s_vals[k] = ins[p + order[pos]] ? 0u : 1u;
      ++k;
    }
    if (b >= 0) {
      s_keys[k] = ((uint64_t)(uint32_t)b << 32) | (uint64_t)pos;
      s_vals[k] = 1u;
    }
  }
  // bitonic sort of the keys (with their values) over the next power of two
  int np2 = 1;
  while (np2 < nk) np2 <<= 1;
  for (int k = nk + tid; k < np2; k += kRoundThreads) {
    s_keys[k] = ~0ull;
    s_vals[k] = 0u;
  }
  __syncthreads();
  for (int size = 2; size <= np2; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = tid; t < (np2 >> 1); t += kRoundThreads) {
        const int lo = 2 * t - (t & (stride - 1));
        const int hi = lo + stride;
        const bool up = (lo & size) == 0;
        const uint64_t x = s_keys[lo], y = s_keys[hi];
        if ((x > y) == up) {
          s_keys[lo] = y;
          s_keys[hi] = x;
          const uint32_t vx = s_vals[lo];
          s_vals[lo] = s_vals[hi];
          s_vals[hi] = vx;
        }
      }
      __syncthreads();
    }
  }
  // the previous view's pending flags go
  for (int64_t k = tid; k < nview_old; k += kRoundThreads) m[view_keys[k] >> 32] &= 1;
  __syncthreads();
  const unsigned long long f = s_f;
  const uint64_t last = (uint64_t)min((int64_t)f, cnt - 1);
  // commit every write at a position <= last that is the last such write to its vertex
  for (int k = tid; k < nk; k += kRoundThreads) {
    const uint64_t key = s_keys[k];
    if ((key & 0xffffffffull) > last) continue;
    if (k + 1 < nk) {
      const uint64_t nx = s_keys[k + 1];
      if ((nx >> 32) == (key >> 32) && (nx & 0xffffffffull) <= last) continue;
    }
    m[key >> 32] = (uint8_t)s_vals[k];
  }
  __syncthreads();
  // writes after `last` become the next view (in key order) and flag their vertex
  const int k0 = 2 * tid, k1 = 2 * tid + 1;
  const bool keep0 = k0 < nk && (s_keys[k0] & 0xffffffffull) > last;
  const bool keep1 = k1 < nk && (s_keys[k1] & 0xffffffffull) > last;
  if (keep0) m[s_keys[k0] >> 32] |= 2;
  if (keep1) m[s_keys[k1] >> 32] |= 2;
  int nview = 0;
  int w = round_scan((int)keep0 + (int)keep1, s_warp, &nview);
  if (keep0) {
    view_keys[w] = s_keys[k0];
    view_vals[w] = s_vals[k0];
    ++w;
  }
  if (keep1) {
    view_keys[w] = s_keys[k1];
    view_vals[w] = s_vals[k1];
  }
  if (tid == 0) {
    out[0] = f;
    out[1] = (unsigned long long)nview;
    if (sa.dyn != nullptr) {
      // the next queued round: after the first changed position, with this
      // round's writes as its view; the per-round counters start over
      sa.dyn[0] = (int64_t)f + 1;
      sa.dyn[1] = nview;
      sa.dyn[2] = (int64_t)f >= cnt ? 1 : 0;
      sa.dyn[3] += 1;
      for (int k = 0; k < 6; ++k) sa.big_count[k] = 0;   // deferrals, prefix use, queue (2), spare, done
    }
  }
}

__global__ void k_clear(const int32_t* seeds, int64_t ns, const int32_t* cands, int64_t nct, int32_t* cid,
                        int32_t* v2i) {
  pdl_wait();
  pdl_trigger();
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ns + nct) return;
  const int32_t x = i < ns ? seeds[i] : cands[i - ns];
  cid[x] = -1;
  v2i[x] = -1;
}

template <typename T>
std::vector<T> fetch(const T* d, int64_t cnt, cudaStream_t s) {
  std::vector<T> h((size_t)std::max<int64_t>(cnt, 0));
  if (cnt > 0) MF_CUDA(cudaMemcpyAsync(h.data(), d, sizeof(T) * (size_t)cnt, cudaMemcpyDeviceToHost, s));
  MF_CUDA(cudaStreamSynchronize(s));
  return h;
}

// Grid of a load-balanced (grid-stride) kernel: as many 256-thread CTAs as
// can be resident at once, so that no CTA waits for a second wave.
template <class K>
unsigned lb_grid(mf_ctx* c, K kernel) {
  static std::mutex mu;
  static std::unordered_map<const void*, unsigned> cache;
  std::lock_guard<std::mutex> lock(mu);
  const void* key = reinterpret_cast<const void*>(kernel);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  int sms = 0, per = 0;
  MF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  MF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, kTB, 0));
  const unsigned g = (unsigned)(sms * std::max(per, 1));
  cache.emplace(key, g);
  return g;
}

// Row-position prefix of list[0..cnt) for lb_rows into c->lb_offs.
void row_offsets(mf_ctx* c, const int32_t* list, int64_t cnt, int kind, int64_t ns, uint32_t epoch) {
  cudaStream_t s = c->stream;
  c->lb_offs.reserve(cnt + 1);
  scan_exclusive_with(RowCounts{c->view(), list, kind, c->rowcid.p, ns, c->bval.p, epoch, c->v2i.p}, c->lb_offs.p, cnt,
                      c->ws, s);
}

// Row-position prefix of the rows i of list[0..cnt) with marks[i] >= 0.
void row_offsets_marked(mf_ctx* c, const int32_t* list, const int32_t* marks, int64_t cnt) {
  c->lb_offs.reserve(cnt + 1);
  scan_exclusive_with(RowCounts{c->view(), list, kCntMarked, marks, 0, c->bval.p, 0, c->v2i.p}, c->lb_offs.p, cnt,
                      c->ws, c->stream);
}

// row_offsets into caller-given buffers on a given stream (the fronts).
void row_offsets_into(mf_ctx* c, const int32_t* list, int64_t cnt, DBuf<int64_t>& offs, Scratch& ws,
                      cudaStream_t s) {
  offs.reserve(cnt + 1);
  scan_exclusive_with(RowCounts{c->view(), list, kCntAll, c->rowcid.p, 0, c->bval.p, 0, c->v2i.p}, offs.p, cnt, ws, s);
}

// Buffers of both fronts at their largest sizes for a batch of m updates, so
// that no front allocates while another stream may use its memory.
void front_reserve(mf_ctx* c, int64_t m) {
  const int64_t words = ((int64_t)c->n + 31) / 32;
  const int64_t bblocks = (words + kBitsWords - 1) / kBitsWords;
  const int64_t max_ns = 2 * std::min<int64_t>(m, kMaxBatchEdges);
  for (auto& f : c->front) {
    f.bits.reserve(std::max<int64_t>(2 * words, 1));
    f.bits_sums.reserve(bblocks + 1);
    f.uacc.reserve(std::max<int64_t>(max_ns, 1));
    f.hlist.reserve(std::max<int32_t>(c->n, 1));
    f.cands.reserve(kMaxRows);
    f.lb_offs.reserve(2 * max_ns + 2);
    f.cnt.reserve(2);
  }
}

// Front of a sub-batch with `ns` seeds: hop-1 and seed bitmaps, the hop-1
// list and the candidate list in ascending id (no row map yet), and the
// packed-size upper bound; cnt[0] = (hop-1 << 32 | candidates), cnt[1] =
// bound.  Everything on stream `st`; it reads only the graph, the seeds and
// the per-batch size caches.
void front_compute(mf_ctx* c, Front& f, const int32_t* seeds, int64_t ns, cudaStream_t st) {
  const GraphView g = c->view();
  const int32_t n = c->n;
  const int64_t words = ((int64_t)n + 31) / 32;
  const int64_t bblocks = (words + kBitsWords - 1) / kBitsWords;
  uint32_t* hbits = f.bits.p;
  uint32_t* sbits = f.bits.p + words;
  MF_CUDA(cudaMemsetAsync(hbits, 0, sizeof(uint32_t) * (size_t)(2 * words), st));
  MF_CUDA(cudaMemsetAsync(f.uacc.p, 0, sizeof(unsigned long long) * (size_t)std::max<int64_t>(ns, 1), st));
  MF_CUDA(cudaMemsetAsync(f.cnt.p + 1, 0, sizeof(int64_t), st));
  row_offsets_into(c, seeds, ns, f.lb_offs, f.ws, st);
  MF_K(launch_pdl(k_lb_hop1_bound, lb_grid(c, k_lb_hop1_bound), kTB, 0, st, g, c->deg.p, seeds, f.lb_offs.p, ns, hbits, f.uacc.p,
                                                                    c->work.p + 2 * kStHop1));
  if (ns > 0) MF_K(launch_pdl(k_seed_bits, grid_for(ns), kTB, 0, st, seeds, ns, sbits));
  const int64_t capc = std::max<int64_t>(0, kMaxRows - ns);
  MF_K(launch_pdl(k_bits_reduce, (unsigned)bblocks, kBitsThreads, 0, st, hbits, sbits, words, f.bits_sums.p));
  MF_K(launch_pdl(k_bits_scan_sums, 1, kBitsThreads, 0, st, f.bits_sums.p, bblocks, f.cnt.p));
  MF_K(launch_pdl(k_bits_compact, (unsigned)bblocks, kBitsThreads, 0, st, hbits, sbits, words, f.bits_sums.p, capc, ns,
                                                                  f.hlist.p, f.cands.p, nullptr));
  MF_K(launch_pdl(k_bound_finish, lb_grid(c, k_bound_finish), kTB, 0, st, 
      g, seeds, ns, f.cands.p, f.cnt.p, capc, f.uacc.p, c->n2cache.p, c->n2stamp.p, c->n2bound.p, c->n2bstamp.p,
      c->n2batch, reinterpret_cast<unsigned long long*>(f.cnt.p + 1)));
}

double host_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

bool debug_counters() {
  static const bool on = std::getenv("MISFIT_GB_DEBUG") != nullptr;
  return on;
}

// MISFIT_GB_P2_BULK=0: the row pass's chunk tasks read their row entries
// with plain loads instead of the bulk-copy staging (same results, same
// speed where measured; kept for comparisons).
bool p2_bulk_on() {
  static const bool on = [] {
    const char* e = std::getenv("MISFIT_GB_P2_BULK");
    return !(e != nullptr && std::strcmp(e, "0") == 0);
  }();
  return on;
}

// MISFIT_GB_DEBUG=2: also the elements of every k_lb_push_hop launch.
bool debug_launches() {
  static const bool on = [] {
    const char* e = std::getenv("MISFIT_GB_DEBUG");
    return e != nullptr && std::atoi(e) >= 2;
  }();
  return on;
}

// Counter value before a k_lb_push_hop launch (debug only).
unsigned long long debug_counter(mf_ctx* c, const unsigned long long* counter) {
  unsigned long long v = 0;
  MF_CUDA(cudaStreamSynchronize(c->stream));
  MF_CUDA(cudaMemcpy(&v, counter, sizeof(v), cudaMemcpyDeviceToHost));
  return v;
}

// Prints the elements the k_lb_push_hop launch just made pushed (debug only).
void debug_push_hop(mf_ctx* c, const unsigned long long* counter, unsigned long long before) {
  static long long launch = 0;
  std::fprintf(stderr, "[misfit_gb] k_lb_push_hop launch %lld elements %llu\n", launch++,
               debug_counter(c, counter) - before);
}

template <int SW>
void pull_pass(mf_ctx* c, const int32_t* grp, int k, int64_t hcap, int64_t tcap) {
  cudaStream_t s = c->stream;
  const GraphView g = c->view();
  const int32_t n = c->n;
  unsigned long long* cnt = c->p2_cnt.p;   // 32*kP2MaxWords counts, then next, nhuge, ntasks, bulk error
  unsigned long long* ctl = cnt + 32 * kP2MaxWords;
  const P2Work wk{ctl, c->p2_huge.p, ctl + 1, hcap, c->p2_tasks.p, ctl + 2, tcap};
  const int64_t fwords = ((int64_t)n + 31) / 32;
  MF_CUDA(cudaMemsetAsync(c->p2_mask.p, 0, sizeof(uint32_t) * (size_t)n * SW, s));
  MF_CUDA(cudaMemsetAsync(c->p2_filt.p, 0, sizeof(uint32_t) * (size_t)fwords, s));
  MF_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * (32 * kP2MaxWords + 3), s));
  MF_K(k_p2_mark<SW><<<dim3((unsigned)k, 16), kTB, 0, s>>>(g, c->seeds.p, grp, k, c->p2_mask.p, c->p2_filt.p));
  MF_K(k_p2_rows<SW><<<lb_grid(c, k_p2_rows<SW>), kTB, 0, s>>>(g, c->p2_mask.p, c->p2_filt.p, cnt, wk));
  MF_CUDA(cudaMemsetAsync(c->p2_racc.p, 0, sizeof(uint32_t) * (size_t)hcap * SW, s));
  {
    const size_t smem = (size_t)(kTB / 32) * (2 * kP2SubBuf * 4 + 2 * 8);
    // resident blocks of this kernel (pool workers may get here at once)
    static std::atomic<int> grid_huge{0};
    int grid = grid_huge.load(std::memory_order_relaxed);
    if (grid == 0) {
      int sms = 0, per = 0;
      MF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
      MF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_p2_huge<SW>, kTB, smem));
      grid = sms * std::max(per, 1);
      grid_huge.store(grid, std::memory_order_relaxed);
    }
    MF_K(k_p2_huge<SW><<<grid, kTB, smem, s>>>(g, c->p2_mask.p, c->p2_filt.p, wk, c->p2_racc.p, p2_bulk_on(),
                                               ctl + 3));
  }
  MF_K(k_p2_huge_count<SW><<<grid_for(hcap), kTB, 0, s>>>(c->p2_mask.p, c->p2_huge.p, ctl + 1, hcap, c->p2_racc.p,
                                                            cnt));
  MF_K(k_p2_store<<<1, 256, 0, s>>>(cnt, grp, k, c->rowlens.p));
}

// Exact 2-hop sizes, by one pass over every row per group of up to 256
// seeds, of the todo seeds whose neighbourhood volume pays for it
// (tune.pull_sizes 1; 2 takes all of them; symmetric graphs only).  Sizes
// go to c->rowlens; the seeds left for the push form are written back to
// todo, and their count is returned.
int64_t pull_exact(mf_ctx* c, int32_t* todo, int64_t ntodo) {
  if (c->tune.pull_sizes == 0 || !c->symmetric || ntodo == 0) return ntodo;
  cudaStream_t s = c->stream;
  const int32_t n = c->n;
  // mask words per vertex within 8 GB
  int max_words = kP2MaxWords;
  while (max_words > 0 && (int64_t)n * max_words * 4 > ((int64_t)8 << 30)) max_words >>= 1;
  if (max_words == 0) return ntodo;
  const GraphView g = c->view();
  c->p2_vol.reserve(ntodo);
  MF_CUDA(cudaMemsetAsync(c->p2_vol.p, 0, sizeof(int64_t) * (size_t)ntodo, s));
  MF_K(k_p2_volume<<<dim3((unsigned)ntodo, 4), kTB, 0, s>>>(g, c->deg.p, c->seeds.p, todo, ntodo, c->p2_vol.p));
  std::vector<int64_t> vol((size_t)ntodo);
  std::vector<int32_t> idx((size_t)ntodo);
  MF_CUDA(cudaMemcpyAsync(vol.data(), c->p2_vol.p, sizeof(int64_t) * (size_t)ntodo, cudaMemcpyDeviceToHost, s));
  MF_CUDA(cudaMemcpyAsync(idx.data(), todo, sizeof(int32_t) * (size_t)ntodo, cudaMemcpyDeviceToHost, s));
  MF_CUDA(cudaStreamSynchronize(s));
  std::vector<int64_t> order((size_t)ntodo);
  for (int64_t t = 0; t < ntodo; ++t) order[(size_t)t] = t;
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return vol[(size_t)a] > vol[(size_t)b]; });
  // Measured on R-MAT scale 26 (2.6e9 positions): a pass (about 13 ms) takes
  // as long as the push form takes for a neighbourhood volume of about half
  // the positions.
  const int64_t positions = c->nnz + c->a_total;
  const double pass_cost = (double)positions * kP2PassVolume + 65536.0;
  const int64_t gmax = 32 * (int64_t)max_words;
  std::vector<int32_t> pull, push;
  std::vector<int> group_sizes;
  size_t t = 0;
  while (t < order.size()) {
    const size_t end = std::min(order.size(), t + (size_t)gmax);
    double sum = 0;
    for (size_t u = t; u < end; ++u) sum += (double)vol[(size_t)order[u]];
    if (c->tune.pull_sizes == 1 && sum < pass_cost) break;
    for (size_t u = t; u < end; ++u) pull.push_back(idx[(size_t)order[u]]);
    group_sizes.push_back((int)(end - t));
    t = end;
  }
  if (pull.empty()) return ntodo;
  double pulled_vol = 0;
  for (size_t u = 0; u < t; ++u) pulled_vol += (double)vol[(size_t)order[u]];
  for (; t < order.size(); ++t) push.push_back(idx[(size_t)order[t]]);
  const bool dbg = debug_counters();
  const double t0 = dbg ? host_ms() : 0.0;
  // rows over kP2Huge positions, and their chunks
  const int64_t hcap = positions / (kP2Huge + 1) + 1;
  const int64_t tcap = hcap + positions / kP2Chunk + 1;
  c->p2_grp.reserve((int64_t)pull.size());
  const int first = group_sizes.front();
  c->p2_mask.reserve((int64_t)n * (first <= 32 ? 1 : first <= 64 ? 2 : first <= 128 ? 4 : 8));
  c->p2_cnt.reserve(32 * kP2MaxWords + 4);
  c->p2_filt.reserve(((int64_t)n + 31) / 32);
  c->p2_huge.reserve(hcap);
  c->p2_tasks.reserve(tcap);
  c->p2_racc.reserve(hcap * kP2MaxWords);
  MF_CUDA(cudaMemcpyAsync(c->p2_grp.p, pull.data(), sizeof(int32_t) * pull.size(), cudaMemcpyHostToDevice, s));
  MF_CUDA(cudaMemsetAsync(c->p2_cnt.p + 32 * kP2MaxWords + 3, 0, sizeof(unsigned long long), s));
  if (!push.empty())
    MF_CUDA(cudaMemcpyAsync(todo, push.data(), sizeof(int32_t) * push.size(), cudaMemcpyHostToDevice, s));
  size_t off = 0;
  for (const int k : group_sizes) {
    const int32_t* grp = c->p2_grp.p + off;
    if (k <= 32) pull_pass<1>(c, grp, k, hcap, tcap);
    else if (k <= 64) pull_pass<2>(c, grp, k, hcap, tcap);
    else if (k <= 128) pull_pass<4>(c, grp, k, hcap, tcap);
    else pull_pass<8>(c, grp, k, hcap, tcap);
    off += (size_t)k;
  }
  // the host vectors of the copies above stay alive until the stream reaches them
  unsigned long long bulk_err = 0;
  MF_CUDA(cudaMemcpyAsync(&bulk_err, c->p2_cnt.p + 32 * kP2MaxWords + 3, sizeof(bulk_err), cudaMemcpyDeviceToHost,
                          s));
  MF_CUDA(cudaStreamSynchronize(s));
  if (bulk_err) MF_FAIL(MF_ESTATE, "exact 2-hop sizes: a bulk-copy wait of the row pass ran out");
  if (dbg)
    std::fprintf(stderr, "[misfit_gb] pull sizes: seeds %lld of %lld in %zu passes, volume %.0f, positions %lld, "
                 "%.3f ms\n", (long long)pull.size(), (long long)ntodo, group_sizes.size(), pulled_vol,
                 (long long)positions, host_ms() - t0);
  return (int64_t)push.size();
}

// Exact 2-hop list sizes of the seeds into c->rowlens[0..ns).
// With bound_only, dense seeds get an upper bound (k_dense_bound) instead of
// their exact size, and the results go to the bound cache.
void exact_sizes(mf_ctx* c, int64_t ns, uint32_t ep, bool bound_only) {
  cudaStream_t s = c->stream;
  const int32_t n = c->n;
  const GraphView g = c->view();
  int64_t* h = c->h_counters;
  const int64_t words = ((int64_t)n + 31) / 32;
  if (c->bitmap_ctas == 0 || c->bitmap_words != words) {
    c->bitmap_words = words;
    int sms = 0;
    MF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
    const int64_t budget = (int64_t)1 << 31;  // bytes for the per-CTA private bitmaps
    const int64_t ctas = std::max<int64_t>(1, std::min<int64_t>((int64_t)sms * 2, budget / (words * 4)));
    c->bitmap_ctas = (int)ctas;
    c->bitmaps.release();
    c->bitmaps.reserve(ctas * words);
    MF_CUDA(cudaMemsetAsync(c->bitmaps.p, 0, sizeof(uint32_t) * (size_t)(ctas * words), s));
    // heavy-vertex bitmap cache: at most 2 GB and 4096 vertices
    c->heavy_cap = std::max<int64_t>(0, std::min<int64_t>(4096, ((int64_t)1 << 31) / (words * 4)));
    c->heavy_bits.release();
    if (c->heavy_cap > 0) c->heavy_bits.reserve(c->heavy_cap * words);
    c->heavy_list.reserve(std::max<int64_t>(n, 1));
    c->heavy_slot.reserve(std::max<int64_t>(n, 1));
    MF_CUDA(cudaMemsetAsync(c->heavy_slot.p, 0xFF, sizeof(int32_t) * (size_t)std::max<int32_t>(n, 1), s));
    c->heavy_used = 0;
  }
  const int64_t thr = std::max<int64_t>(c->tune.heavy_min, words / 8);
  // collect the heavy members of the seeds' closed neighbourhoods not cached yet
  h[30] = c->heavy_used;
  MF_CUDA(cudaMemcpyAsync(c->counters.p + 30, h + 30, sizeof(int64_t), cudaMemcpyHostToDevice, s));
  row_offsets(c, c->seeds.p, ns, kCntAll, ns, ep);
  MF_K(k_heavy_collect<<<lb_grid(c, k_heavy_collect), kTB, 0, s>>>(g, c->seeds.p, c->lb_offs.p, ns, thr, c->heavy_slot.p,
                                                  c->heavy_list.p,
                                                  reinterpret_cast<unsigned long long*>(c->counters.p) + 30));
  MF_CUDA(cudaMemcpyAsync(h + 30, c->counters.p + 30, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  MF_CUDA(cudaStreamSynchronize(s));
  const int64_t total = h[30];
  const int64_t from = c->heavy_used;
  if (total > from) {
    MF_K(k_heavy_assign<<<grid_for(total - from), kTB, 0, s>>>(c->heavy_list.p, from, total, c->heavy_cap,
                                                               c->heavy_slot.p));
    const int64_t build_to = std::min<int64_t>(total, c->heavy_cap);
    if (build_to > from) {
      MF_CUDA(cudaMemsetAsync(c->heavy_bits.p + from * words, 0,
                              sizeof(uint32_t) * (size_t)((build_to - from) * words), s));
      row_offsets(c, c->heavy_list.p + from, build_to - from, kCntAll, ns, ep);
      MF_K(k_heavy_build<<<lb_grid(c, k_heavy_build), kTB, 0, s>>>(g, c->heavy_list.p + from, c->lb_offs.p, build_to - from, from,
                                                     words, c->heavy_bits.p));
    }
    c->heavy_used = total;
  }
  if (ns == 0) return;
  // per-pass capacity of the dense bitmaps: 1 GB, at least one seed
  int64_t dmax = std::max<int64_t>(1, std::min<int64_t>(ns, ((int64_t)1 << 30) / (words * 4)));
  if (c->exact_cap_dense > 0) dmax = std::min<int64_t>(dmax, c->exact_cap_dense);
  c->dense_bits.reserve(dmax * words);
  c->dense_idx.reserve(3 * dmax);
  c->dense_light.reserve(dmax);
  c->dense_hl.reserve(std::max<int64_t>(kMaxHeavyPerSeed, std::min<int64_t>(dmax * 64, (int64_t)1 << 22)));
  int64_t pcap = std::max<int64_t>(4096, std::min<int64_t>((int64_t)1 << 26, 2 * c->nnz + 1));
  if (c->exact_cap_pairs > 0) pcap = std::min<int64_t>(pcap, c->exact_cap_pairs);
  c->pair_d.reserve(pcap);
  c->pair_h.reserve(pcap);
  c->todo.reserve(3 * ns);
  MF_CUDA(cudaMemsetAsync(c->counters.p + 44, 0, sizeof(int64_t), s));
  MF_K(k_exact_todo<<<grid_for(ns), kTB, 0, s>>>(c->seeds.p, ns, c->n2cache.p, c->n2stamp.p, c->n2bound.p,
                                                 c->n2bstamp.p, bound_only, c->n2batch, c->rowlens.p, c->todo.p,
                                                 reinterpret_cast<unsigned long long*>(c->counters.p) + 44));
  MF_CUDA(cudaMemcpyAsync(h + 44, c->counters.p + 44, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  MF_CUDA(cudaStreamSynchronize(s));
  const int64_t nnew = h[44];
  int32_t* computed = c->todo.p + 2 * ns;   // the seeds computed here, for the cache
  if (nnew > 0)
    MF_CUDA(cudaMemcpyAsync(computed, c->todo.p, sizeof(int32_t) * (size_t)nnew, cudaMemcpyDeviceToDevice, s));
  int32_t* todo = c->todo.p;
  int32_t* todo_next = c->todo.p + ns;
  int64_t ntodo = nnew;
  if (!bound_only) ntodo = pull_exact(c, todo, ntodo);
  unsigned long long* cnts = reinterpret_cast<unsigned long long*>(c->counters.p) + 40;
  while (ntodo > 0) {
    MF_CUDA(cudaMemsetAsync(cnts, 0, sizeof(unsigned long long) * 4, s));
    DenseOut o{cnts + 0, c->dense_idx.p, c->dense_idx.p + dmax, c->dense_idx.p + 2 * dmax, c->dense_hl.p, cnts + 1,
               c->pair_d.p, c->pair_h.p, cnts + 2, c->dense_light.p, dmax, c->dense_hl.cap, pcap};
    MF_K(k_exact_classify<<<(unsigned)std::min<int64_t>(c->bitmap_ctas, ntodo), 512, 0, s>>>(
        g, c->seeds.p, todo, ntodo, c->heavy_slot.p, words, c->bitmaps.p, words / 8, c->rowlens.p, o));
    MF_CUDA(cudaMemcpyAsync(h + 40, c->counters.p + 40, sizeof(int64_t) * 3, cudaMemcpyDeviceToHost, s));
    MF_CUDA(cudaStreamSynchronize(s));
    const int64_t nd = std::min<int64_t>((int64_t)h[40], dmax);
    const int64_t np = std::min<int64_t>((int64_t)h[42], pcap);
    const bool dbg = debug_counters();
    double dbg_t0 = dbg ? host_ms() : 0.0;
    if (nd > 0) {
      const dim3 grid((unsigned)nd, (unsigned)((words + kDenseTile - 1) / kDenseTile));
      MF_K(k_dense_or<<<grid, 256, 0, s>>>(nd, c->dense_idx.p, c->dense_idx.p + dmax, c->dense_idx.p + 2 * dmax,
                                           c->dense_hl.p, c->heavy_bits.p, words, c->dense_bits.p));
      if (np > 0 && !bound_only) {
        row_offsets_marked(c, c->pair_h.p, c->pair_d.p, np);
        MF_K(k_dense_light<<<lb_grid(c, k_dense_light), kTB, 0, s>>>(g, c->pair_d.p, c->pair_h.p, c->lb_offs.p, np, words,
                                                       c->dense_bits.p));
      }
      MF_K(k_dense_pop<<<grid, 256, 0, s>>>(nd, c->dense_idx.p, words, c->dense_bits.p, c->rowlens.p));
      if (bound_only)
        MF_K(k_dense_bound<<<grid_for(nd), kTB, 0, s>>>(nd, c->dense_idx.p, c->dense_light.p, n, c->rowlens.p));
    }
    if (dbg) {
      MF_CUDA(cudaStreamSynchronize(s));
      std::fprintf(stderr, "[misfit_gb] %s pass: seeds %lld dense %lld heavy-slots %lld light-pairs %lld "
                   "dense-ms %.3f\n", bound_only ? "bound" : "exact", (long long)ntodo, (long long)nd,
                   (long long)h[41], (long long)np, host_ms() - dbg_t0);
    }
    // seeds that did not fit this pass
    MF_CUDA(cudaMemsetAsync(cnts + 3, 0, sizeof(unsigned long long), s));
    MF_K(k_todo_retry<<<grid_for(ntodo), kTB, 0, s>>>(c->rowlens.p, todo, ntodo, todo_next, cnts + 3));
    MF_CUDA(cudaMemcpyAsync(h + 43, c->counters.p + 43, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    MF_CUDA(cudaStreamSynchronize(s));
    const int64_t left = h[43];
    if (left >= ntodo) MF_FAIL(MF_ESTATE, "exact 2-hop sizes made no progress");
    std::swap(todo, todo_next);
    ntodo = left;
  }
  if (nnew > 0)
    MF_K(k_exact_store<<<grid_for(nnew), kTB, 0, s>>>(c->seeds.p, computed, nnew, c->rowlens.p,
                                                      bound_only ? c->n2bound.p : c->n2cache.p,
                                                      bound_only ? c->n2bstamp.p : c->n2stamp.p, c->n2batch));
  MF_CUDA(cudaGetLastError());
}


// First-hit search of `pred` over the rows of list[0 .. *dcnt) into c->fpos;
// `upper` bounds *dcnt.  No host round trip: every level reads its count on
// the device.
template <class P>
void first_hits(mf_ctx* c, const int32_t* list, const unsigned long long* dcnt, int64_t upper, P pred,
                unsigned long long* qcnt) {
  cudaStream_t s = c->stream;
  const int64_t cap = std::max<int64_t>(upper, 1);
  c->fpos.reserve(cap);
  c->un_idx.reserve(cap);
  c->un_v.reserve(cap);
  c->un_cnt.reserve(cap);
  c->rq_idx.reserve(cap);
  c->rq_v.reserve(cap);
  const FirstQueues q{c->un_idx.p, c->un_v.p, qcnt, ChunkQueue{c->rq_idx.p, c->rq_v.p, c->un_cnt.p, qcnt + 1},
                      std::max<int64_t>(c->tune.first_bound, kProbe)};
  const GraphView g = c->view();
  MF_K(launch_pdl(k_first_probe<P>, lb_grid(c, k_first_probe<P>), kTB, 0, s, g, list, dcnt, pred, c->fpos.p, q));
  MF_K(launch_pdl(k_first_warp<P>, lb_grid(c, k_first_warp<P>), kTB, 0, s, g, pred, c->fpos.p, q));
  MF_K(launch_pdl(k_first_chunks<P>, lb_grid(c, k_first_chunks<P>), kTB, 0, s, g, pred, c->fpos.p, q));
  if (debug_counters()) {
    unsigned long long v[3] = {0, 0, 0};
    MF_CUDA(cudaStreamSynchronize(s));
    MF_CUDA(cudaMemcpy(v, dcnt, sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    MF_CUDA(cudaMemcpy(v + 1, qcnt, sizeof(unsigned long long) * 2, cudaMemcpyDeviceToHost));
    c->dbg_first[0] += 1;
    c->dbg_first[1] += (int64_t)v[0];
    c->dbg_first[2] += (int64_t)v[1];
    c->dbg_first[3] += (int64_t)(v[2] >> kChunkShift);
    c->dbg_first[4] += (int64_t)(v[2] & kChunkMask);
  }
}

void next_epoch(mf_ctx* c) {
  if (c->epoch >= kMaxEpoch) {
    cudaStream_t s = c->stream;
    MF_CUDA(cudaMemsetAsync(c->bval.p, 0, sizeof(uint32_t) * (size_t)c->n, s));
    MF_CUDA(cudaMemsetAsync(c->wval.p, 0, sizeof(uint32_t) * (size_t)c->n, s));
    MF_CUDA(cudaMemsetAsync(c->nmark.p, 0, sizeof(uint32_t) * (size_t)c->n, s));
    c->epoch = 0;
  }
  ++c->epoch;
}


bool sequential_repair_forced() {
  static const bool forced = [] {
    const char* e = std::getenv("MISFIT_GB_REPAIR");
    return e != nullptr && std::strcmp(e, "sequential") == 0;
  }();
  return forced;
}

// MISFIT_GB_REPAIR=rounds: every round read back by the host before the next
// is queued (instead of kRoundsPerSync rounds per read-back).
bool host_rounds_forced() {
  static const bool forced = [] {
    const char* e = std::getenv("MISFIT_GB_REPAIR");
    return e != nullptr && std::strcmp(e, "rounds") == 0;
  }();
  return forced;
}

// Repair of one sub-batch: c->vals holds the order (sub-batch indices),
// nproc entries.  Returns the number of speculative rounds.
int64_t repair(mf_ctx* c, const GraphView& g, int64_t p, int64_t nproc, int64_t ns) {
  cudaStream_t s = c->stream;
  int64_t* h = c->h_counters;
  unsigned long long* ucnt = reinterpret_cast<unsigned long long*>(c->counters.p);
  const uint32_t* order = c->vals.p;
  if (sequential_repair_forced()) {
    RepairArgs ra{g, c->bu.p, c->bv.p, c->bins.p, p, order, nproc, ns, c->v2i.p, c->mis.p};
    MF_K(k_repair_sequential<<<1, 1024, 0, s>>>(ra));
    MF_CUDA(cudaGetLastError());
    return 0;
  }
  c->rp_w0.reserve(nproc);
  c->rp_w1.reserve(nproc);
  c->rp_n0.reserve(nproc);
  c->rp_n1.reserve(nproc);
  c->rp_keys.reserve(2 * nproc);
  c->rp_vals.reserve(2 * nproc);
  c->rp_keys2.reserve(2 * nproc);
  c->rp_vals2.reserve(2 * nproc);
  c->rp_u8.reserve(2 * nproc);
  c->rp_pos.reserve(2 * nproc + 1);
  c->big_pos.reserve(nproc);
  c->big_r.reserve(nproc);
  c->big_off.reserve(nproc);
  c->big_nr.reserve(nproc);
  c->big_chunks.reserve(nproc + 1);
  c->big_best.reserve(nproc);
  c->big_pre.reserve(std::max<int64_t>(4096, std::min<int64_t>((int64_t)1 << 22, 4 * (int64_t)c->n)));
  if (c->big_grid == 0) {
    int sms = 0;
    MF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
    c->big_grid = 4 * sms;
  }
  const int nbits = bits_for(std::max<int32_t>(c->n - 1, 1));
  int64_t p0 = 0, nview = 0, rounds = 0;
  if (nproc <= kRoundCap && !host_rounds_forced() && !debug_counters()) {
    // Every round fits one commit block: rounds are queued kRoundsPerSync at
    // a time and read back once; a queued round finds its start and view on
    // the device and does nothing once the repair is done.  Round r writes
    // into one pair of result buffers and compares with the other, in turn.
    int64_t* dyn = c->counters.p + 58;
    MF_K(launch_pdl(k_repair_init, grid_for(std::max<int64_t>(nproc, 6)), kTB, 0, s, c->rp_w0.p, c->rp_w1.p, nproc,
                    dyn, c->counters.p + 24));
    std::optional<StageScope> dsc;
    int64_t queued = 0;
    while (true) {
      const int64_t k = std::min<int64_t>(kRoundsPerSync, kMaxRounds - queued);
      for (int64_t j = 0; j < k; ++j, ++queued) {
        const bool even = (queued & 1) == 0;
        int32_t* o0 = even ? c->rp_n0.p : c->rp_w0.p;
        int32_t* o1 = even ? c->rp_n1.p : c->rp_w1.p;
        int32_t* r0 = even ? c->rp_w0.p : c->rp_n0.p;
        int32_t* r1 = even ? c->rp_w1.p : c->rp_n1.p;
        SpecArgs a{g, c->bu.p, c->bv.p, c->bins.p, p, order, 0, nproc, ns, c->v2i.p,
                   View{c->mis.p, c->rp_keys.p, c->rp_vals.p, 0}, o0, o1, c->tune.big_threshold, ucnt + 24,
                   c->big_pos.p, c->big_r.p, c->big_off.p, c->big_nr.p, c->big_pre.p, ucnt + 25, c->big_pre.cap,
                   dyn};
        dsc.emplace(c, kStRepair);
        MF_K(launch_pdl(k_spec_eval, warps_grid(nproc), kTB, 0, s, a, c->big_chunks.p, c->big_best.p, ucnt + 26,
                        reinterpret_cast<unsigned int*>(ucnt + 29)));
        dsc.emplace(c, kStRepairBig);
        MF_K(launch_pdl(k_big_scan, (unsigned)c->big_grid, kBigChunk, 0, s, a, c->big_chunks.p, c->big_best.p,
                        ucnt + 26));
        dsc.emplace(c, kStRepair);
        MF_K(launch_pdl(k_spec_round, 1, kRoundThreads, 0, s, o0, o1, r0, r1, (int64_t)0, nproc, c->bins.p, p, order,
                        c->rp_keys.p, c->rp_vals.p, (int64_t)0, c->mis.p, ucnt + 20, a, c->big_best.p));
      }
      MF_CUDA(cudaMemcpyAsync(h + 58, dyn, sizeof(int64_t) * 4, cudaMemcpyDeviceToHost, s));
      MF_CUDA(cudaStreamSynchronize(s));
      dsc.reset();
      if (h[60] != 0) break;
      if (queued >= kMaxRounds) {
        // round limit: the rest in order by the sequential kernel
        p0 = h[58];
        nview = h[59];
        if (nview > 0) MF_K(k_spec_clear_flags<<<grid_for(nview), kTB, 0, s>>>(c->rp_keys.p, nview, c->mis.p));
        RepairArgs ra{g, c->bu.p, c->bv.p, c->bins.p, p, order + p0, nproc - p0, ns, c->v2i.p, c->mis.p};
        MF_K(k_repair_sequential<<<1, 1024, 0, s>>>(ra));
        MF_CUDA(cudaGetLastError());
        break;
      }
    }
    return h[61];
  }
  MF_CUDA(cudaMemsetAsync(c->rp_w0.p, 0xFF, sizeof(int32_t) * (size_t)nproc, s));
  MF_CUDA(cudaMemsetAsync(c->rp_w1.p, 0xFF, sizeof(int32_t) * (size_t)nproc, s));
  int64_t dbg_big = 0, dbg_chunks = 0, dbg_scanned = 0;
  std::optional<StageScope> rsc;
  rsc.emplace(c, kStRepair);
  while (p0 < nproc) {
    if (rounds >= kMaxRounds) {
      if (nview > 0) MF_K(k_spec_clear_flags<<<grid_for(nview), kTB, 0, s>>>(c->rp_keys.p, nview, c->mis.p));
      RepairArgs ra{g, c->bu.p, c->bv.p, c->bins.p, p, order + p0, nproc - p0, ns, c->v2i.p, c->mis.p};
      MF_K(k_repair_sequential<<<1, 1024, 0, s>>>(ra));
      MF_CUDA(cudaGetLastError());
      break;
    }
    ++rounds;
    const int64_t pending = nproc - p0;
    MF_CUDA(cudaMemsetAsync(c->counters.p + 24, 0, sizeof(int64_t) * 6, s));  // deferrals, prefix use, queue, done
    SpecArgs a{g, c->bu.p, c->bv.p, c->bins.p, p, order, p0, nproc, ns, c->v2i.p,
               View{c->mis.p, c->rp_keys.p, c->rp_vals.p, nview}, c->rp_n0.p, c->rp_n1.p,
               c->tune.big_threshold, ucnt + 24, c->big_pos.p, c->big_r.p, c->big_off.p, c->big_nr.p,
               c->big_pre.p, ucnt + 25, c->big_pre.cap};
    rsc.emplace(c, kStRepair);
    MF_K(launch_pdl(k_spec_eval, warps_grid(pending), kTB, 0, s, a, c->big_chunks.p, c->big_best.p, ucnt + 26,
                                                          reinterpret_cast<unsigned int*>(ucnt + 29)));
    rsc.emplace(c, kStRepairBig);
    MF_K(launch_pdl(k_big_scan, (unsigned)c->big_grid, kBigChunk, 0, s, a, c->big_chunks.p, c->big_best.p, ucnt + 26));
    rsc.emplace(c, kStRepair);
    if (pending <= kRoundCap) {
      // small round: one CTA finalizes the grid-wide searches and finishes
      // the round, one host round trip
      MF_K(launch_pdl(k_spec_round, 1, kRoundThreads, 0, s, c->rp_n0.p, c->rp_n1.p, c->rp_w0.p, c->rp_w1.p, p0, nproc, c->bins.p,
                                                    p, order, c->rp_keys.p, c->rp_vals.p, nview, c->mis.p, ucnt + 20,
                                                    a, c->big_best.p));
      MF_CUDA(cudaMemcpyAsync(h + 20, c->counters.p + 20, sizeof(int64_t) * 2, cudaMemcpyDeviceToHost, s));
      MF_CUDA(cudaStreamSynchronize(s));
      const int64_t f = h[20];
      if (debug_counters()) {
        unsigned long long q[4];
        MF_CUDA(cudaMemcpy(q, c->counters.p + 24, sizeof(q), cudaMemcpyDeviceToHost));
        int64_t tot = 0;
        if (q[0] > 0) MF_CUDA(cudaMemcpy(&tot, c->big_chunks.p + q[0], sizeof(tot), cudaMemcpyDeviceToHost));
        dbg_big += (int64_t)q[0];
        dbg_chunks += tot;
        dbg_scanned += (int64_t)q[3];
      }
      if (f >= nproc) break;
      nview = h[21];
      std::swap(c->rp_w0, c->rp_n0);
      std::swap(c->rp_w1, c->rp_n1);
      p0 = f + 1;
      continue;
    }
    MF_K(launch_pdl(k_big_finalize, grid_for(pending), kTB, 0, s, a, c->big_best.p));
    h[20] = (int64_t)nproc;
    MF_CUDA(cudaMemcpyAsync(c->counters.p + 20, h + 20, sizeof(int64_t), cudaMemcpyHostToDevice, s));
    MF_K(k_spec_first_change<<<grid_for(pending), kTB, 0, s>>>(c->rp_n0.p, c->rp_n1.p, c->rp_w0.p, c->rp_w1.p, p0,
                                                                 nproc, ucnt + 20));
    // all writes of this round, sorted by (vertex, position)
    MF_K(k_spec_count<<<grid_for(pending), kTB, 0, s>>>(c->rp_n0.p, c->rp_n1.p, p0, nproc, c->rp_u8.p));
    scan_exclusive_u8(c->rp_u8.p, c->rp_pos.p, pending, c->ws, s);
    MF_CUDA(cudaMemcpyAsync(h + 21, c->rp_pos.p + pending, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    MF_CUDA(cudaMemcpyAsync(h + 20, c->counters.p + 20, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    MF_K(k_spec_fill<<<grid_for(pending), kTB, 0, s>>>(c->rp_n0.p, c->rp_n1.p, c->rp_pos.p, p0, nproc, c->bu.p,
                                                         c->bv.p, c->bins.p, p, order, c->rp_keys2.p,
                                                         c->rp_vals2.p));
    MF_CUDA(cudaStreamSynchronize(s));
    const int64_t f = h[20];          // first changed position, nproc when none
    const int64_t nk = h[21];
    if (debug_counters()) {
      unsigned long long q[4];
      MF_CUDA(cudaMemcpy(q, c->counters.p + 24, sizeof(q), cudaMemcpyDeviceToHost));
      int64_t tot = 0;
      if (q[0] > 0) MF_CUDA(cudaMemcpy(&tot, c->big_chunks.p + q[0], sizeof(tot), cudaMemcpyDeviceToHost));
      dbg_big += (int64_t)q[0];
      dbg_chunks += tot;
      dbg_scanned += (int64_t)q[3];
    }
    radix_sort_pairs(c->rp_keys2.p, c->rp_vals2.p, nk, 32 + nbits, c->ws, s);
    if (nview > 0) MF_K(k_spec_clear_flags<<<grid_for(nview), kTB, 0, s>>>(c->rp_keys.p, nview, c->mis.p));
    const uint64_t last = (uint64_t)std::min<int64_t>(f, nproc - 1);
    if (nk > 0) MF_K(k_spec_commit<<<grid_for(nk), kTB, 0, s>>>(c->rp_keys2.p, c->rp_vals2.p, nk, last, c->mis.p));
    if (f >= nproc) break;
    nview = 0;
    if (nk > 0) {
      MF_K(k_spec_keep_flags<<<grid_for(nk), kTB, 0, s>>>(c->rp_keys2.p, nk, last, c->mis.p, c->rp_u8.p));
      scan_exclusive_u8(c->rp_u8.p, c->rp_pos.p, nk, c->ws, s);
      MF_K(k_spec_compact<<<grid_for(nk), kTB, 0, s>>>(c->rp_keys2.p, c->rp_vals2.p, c->rp_u8.p, c->rp_pos.p, nk,
                                                         c->rp_keys.p, c->rp_vals.p));
      MF_CUDA(cudaMemcpyAsync(h + 22, c->rp_pos.p + nk, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
      MF_CUDA(cudaStreamSynchronize(s));
      nview = h[22];
    }
    std::swap(c->rp_w0, c->rp_n0);
    std::swap(c->rp_w1, c->rp_n1);
    p0 = f + 1;
  }
  MF_CUDA(cudaGetLastError());
  if (debug_counters() && dbg_scanned > 0)
    std::fprintf(stderr, "[misfit_gb] repair: nproc %lld rounds %lld deferred %lld chunks %lld scanned %lld\n",
                 (long long)nproc, (long long)rounds, (long long)dbg_big, (long long)dbg_chunks,
                 (long long)dbg_scanned);
  return rounds;
}

}  // namespace

void process_batch(mf_ctx* c, int64_t m) {
  cudaStream_t s = c->stream;
  const int32_t n = c->n;
  const GraphView g = c->view();
  int64_t* cnt = c->counters.p;
  unsigned long long* ucnt = reinterpret_cast<unsigned long long*>(cnt);
  int64_t* h = c->h_counters;

  if (c->profile & 4) MF_CUDA(cudaMemsetAsync(cnt + 56, 0, sizeof(int64_t) * 2, s));
  // previous occurrence of every endpoint slot (for "not seen in this sub-batch")
  const int sbits = bits_for(std::max<int64_t>(2 * m - 1, 1));
  const int nbits = bits_for(std::max<int32_t>(n - 1, 1));
  c->keys.reserve(2 * m);
  c->vals.reserve(2 * m);
  c->prev.reserve(2 * m);
  std::optional<StageScope> sc;
  sc.emplace(c, kStSplit);
  MF_K(k_slot_keys<<<grid_for(2 * m), kTB, 0, s>>>(c->bu.p, c->bv.p, m, sbits, c->keys.p, c->vals.p));
  radix_sort_pairs(c->keys.p, c->vals.p, 2 * m, sbits + nbits, c->ws, s);
  MF_K(k_prev<<<grid_for(2 * m), kTB, 0, s>>>(c->keys.p, c->vals.p, 2 * m, sbits, c->prev.p));
  MF_CUDA(cudaGetLastError());
  sc.reset();

  if (c->heavy_used > 0) {
    MF_K(k_heavy_reset<<<grid_for(c->heavy_used), kTB, 0, s>>>(c->heavy_list.p, c->heavy_used, c->heavy_slot.p));
    c->heavy_used = 0;
  }
  // exact 2-hop sizes stay valid for the rows of this batch only
  c->n2cache.reserve(std::max<int32_t>(n, 1));
  c->n2stamp.reserve(std::max<int32_t>(n, 1));
  c->n2bound.reserve(std::max<int32_t>(n, 1));
  c->n2bstamp.reserve(std::max<int32_t>(n, 1));
  if (c->n2batch == 0 || c->n2batch == 0xffffffffu) {
    MF_CUDA(cudaMemsetAsync(c->n2stamp.p, 0, sizeof(uint32_t) * (size_t)std::max<int32_t>(n, 1), s));
    MF_CUDA(cudaMemsetAsync(c->n2bstamp.p, 0, sizeof(uint32_t) * (size_t)std::max<int32_t>(n, 1), s));
    c->n2batch = 0;
  }
  ++c->n2batch;
  const int64_t big = 2 * std::min<int64_t>(m, kMaxBatchEdges) + (int64_t)n + 2;
  c->i64a.reserve(big);
  c->i64b.reserve(big);
  c->u8a.reserve(big);
  c->seeds.reserve(2 * std::min<int64_t>(m, kMaxBatchEdges));
  c->cands.reserve(kMaxRows);
  c->rowcid.reserve(kMaxRows + 2 * std::min<int64_t>(m, kMaxBatchEdges));
  c->creates.reserve(kMaxRows + 2 * std::min<int64_t>(m, kMaxBatchEdges));
  c->rowlens.reserve(kMaxRows + 2 * std::min<int64_t>(m, kMaxBatchEdges) + 1);

  // ---- sub-batch plan: cuts, estimates and seed lists of the whole batch
  // from p0 (re-planned from the next sub-batch when MAX_CSR_ELEMENTS grows)
  c->plan_cuts.reserve(std::max<int64_t>(m, 1));
  c->plan_ests.reserve(std::max<int64_t>(m, 1));
  c->plan_send.reserve(std::max<int64_t>(m, 1));
  c->plan_flags.reserve(2 * m);
  c->plan_pos.reserve(2 * m + 1);
  c->seeds_all.reserve(2 * m);
  std::vector<int64_t> cuts, ests, seed_end;
  size_t kidx = 0;
  int64_t seed_base = 0;
  auto plan = [&](int64_t p0) {
    sc.emplace(c, kStSplit);
    unsigned long long* kcount = ucnt + 37;
    MF_K(k_cuts<<<1, kCutThreads, 0, s>>>(c->bu.p, c->bv.p, c->prev.p, c->deg.p, m, p0, c->max_csr,
                                          c->plan_cuts.p, c->plan_ests.p, kcount));
    const int64_t nslots = 2 * (m - p0);
    MF_K(k_plan_seed_flags<<<grid_for(nslots), kTB, 0, s>>>(c->prev.p, c->plan_cuts.p, kcount, m, p0,
                                                              c->plan_flags.p));
    scan_exclusive_u8(c->plan_flags.p, c->plan_pos.p, nslots, c->ws, s);
    MF_K(k_plan_seed_compact<<<grid_for(nslots), kTB, 0, s>>>(c->bu.p, c->bv.p, c->plan_flags.p, c->plan_pos.p, m,
                                                                p0, c->seeds_all.p));
    MF_K(k_plan_seed_ends<<<grid_for(m - p0), kTB, 0, s>>>(c->plan_cuts.p, kcount, c->plan_pos.p, p0,
                                                             c->plan_send.p));
    MF_CUDA(cudaMemcpyAsync(h + 37, cnt + 37, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    MF_CUDA(cudaStreamSynchronize(s));
    const int64_t nk = h[37];
    cuts.resize((size_t)nk);
    ests.resize((size_t)nk);
    seed_end.resize((size_t)nk);
    MF_CUDA(cudaMemcpyAsync(cuts.data(), c->plan_cuts.p, sizeof(int64_t) * (size_t)nk, cudaMemcpyDeviceToHost, s));
    MF_CUDA(cudaMemcpyAsync(ests.data(), c->plan_ests.p, sizeof(int64_t) * (size_t)nk, cudaMemcpyDeviceToHost, s));
    MF_CUDA(cudaMemcpyAsync(seed_end.data(), c->plan_send.p, sizeof(int64_t) * (size_t)nk, cudaMemcpyDeviceToHost,
                            s));
    MF_CUDA(cudaStreamSynchronize(s));
    kidx = 0;
    seed_base = 0;
    sc.reset();
  };
  plan(0);

  // the first sub-batch's front, on this stream.  Later fronts overlap the
  // previous sub-batch on the second stream for large graphs; for small ones
  // the stream switch costs more than the front, which then runs inline.
  const bool overlap_fronts = c->n >= (1 << 20);
  front_reserve(c, m);
  int cur = 0;
  bool front_on_b = false;
  front_compute(c, c->front[0], c->seeds_all.p, seed_end.empty() ? 0 : seed_end[0], s);

  int64_t p = 0;
  while (p < m) {
    if (kidx >= cuts.size()) MF_FAIL(MF_ESTATE, "sub-batch plan ended before the batch");
    const int64_t q = cuts[kidx];
    const int64_t est = ests[kidx];
    const int64_t ns = seed_end[kidx] - seed_base;

    // ---- seeds (first appearance) of this sub-batch into their rows
    sc.emplace(c, kStSeeds);
    if (ns > 0)
      MF_K(launch_pdl(k_seed_rows, grid_for(ns), kTB, 0, s, c->seeds_all.p + seed_base, ns, c->seeds.p, c->v2i.p));
    const int64_t max_before = c->max_csr;

    // ---- hop-1 set and size bound: this sub-batch's front (computed on the
    // second stream while the previous sub-batch ran, or just now for the
    // first one); its lists become the context's
    sc.emplace(c, kStHop1);
    next_epoch(c);
    const uint32_t ep = c->epoch;
    Front& fr = c->front[cur];
    if (front_on_b) MF_CUDA(cudaStreamWaitEvent(s, c->ev_b, 0));
    std::swap(c->hlist, fr.hlist);
    std::swap(c->cands, fr.cands);

    // ---- packed sizes (upper bound) and MAX_CSR_ELEMENTS growth.  The
    // hop-1 counts and the bound: a front computed on the second stream
    // copied them to its own host slot there, and by now has long finished,
    // so this stream keeps its queue; otherwise one round trip here.
    sc.emplace(c, kStSizes);
    if (front_on_b) {
      MF_CUDA(cudaEventSynchronize(c->ev_b));
      h[2] = h[kFrontSlot + 2 * cur];
      h[3] = h[kFrontSlot + 2 * cur + 1];
    } else {
      MF_CUDA(cudaMemcpyAsync(h + 2, fr.cnt.p, sizeof(int64_t) * 2, cudaMemcpyDeviceToHost, s));
      MF_CUDA(cudaStreamSynchronize(s));
    }
    h[4] = h[3];
    h[3] = h[2] & 0xffffffffll;
    h[2] = h[2] >> 32;
    const int64_t nh = h[2];
    const int64_t capc = std::max<int64_t>(0, kMaxRows - ns);
    const int64_t nct = std::min<int64_t>(h[3], capc);
    const int64_t rows = ns + nct;
    if (nct > 0) MF_K(launch_pdl(k_cand_v2i, grid_for(nct), kTB, 0, s, c->cands.p, nct, ns, c->v2i.p));
    int64_t packed = -1;
    int64_t cand_total = h[4];   // entries of the candidate rows: the bound, exact below if sized
    const bool exact = h[4] >= c->max_csr;
    if (exact) {
      // The limit grows only if the packed total reaches it.  A tighter upper
      // bound (exact sizes except for the light part of dense seeds) settles
      // most of these sub-batches; the exact sizes follow only if it does not.
      // Where the bound has stopped settling them (hub-dominated graphs, whose
      // packed totals sit at the limit), it is tried on one sub-batch in
      // eight only, and the exact sizes are computed directly; either way
      // the growth comes from exact sizes, so results do not depend on it.
      sc.emplace(c, kStExact);
      MF_K(k_cand_lens<<<grid_for(nct), kTB, 0, s>>>(g, c->cands.p, nct, c->rowlens.p + ns));
      const bool bound_useful = c->bound_tries < 8 || __builtin_popcount(c->bound_hist & 0xffu) >= 2;
      bool settled = false;
      if (bound_useful || (++c->bound_skips & 7) == 0) {
        exact_sizes(c, ns, ep, true);
        scan_exclusive_i64(c->rowlens.p, c->i64a.p, rows, c->ws, s);
        MF_CUDA(cudaMemcpyAsync(h + 6, c->i64a.p + rows, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        MF_CUDA(cudaMemcpyAsync(h + 8, c->i64a.p + ns, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        MF_CUDA(cudaStreamSynchronize(s));
        settled = h[6] < c->max_csr;
        cand_total = h[6] - h[8];   // the candidates' lengths are exact in the bound too
        c->bound_hist = (c->bound_hist << 1) | (settled ? 1u : 0u);
        ++c->bound_tries;
      }
      if (!settled) {
        exact_sizes(c, ns, ep, false);
        scan_exclusive_i64(c->rowlens.p, c->i64a.p, rows, c->ws, s);
        h[5] = c->max_csr;
        MF_CUDA(cudaMemcpyAsync(cnt + 5, h + 5, sizeof(int64_t), cudaMemcpyHostToDevice, s));
        MF_K(k_growth<<<1, 32, 0, s>>>(c->i64a.p, rows, cnt + 5));
        MF_CUDA(cudaMemcpyAsync(h + 5, cnt + 5, sizeof(int64_t) * 2, cudaMemcpyDeviceToHost, s));
        MF_CUDA(cudaMemcpyAsync(h + 8, c->i64a.p + ns, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        MF_CUDA(cudaStreamSynchronize(s));
        c->max_csr = h[5];
        packed = h[6];
        cand_total = h[6] - h[8];
        c->stats.exact_sizes += 1;
      }
    }
    if (c->profile & 4) {
      // the algorithmic accounting needs every row's exact length: the
      // seeds' exact 2-hop sizes unless the growth check computed them
      if (packed < 0) {
        exact_sizes(c, ns, ep, false);
        if (nct > 0) MF_K(k_cand_lens<<<grid_for(nct), kTB, 0, s>>>(g, c->cands.p, nct, c->rowlens.p + ns));
      }
      if (rows > 0)
        MF_K(k_acct<<<(unsigned)std::min<int64_t>((rows + kTB - 1) / kTB, 1024), kTB, 0, s>>>(
            c->rowlens.p, rows, c->seeds.p, ns, c->cands.p, c->deg.p, ucnt + 56));
    }
    MF_CUDA(cudaGetLastError());

    // ---- the next sub-batch: re-plan after a growth of the limit, then its
    // front on the second stream, after everything issued so far on this one
    size_t kidx_next = kidx + 1;
    int64_t seed_base_next = seed_end[kidx];
    if (c->max_csr != max_before && q < m) {
      plan(q);  // the cuts after a growth follow the new limit
      kidx_next = 0;
      seed_base_next = 0;
    }
    front_on_b = false;
    if (q < m) {
      if (kidx_next >= cuts.size()) MF_FAIL(MF_ESTATE, "sub-batch plan ended before the batch");
      const int64_t ns_next = seed_end[kidx_next] - seed_base_next;
      if (overlap_fronts) {
        MF_CUDA(cudaEventRecord(c->ev_a, s));
        MF_CUDA(cudaStreamWaitEvent(c->stream_b, c->ev_a, 0));
        g_alloc_stream = c->stream_b;   // any scratch the front's scans grow belongs to its stream
        front_compute(c, c->front[cur ^ 1], c->seeds_all.p + seed_base_next, ns_next, c->stream_b);
        MF_CUDA(cudaMemcpyAsync(h + kFrontSlot + 2 * (cur ^ 1), c->front[cur ^ 1].cnt.p, sizeof(int64_t) * 2,
                                cudaMemcpyDeviceToHost, c->stream_b));
        g_alloc_stream = s;
        MF_CUDA(cudaEventRecord(c->ev_b, c->stream_b));
        front_on_b = true;
      } else {
        front_compute(c, c->front[cur ^ 1], c->seeds_all.p + seed_base_next, ns_next, s);
      }
    }

    // ---- clustering (bulk-synchronous); counts stay on the device
    sc.emplace(c, kStFirst);
    c->live_i.reserve(std::max<int64_t>(rows, 1));
    c->live_v.reserve(std::max<int64_t>(rows, 1));
    c->need.reserve(std::max<int64_t>(ns, 1));
    c->needv.reserve(std::max<int64_t>(ns, 1));
    c->mq_idx.reserve(std::max<int64_t>(ns, 1));
    c->mq_v.reserve(std::max<int64_t>(ns, 1));
    c->mq_base.reserve(std::max<int64_t>(ns, 1));
    // [33] live rows, [34] need seeds, [35] their neighbours, [36] the pull's
    // long rows; [48, 49], [51, 52], [53, 54] the queues of the three
    // first-hit searches, [50] the chunk queue of the need seeds' rows, [55]
    // the assignment's count
    MF_CUDA(cudaMemsetAsync(cnt + 33, 0, sizeof(int64_t) * 4, s));
    MF_CUDA(cudaMemsetAsync(cnt + 48, 0, sizeof(int64_t) * 8, s));
    const ChunkQueue mq{c->mq_idx.p, c->mq_v.p, c->mq_base.p, ucnt + 50};
    MF_K(launch_pdl(k_row_skip, grid_for(rows), kTB, 0, s, c->seeds.p, ns, c->cands.p, nct, c->cid.p, c->rowcid.p,
                                                    c->creates.p, c->live_i.p, c->live_v.p, ucnt + 33));
    c->cidbits.reserve(((int64_t)n + 31) / 32 + 1);
    MF_K(launch_pdl(k_cid_bits, warps_grid(((int64_t)n + kCidBitsPerWarp - 1) / kCidBitsPerWarp), kTB, 0, s, c->cid.p, n,
                    c->cidbits.p));
    const HasCidBit has_cid{c->cidbits.p};
    first_hits(c, c->live_v.p, ucnt + 33, rows, has_cid, ucnt + 48);
    MF_K(launch_pdl(k_live_decide, lb_grid(c, k_live_decide), kTB, 0, s, g, c->live_i.p, c->live_v.p, ucnt + 33, ns,
                                                                 c->fpos.p, c->cid.p, c->rowcid.p, c->creates.p,
                                                                 c->seeds.p, c->need.p, c->needv.p, ucnt + 34, mq));
    sc.emplace(c, kStFirstNeed);
    MF_K(launch_pdl(k_mark_need, lb_grid(c, k_mark_need), kTB, 0, s, g, mq, ep, c->nmark.p, c->nlist_need.p, ucnt + 35));
    first_hits(c, c->nlist_need.p, ucnt + 35, n, has_cid, ucnt + 51);
    MF_K(launch_pdl(k_f1_finish, lb_grid(c, k_f1_finish), kTB, 0, s, g, c->nlist_need.p, ucnt + 35, c->fpos.p, c->cid.p,
                                                             c->f1.p));
    first_hits(c, c->needv.p, ucnt + 34, ns, HasF1{c->f1.p}, ucnt + 53);
    MF_K(launch_pdl(k_need_decide, lb_grid(c, k_need_decide), kTB, 0, s, g, c->need.p, c->needv.p, ucnt + 34, c->fpos.p,
                                                                 c->f1.p, c->rowcid.p, c->creates.p));
    scan_exclusive_u8(c->creates.p, c->i64b.p, rows, c->ws, s);
    MF_K(launch_pdl(k_new_ids, grid_for(rows), kTB, 0, s, rows, c->i64b.p, c->rowcid.p, c->seeds.p, ns, ep,
                    c->bval.p));
    MF_CUDA(cudaMemcpyAsync(h + 7, c->i64b.p + rows, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    sc.emplace(c, kStPush);
    unsigned long long* wk_extra = c->work.p + 2 * kStCount;   // [0] seed, [1] hop, [2] candidate pushes
    row_offsets(c, c->seeds.p, ns, kCntSeedRows, ns, ep);
    MF_K(launch_pdl(k_lb_push_seed, lb_grid(c, k_lb_push_seed), kTB, 0, s, g, c->seeds.p, c->lb_offs.p, ns, ep, c->bval.p, wk_extra + 0));
    MF_K(launch_pdl(k_self_push, grid_for(ns + nh), kTB, 0, s, c->seeds.p, ns, c->hlist.p, nh, ep, c->bval.p,
                    c->wval.p));
    row_offsets(c, c->seeds.p, ns, kCntSeedPushers, ns, ep);
    const unsigned long long dbg0 = debug_launches() ? debug_counter(c, wk_extra + 1) : 0;
    sc.emplace(c, kStPushHop);
    MF_K(launch_pdl(k_lb_push_hop, lb_grid(c, k_lb_push_hop), kTB, 0, s, g, c->seeds.p, c->lb_offs.p, ns, ep, c->bval.p,
                                                                 c->wval.p, wk_extra + 1));
    sc.emplace(c, kStPush);
    if (debug_launches()) debug_push_hop(c, wk_extra + 1, dbg0);
    row_offsets(c, c->hlist.p, nh, kCntHopPushers, ns, ep);
    const unsigned long long dbg1 = debug_launches() ? debug_counter(c, wk_extra + 1) : 0;
    sc.emplace(c, kStPushHop);
    MF_K(launch_pdl(k_lb_push_hop, lb_grid(c, k_lb_push_hop), kTB, 0, s, g, c->hlist.p, c->lb_offs.p, nh, ep, c->bval.p,
                                                                 c->wval.p, wk_extra + 1));
    sc.emplace(c, kStPush);
    if (debug_launches()) debug_push_hop(c, wk_extra + 1, dbg1);
    // Pull or push.  The pull costs ~28 B per vertex plus 4 B per row entry
    // it reads (as many per vertex as in the last batch that pulled); the
    // push at most 12 B per entry of the candidate rows plus the 8 B per
    // vertex of its finalising pass.  With cand_push 0 the push is taken
    // when that bound is under half the pull's estimate (sparse candidate
    // rows on a large graph, where the pull walks most rows to their end).
    bool use_pull = c->symmetric && c->rows_sorted && c->tune.cand_push != 1;
    if (use_pull && c->tune.cand_push == 0) {
      const double push_b = 12.0 * (double)cand_total + 8.0 * (double)n;
      const double pull_b = (28.0 + 4.0 * c->pull_visit_ratio) * (double)n;
      if (2.0 * push_b < pull_b) use_pull = false;
    }
    sc.emplace(c, use_pull ? kStPull : kStPush);
    if (use_pull) {
      ++c->pull_runs;
      c->pull_long.reserve(std::max<int32_t>(n, 1));
      const int64_t nwords = ((int64_t)n + 31) / 32;
      c->ncbits.reserve(std::max<int64_t>(nwords, 1));
      MF_CUDA(cudaMemsetAsync(c->ncbits.p, 0, sizeof(uint32_t) * (size_t)nwords, s));   // [36] zeroed above
      if (nct > 0)
        MF_K(launch_pdl(k_cand_bits, grid_for(nct), kTB, 0, s, c->cands.p, nct, ns, c->rowcid.p, c->ncbits.p));
      const PullArgs pa{g,  c->v2i.p, c->rowcid.p, c->ncbits.p, ns, c->wval.p, ep, c->cid.p, c->pull_long.p,
                        ucnt + 36, wk_extra + 2, c->tune.pull_long};
      MF_K(launch_pdl(k_pull_cand, grid_for(n), kTB, 0, s, pa));
      MF_K(launch_pdl(k_pull_cand_long, lb_grid(c, k_pull_cand_long), kTB, 0, s, pa));
      // per vertex: row bounds (8 B of nindex, 8 B of aoff), tombstone count,
      // tag and id (4 B each); the row entries read are counted on the device
      if (c->profile) c->stage_bytes[kStPull] += 28.0 * (double)n;
    } else {
      row_offsets(c, c->cands.p, nct, kCntCandRows, ns, ep);
      MF_K(launch_pdl(k_lb_push_cand, lb_grid(c, k_lb_push_cand), kTB, 0, s, g, c->cands.p, c->lb_offs.p, nct, ns, ep, c->wval.p,
                                                     wk_extra + 3));
      MF_K(launch_pdl(k_finalize_all, grid_for(((int64_t)n + 3) / 4), kTB, 0, s, c->wval.p, n, ep, c->rowcid.p, c->cid.p));
    }
    c->touched_total += n;
    MF_CUDA(cudaGetLastError());

    sc.reset();
    SubBatchTrace* tr = nullptr;
    if (c->trace) {
      c->traces.emplace_back();
      tr = &c->traces.back();
      tr->hdr[0] = p; tr->hdr[1] = q; tr->hdr[2] = ns; tr->hdr[3] = nct; tr->hdr[4] = packed;
      tr->hdr[5] = c->max_csr; tr->hdr[8] = rows; tr->hdr[9] = est;   // hdr[6] after the assignment
      tr->seeds = fetch(c->seeds.p, ns, s);
      tr->cands = fetch(c->cands.p, nct, s);
      tr->cid_after = fetch(c->cid.p, n, s);
      if (packed >= 0) tr->row_len = fetch(c->rowlens.p, rows, s);
    }

    // ---- assignment + order (cluster ascending, index descending)
    sc.emplace(c, kStAssign);
    MF_K(launch_pdl(k_assign, grid_for(q - p), kTB, 0, s, c->bu.p, c->bv.p, p, q - p, c->cid.p, c->i64b.p + rows, c->keys.p,
                                                  c->vals.p, ucnt + 55));
    MF_CUDA(cudaMemcpyAsync(h + 9, cnt + 55, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    MF_CUDA(cudaStreamSynchronize(s));
    const int64_t cc = h[7];
    const int64_t limit = std::min<int64_t>(cc, kMaxBatchEdges);
    const int64_t nproc = h[9];
    if (tr) tr->hdr[6] = cc;
    radix_sort_pairs(c->keys.p, c->vals.p, nproc, kRowBits + bits_for(std::max<int64_t>(limit, 1)), c->ws, s);

    // ---- repair (times itself: rounds vs grid-wide searches)
    sc.reset();
    if (nproc > 0) c->stats.repair_rounds += repair(c, g, p, nproc, ns);
    sc.reset();
    if (tr) {
      tr->hdr[7] = nproc;
      std::vector<uint32_t> ord = fetch(c->vals.p, nproc, s);
      tr->order.resize(ord.size());
      for (size_t i = 0; i < ord.size(); ++i) tr->order[i] = (int32_t)(p + ord[i]);
      tr->mis_after = fetch(c->mis.p, n, s);
    }

    // ---- clear (mapped vertices only)
    sc.emplace(c, kStClear);
    MF_K(launch_pdl(k_clear, grid_for(rows), kTB, 0, s, c->seeds.p, ns, c->cands.p, nct, c->cid.p, c->v2i.p));
    MF_CUDA(cudaGetLastError());

    sc.reset();
    c->stats.sub_batches += 1;
    c->stats.seeds += ns;
    c->stats.candidates += nct;
    c->stats.clusters += cc;
    c->stats.processed_edges += nproc;
    p = q;
    seed_base = seed_base_next;
    kidx = kidx_next;
    cur ^= 1;
  }
  if (front_on_b) MF_CUDA(cudaStreamSynchronize(c->stream_b));
  c->stats.max_csr = c->max_csr;
  if (c->profile & 4) {
    MF_CUDA(cudaMemcpyAsync(h + 56, cnt + 56, sizeof(int64_t) * 2, cudaMemcpyDeviceToHost, s));
    MF_CUDA(cudaStreamSynchronize(s));
    c->stats.packed_total = h[56];
    c->stats.row_degree_total = h[57];
  }
}

}  // namespace mf
