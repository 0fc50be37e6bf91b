// mf_cta.cuh -- one update batch of one graph, executed by a single CTA.
//
// This is the engine of the batched form (mf_apply_batches): a persistent
// kernel takes graph batches from a device work queue, and the CTA that
// takes an item runs that graph's whole path for the batch -- overlay apply,
// split rule, seeds and candidates, packed-size growth, clustering read and
// write, assignment order, MIS repair, clear -- with block-wide barriers
// between the stages and no host round trip.  It computes exactly what the
// multi-launch path in mf_overlay.cu / mf_repair.cu computes (the same
// canonical schedule) on the same device state of an mf_ctx, so a graph can
// take one batch here and the next through mf_apply_batch.
//
// Reference, src/misfit/misfit.cu of anonymous-artifacts/MISFIT:
//   batch apply          :704-716 and core/FlashGraph.h:172-276
//   split and seeds      :486-523
//   2-hop rows           :159-202, candidate rows :550-558
//   packing and growth   :560-599
//   clustering           :219-259, assignment :261-275
//   repair               :277-349, clear :351-358
//
// Portability: the file is CUDA, but it also compiles as plain C++ so that
// tests can run one CTA on the CPU (one OS thread per CUDA thread, a real
// barrier for __syncthreads, function-static variables for __shared__ ones).
// Everything here therefore uses only block-level constructs: barriers,
// shared memory and atomics; no warp intrinsics.  Every value that steers
// control flow around a barrier is read from shared memory after a barrier,
// so all threads take the same path.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define CTA_FN __device__ __forceinline__
#define CTA_SHARED __shared__
#define CTA_SYNC() __syncthreads()
#define CTA_TID ((int)threadIdx.x)
#define CTA_NT ((int)blockDim.x)
#else
#define CTA_FN inline
#define CTA_SHARED static
#define CTA_SYNC() ::mf::cta::emul_sync()
#define CTA_TID (::mf::cta::emul_tid)
#define CTA_NT (::mf::cta::emul_nt)
#endif

namespace mf {
namespace cta {

#if !defined(__CUDACC__)
// CPU execution of one CTA (test harness only): provided by the harness.
extern thread_local int emul_tid;
extern int emul_nt;
void emul_sync();
inline int32_t at_add(int32_t* p, int32_t v) { return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST); }
inline unsigned long long at_add(unsigned long long* p, unsigned long long v) {
  return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST);
}
inline uint32_t at_or(uint32_t* p, uint32_t v) { return __atomic_fetch_or(p, v, __ATOMIC_SEQ_CST); }
inline uint32_t at_and(uint32_t* p, uint32_t v) { return __atomic_fetch_and(p, v, __ATOMIC_SEQ_CST); }
inline uint32_t at_max(uint32_t* p, uint32_t v) {
  uint32_t cur = __atomic_load_n(p, __ATOMIC_SEQ_CST);
  while (cur < v && !__atomic_compare_exchange_n(p, &cur, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {
  }
  return cur;
}
inline unsigned long long at_min(unsigned long long* p, unsigned long long v) {
  unsigned long long cur = __atomic_load_n(p, __ATOMIC_SEQ_CST);
  while (cur > v && !__atomic_compare_exchange_n(p, &cur, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {
  }
  return cur;
}
inline int popc32(uint32_t x) { return __builtin_popcount(x); }
inline int ffs32(uint32_t x) { return __builtin_ffs((int)x); }
inline uint64_t now_ns() { return 0; }
#else
CTA_FN int32_t at_add(int32_t* p, int32_t v) { return atomicAdd(p, v); }
CTA_FN unsigned long long at_add(unsigned long long* p, unsigned long long v) { return atomicAdd(p, v); }
CTA_FN uint32_t at_or(uint32_t* p, uint32_t v) { return atomicOr(p, v); }
CTA_FN uint32_t at_and(uint32_t* p, uint32_t v) { return atomicAnd(p, v); }
CTA_FN uint32_t at_max(uint32_t* p, uint32_t v) { return atomicMax(p, v); }
CTA_FN unsigned long long at_min(unsigned long long* p, unsigned long long v) { return atomicMin(p, v); }
CTA_FN int popc32(uint32_t x) { return __popc(x); }
CTA_FN int ffs32(uint32_t x) { return __ffs((int)x); }
CTA_FN uint64_t now_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
#endif

// Constants of the reference engine (src/misfit/misfit.cu:37,503-506,560).
constexpr int64_t kMaxBatchEdges = 1048576;
constexpr int64_t kMaxRows = 2 * kMaxBatchEdges;
constexpr int64_t kEstimateWeight = 1000;
// Clustering-write tags: epoch in the high bits, row index (< 2^21) low.
constexpr int kTagBits = 21;
constexpr uint32_t kTagMask = (1u << kTagBits) - 1;
constexpr uint32_t kMaxEpoch = (1u << (32 - kTagBits)) - 1;
constexpr int kMaxThreads = 1024;
constexpr int kBuckets = 16;          // radix digit of 4 bits
constexpr int64_t kRankSortMax = 2048;
// Shared memory the caller provides: kMaxThreads int64 + kBuckets*kMaxThreads int32.
constexpr int kSmemBytes = kMaxThreads * 8 + kBuckets * kMaxThreads * 4;

// Outputs per item (int64 words).
enum : int {
  kOutATotal = 0,   // added entries after the batch
  kOutSwapped,      // 1 if the added CSR was rebuilt into the *_new arrays
  kOutMaxCsr,       // MAX_CSR_ELEMENTS after the batch
  kOutSubBatches,
  kOutSeeds,
  kOutCands,
  kOutClusters,
  kOutProcessed,
  kOutExactSizes,
  kOutEpoch,        // clustering-write epoch after the batch
  kOutT0,           // %globaltimer at the start and the end of the item
  kOutT1,
  kOutStatus,       // 0 ok
  kOutWords = 16
};

// One graph batch.  Graph state pointers are the mf_ctx arrays; scratch is
// carved by the host from the context's own buffers.  Sizes:
//   win[n] (epoch tags), map[n] (-1 between batches), hbits/sbits/xbits
//   [ceil(n/32)] (zero between batches): kept by the context;
//   k0/k1/ak [2m] u64, v0/v1/av [2m] u32, prev [2m], rows/rowcid [2m+n],
//   ends [2m+n+1], acnt [n], akill [a_total], kp [a_total+1]: per batch.
struct Item {
  int32_t n;
  int32_t sorted;
  const int64_t* nindex;
  const int32_t* nlist;
  uint32_t* live;
  int32_t* dead;
  int32_t* rcnt;
  int32_t* deg;
  const int64_t* aoff;
  const int32_t* aadj;
  const int32_t* aown;
  int64_t a_total;
  int64_t* aoff_new;
  int32_t* aadj_new;
  int32_t* aown_new;
  uint8_t* mis;
  int32_t* cid;
  const int32_t* u;
  const int32_t* v;
  const uint8_t* ins;
  int64_t m;
  int64_t max_csr;
  uint32_t epoch;
  uint32_t* win;
  int32_t* map;
  uint32_t* hbits;
  uint32_t* sbits;
  uint32_t* xbits;
  uint64_t* k0;
  uint32_t* v0;
  uint64_t* k1;
  uint32_t* v1;
  uint64_t* ak;
  uint32_t* av;
  int32_t* prev;
  int32_t* rows;
  int32_t* rowcid;
  int64_t* ends;
  int32_t* acnt;
  uint8_t* akill;
  int64_t* kp;
  int64_t* out;
};

// ---- graph view ----------------------------------------------------------------

struct View {
  int32_t n;
  const int64_t* nindex;
  const int32_t* nlist;
  const uint32_t* live;
  const int32_t* dead;
  const int64_t* aoff;
  const int32_t* aadj;
};

CTA_FN bool is_live(const uint32_t* live, int64_t k) { return (live[k >> 5] >> (k & 31)) & 1u; }

CTA_FN int64_t row_len(const View& g, int32_t x) {
  return (g.nindex[x + 1] - g.nindex[x]) - g.dead[x] + (g.aoff[x + 1] - g.aoff[x]);
}
CTA_FN int64_t row_positions(const View& g, int32_t x) {
  return (g.nindex[x + 1] - g.nindex[x]) + (g.aoff[x + 1] - g.aoff[x]);
}
// Element at row position k of x (base positions, then added), -1 if tombstoned.
CTA_FN int32_t row_at(const View& g, int32_t x, int64_t k) {
  const int64_t b = g.nindex[x], nb = g.nindex[x + 1] - b;
  if (k < nb) {
    if (g.dead[x] != 0 && !is_live(g.live, b + k)) return -1;
    return g.nlist[b + k];
  }
  return g.aadj[g.aoff[x] + (k - nb)];
}

// f(y) for y in row(x) in order (DeltaOverlay::neighbors_into); stops when f
// returns true and reports whether it did.
template <class F>
CTA_FN bool row_until(const View& g, int32_t x, F f) {
  const int64_t b = g.nindex[x], e = g.nindex[x + 1];
  if (g.dead[x] == 0) {
    for (int64_t k = b; k < e; ++k)
      if (f(g.nlist[k])) return true;
  } else {
    for (int64_t k = b; k < e; ++k)
      if (is_live(g.live, k) && f(g.nlist[k])) return true;
  }
  for (int64_t k = g.aoff[x]; k < g.aoff[x + 1]; ++k)
    if (f(g.aadj[k])) return true;
  return false;
}

// The packed row of a mapped vertex: for a seed its 2-hop list
// [s] ++ row(s) ++ rows of row(s) (get_h_hop_neighborhood, :159-202) with
// repeats left in -- first hits, "any member" and the set of written
// elements are the same with or without them -- and for a candidate its
// adjacency row (:550-558).
template <class F>
CTA_FN bool seq_until(const View& g, int32_t x, bool seed, F f) {
  if (!seed) return row_until(g, x, f);
  if (f(x)) return true;
  if (row_until(g, x, f)) return true;
  return row_until(g, x, [&](int32_t h) { return row_until(g, h, f); });
}

// ---- block primitives ------------------------------------------------------------

// Inclusive scan of one value per thread (Hillis-Steele over sh[0..nt)).
CTA_FN int64_t block_incl(int64_t v, int64_t* sh) {
  const int tid = CTA_TID, nt = CTA_NT;
  sh[tid] = v;
  CTA_SYNC();
  for (int d = 1; d < nt; d <<= 1) {
    const int64_t add = tid >= d ? sh[tid - d] : 0;
    CTA_SYNC();
    sh[tid] += add;
    CTA_SYNC();
  }
  const int64_t r = sh[tid];
  CTA_SYNC();
  return r;
}

// Exclusive scan over [0, n): each thread owns a contiguous chunk; calls
// put(i, prefix) in index order within the chunk (get(i) is read before
// put(i) is called, so in-place scans work).  Returns the total.
template <class Get, class Put>
CTA_FN int64_t scan(int64_t n, Get get, Put put, int64_t* sh) {
  const int tid = CTA_TID, nt = CTA_NT;
  const int64_t per = (n + nt - 1) / nt;
  int64_t lo = (int64_t)tid * per;
  if (lo > n) lo = n;
  const int64_t hi = lo + per < n ? lo + per : n;
  int64_t s = 0;
  for (int64_t i = lo; i < hi; ++i) s += get(i);
  const int64_t incl = block_incl(s, sh);
  // total: the last thread's inclusive value
  CTA_SHARED int64_t s_total;
  if (tid == nt - 1) s_total = incl;
  int64_t run = incl - s;
  for (int64_t i = lo; i < hi; ++i) {
    const int64_t x = get(i);
    put(i, run);
    run += x;
  }
  CTA_SYNC();
  const int64_t total = s_total;
  CTA_SYNC();
  return total;
}

// Sum of one value per thread.
CTA_FN int64_t block_sum(int64_t v, int64_t* sh) {
  const int64_t incl = block_incl(v, sh);
  CTA_SHARED int64_t s_sum;
  if (CTA_TID == CTA_NT - 1) s_sum = incl;
  CTA_SYNC();
  const int64_t r = s_sum;
  CTA_SYNC();
  return r;
}

// Stable sort of (k0, v0)[0, n) by key (keys below 2^bits); the result is in
// (k0, v0).  k1/v1 are the alternate buffers.  Up to kRankSortMax keys: rank
// by counting; above: LSD radix sort with 4-bit digits (per-thread
// contiguous chunks, so the scatter is stable).
CTA_FN void sort_pairs(uint64_t* k0, uint32_t* v0, uint64_t* k1, uint32_t* v1, int64_t n, int bits, int32_t* hist,
                       int64_t* sh) {
  const int tid = CTA_TID, nt = CTA_NT;
  if (n <= 1) return;
  if (n <= kRankSortMax) {
    for (int64_t i = tid; i < n; i += nt) {
      const uint64_t ki = k0[i];
      int64_t r = 0;
      for (int64_t j = 0; j < n; ++j) {
        const uint64_t kj = k0[j];
        r += (kj < ki || (kj == ki && j < i)) ? 1 : 0;
      }
      k1[r] = ki;
      v1[r] = v0[i];
    }
    CTA_SYNC();
    for (int64_t i = tid; i < n; i += nt) {
      k0[i] = k1[i];
      v0[i] = v1[i];
    }
    CTA_SYNC();
    return;
  }
  uint64_t* ka = k0;
  uint32_t* va = v0;
  uint64_t* kb = k1;
  uint32_t* vb = v1;
  const int passes = (bits + 3) / 4;
  const int64_t per = (n + nt - 1) / nt;
  int64_t lo = (int64_t)tid * per;
  if (lo > n) lo = n;
  const int64_t hi = lo + per < n ? lo + per : n;
  for (int pass = 0; pass < passes; ++pass) {
    const int shift = 4 * pass;
    int32_t c[kBuckets];
    for (int b = 0; b < kBuckets; ++b) c[b] = 0;
    for (int64_t i = lo; i < hi; ++i) ++c[(ka[i] >> shift) & (kBuckets - 1)];
    for (int b = 0; b < kBuckets; ++b) hist[b * nt + tid] = c[b];
    CTA_SYNC();
    scan(
        (int64_t)kBuckets * nt, [&](int64_t i) { return (int64_t)hist[i]; },
        [&](int64_t i, int64_t p) { hist[i] = (int32_t)p; }, sh);
    for (int b = 0; b < kBuckets; ++b) c[b] = hist[b * nt + tid];
    for (int64_t i = lo; i < hi; ++i) {
      const uint64_t k = ka[i];
      const int d = (int)((k >> shift) & (kBuckets - 1));
      const int32_t pos = c[d]++;
      kb[pos] = k;
      vb[pos] = va[i];
    }
    CTA_SYNC();
    uint64_t* tk = ka; ka = kb; kb = tk;
    uint32_t* tv = va; va = vb; vb = tv;
  }
  if (ka != k0) {
    for (int64_t i = tid; i < n; i += nt) {
      k0[i] = ka[i];
      v0[i] = va[i];
    }
    CTA_SYNC();
  }
}

CTA_FN int bits_for(int64_t v) {
  int b = 1;
  while (b < 63 && (v >> b) != 0) ++b;
  return b;
}

// ---- overlay apply (DeltaOverlay insert/remove in batch order) ---------------------

// Copies of y in the base row of x, split by live / tombstoned.
CTA_FN void base_copies(const View& g, bool sorted, int32_t x, int32_t y, int32_t* nlive, int32_t* ndead) {
  int32_t l = 0, d = 0;
  const int64_t b = g.nindex[x], e = g.nindex[x + 1];
  if (sorted) {
    int64_t lo = b, hi = e;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (g.nlist[mid] < y) lo = mid + 1; else hi = mid;
    }
    for (int64_t k = lo; k < e && g.nlist[k] == y; ++k) {
      if (is_live(g.live, k)) ++l; else ++d;
    }
  } else {
    for (int64_t k = b; k < e; ++k)
      if (g.nlist[k] == y) {
        if (is_live(g.live, k)) ++l; else ++d;
      }
  }
  *nlive = l;
  *ndead = d;
}

CTA_FN void base_mark(const View& g, uint32_t* live, bool sorted, int32_t x, int32_t y, bool on) {
  const int64_t b = g.nindex[x], e = g.nindex[x + 1];
  int64_t k = b;
  if (sorted) {
    int64_t lo = b, hi = e;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (g.nlist[mid] < y) lo = mid + 1; else hi = mid;
    }
    k = lo;
  }
  for (; k < e; ++k) {
    const int32_t z = g.nlist[k];
    if (sorted && z != y) break;
    if (z != y) continue;
    const uint32_t bit = 1u << (k & 31);
    if (on) at_or(live + (k >> 5), bit); else at_and(live + (k >> 5), ~bit);
  }
}

CTA_FN int64_t added_find(const View& g, int32_t x, int32_t y) {
  for (int64_t k = g.aoff[x]; k < g.aoff[x + 1]; ++k)
    if (g.aadj[k] == y) return k;
  return -1;
}

// Applies the batch; returns the view of the graph after it (the rebuilt
// added CSR when entries were appended or removed).
CTA_FN View apply_overlay(const Item& it, int32_t* hist, int64_t* sh) {
  const int tid = CTA_TID, nt = CTA_NT;
  const int64_t m = it.m;
  const int32_t n = it.n;
  const View g0{n, it.nindex, it.nlist, it.live, it.dead, it.aoff, it.aadj};
  const int nbits = bits_for(n - 1 > 1 ? n - 1 : 1);
  for (int64_t i = tid; i < m; i += nt) {
    const uint64_t a = (uint64_t)(it.u[i] < it.v[i] ? it.u[i] : it.v[i]);
    const uint64_t b = (uint64_t)(it.u[i] < it.v[i] ? it.v[i] : it.u[i]);
    it.k0[i] = (a << nbits) | b;
    it.v0[i] = (uint32_t)i;
  }
  for (int32_t x = tid; x < n; x += nt) it.acnt[x] = (int32_t)(it.aoff[x + 1] - it.aoff[x]);
  for (int64_t j = tid; j < it.a_total; j += nt) it.akill[j] = 0;
  CTA_SHARED unsigned long long s_app, s_kill;
  if (tid == 0) {
    s_app = 0;
    s_kill = 0;
  }
  CTA_SYNC();
  sort_pairs(it.k0, it.v0, it.k1, it.v1, m, 2 * nbits, hist, sh);

  // One thread per run of equal pair keys (the updates of one unordered pair
  // in batch order): the pair's state machine over its updates.
  enum : int { kN = 0, kA = 1, kR = 2 };  // absent, added entry, tombstoned base entry
  for (int64_t j0 = tid; j0 < m; j0 += nt) {
    if (j0 > 0 && it.k0[j0 - 1] == it.k0[j0]) continue;
    const uint64_t key = it.k0[j0];
    const int32_t a = (int32_t)(key >> nbits);
    const int32_t b = (int32_t)(key & ((1ull << nbits) - 1));
    const int64_t pos_ab = added_find(g0, a, b);
    const int64_t pos_ba = added_find(g0, b, a);
    int32_t live_ab, dead_ab, live_ba, dead_ba;
    base_copies(g0, it.sorted != 0, a, b, &live_ab, &dead_ab);
    base_copies(g0, it.sorted != 0, b, a, &live_ba, &dead_ba);
    const bool in_base_ab = live_ab + dead_ab > 0, in_base_ba = live_ba + dead_ba > 0;
    const int st0 = (pos_ab >= 0 || pos_ba >= 0) ? kA : ((dead_ab + dead_ba) > 0 ? kR : kN);
    int st = st0;
    bool appended = false, old_killed = false;
    uint32_t last_seq = 0;
    for (int64_t j = j0; j < m && it.k0[j] == key; ++j) {
      const uint32_t i = it.v0[j];
      const int32_t x = it.u[i];
      const bool base_xy = (x == a) ? in_base_ab : in_base_ba;
      const bool adj = st == kA || (st == kN && base_xy);
      if (it.ins[i] && !adj) {
        if (st == kR) {
          st = kN;
        } else {
          st = kA;
          appended = true;
          last_seq = i;
        }
      } else if (!it.ins[i] && adj) {
        if (st == kA) {
          st = kN;
          if (appended) appended = false; else old_killed = true;
        } else {
          st = kR;
        }
      }
    }
    if ((st0 == kR) != (st == kR)) {
      const bool on = st0 == kR;  // un-tombstone: live again
      base_mark(g0, it.live, it.sorted != 0, a, b, on);
      base_mark(g0, it.live, it.sorted != 0, b, a, on);
      const int32_t sgn = on ? -1 : 1;
      at_add(it.rcnt + a, sgn);
      at_add(it.rcnt + b, sgn);
      at_add(it.dead + a, sgn * (live_ab + dead_ab));
      at_add(it.dead + b, sgn * (live_ba + dead_ba));
    }
    if (old_killed) {
      if (pos_ab >= 0) {
        it.akill[pos_ab] = 1;
        at_add(it.acnt + a, -1);
      }
      if (pos_ba >= 0) {
        it.akill[pos_ba] = 1;
        at_add(it.acnt + b, -1);
      }
      at_add(&s_kill, 2ull);
    }
    if (appended) {
      const unsigned long long slot = at_add(&s_app, 2ull);
      it.ak[slot] = ((uint64_t)a << 32) | last_seq;
      it.av[slot] = (uint32_t)b;
      it.ak[slot + 1] = ((uint64_t)b << 32) | last_seq;
      it.av[slot + 1] = (uint32_t)a;
      at_add(it.acnt + a, 1);
      at_add(it.acnt + b, 1);
    }
  }
  CTA_SYNC();
  const int64_t appended = (int64_t)s_app, killed = (int64_t)s_kill;
  if (appended == 0 && killed == 0) {
    for (int32_t x = tid; x < n; x += nt)
      it.deg[x] = (int32_t)((it.nindex[x + 1] - it.nindex[x]) - it.rcnt[x] + (it.aoff[x + 1] - it.aoff[x]));
    if (tid == 0) {
      it.out[kOutATotal] = it.a_total;
      it.out[kOutSwapped] = 0;
    }
    CTA_SYNC();
    return View{n, it.nindex, it.nlist, it.live, it.dead, it.aoff, it.aadj};
  }
  // Rebuilt added CSR: survivors in their old order, then the appends of
  // each vertex in batch order.
  int64_t* noff = it.aoff_new;
  const int64_t total = scan(
      (int64_t)n, [&](int64_t x) { return (int64_t)it.acnt[x]; }, [&](int64_t x, int64_t p) { noff[x] = p; }, sh);
  if (tid == 0) noff[n] = total;
  if (it.a_total > 0) {
    const int64_t kt = scan(
        it.a_total, [&](int64_t j) { return (int64_t)it.akill[j]; }, [&](int64_t j, int64_t p) { it.kp[j] = p; },
        sh);
    if (tid == 0) it.kp[it.a_total] = kt;
    CTA_SYNC();
    for (int64_t j = tid; j < it.a_total; j += nt) {
      if (it.akill[j]) continue;
      const int32_t x = it.aown[j];
      const int64_t s = it.aoff[x];
      const int64_t r = (j - s) - (it.kp[j] - it.kp[s]);
      const int64_t pos = noff[x] + r;
      it.aadj_new[pos] = it.aadj[j];
      it.aown_new[pos] = x;
    }
  }
  if (appended > 0) {
    sort_pairs(it.ak, it.av, it.k1, it.v1, appended, 32 + nbits, hist, sh);
    for (int64_t k = tid; k < appended; k += nt) {
      const uint64_t owner = it.ak[k] >> 32;
      int64_t lo = 0, hi = k;
      while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if ((it.ak[mid] >> 32) < owner) lo = mid + 1; else hi = mid;
      }
      int64_t lo2 = k + 1, hi2 = appended;
      while (lo2 < hi2) {
        const int64_t mid = (lo2 + hi2) >> 1;
        if ((it.ak[mid] >> 32) <= owner) lo2 = mid + 1; else hi2 = mid;
      }
      const int32_t x = (int32_t)owner;
      const int64_t pos = noff[x + 1] - (lo2 - lo) + (k - lo);
      it.aadj_new[pos] = (int32_t)it.av[k];
      it.aown_new[pos] = x;
    }
  }
  CTA_SYNC();
  for (int32_t x = tid; x < n; x += nt)
    it.deg[x] = (int32_t)((it.nindex[x + 1] - it.nindex[x]) - it.rcnt[x] + (noff[x + 1] - noff[x]));
  if (tid == 0) {
    it.out[kOutATotal] = it.a_total + appended - killed;
    it.out[kOutSwapped] = 1;
  }
  CTA_SYNC();
  return View{n, it.nindex, it.nlist, it.live, it.dead, noff, it.aadj_new};
}

// ---- repair helpers ------------------------------------------------------------------

CTA_FN bool member(const uint8_t* mis, int32_t z) { return (mis[z] & 1) != 0; }

// any_member over the packed row of mapped row index i (one thread).
CTA_FN bool any_member_seq(const View& g, const Item& it, int32_t i, int64_t n_seeds, int32_t except) {
  return seq_until(g, it.rows[i], i < n_seeds, [&](int32_t z) { return z != except && member(it.mis, z); });
}

// Insertion rule candidate test: w not a member, mapped, and no member in
// its row.  `removed` is the endpoint the rule has just taken out of the set:
// it counts as a non-member (its membership byte is cleared at the commit).
CTA_FN bool eligible(const View& g, const Item& it, int32_t w, int64_t n_seeds, int32_t removed) {
  if (w != removed && member(it.mis, w)) return false;
  const int32_t i = it.map[w];
  if (i < 0) return false;
  return !any_member_seq(g, it, i, n_seeds, removed);
}

constexpr unsigned long long kNone = ~0ull;

// First w (in packed-row order of vertex x = rows[ri]) that is eligible;
// -1 if none.  Block-cooperative; the result is uniform.  b1 and b2 are
// shared result slots holding kNone on entry (the caller resets them).
// Ends with a barrier after which the slots are only read.
CTA_FN int32_t block_first_eligible(const View& g, const Item& it, int32_t ri, int64_t n_seeds, int32_t removed,
                                    unsigned long long* b1, unsigned long long* b2) {
  const int tid = CTA_TID, nt = CTA_NT;
  const int32_t x = it.rows[ri];
  const bool seed = ri < n_seeds;
  // x itself (seeds) and row(x): position 0 is x, position 1 + k is row position k.
  const int64_t np = row_positions(g, x);
  for (int64_t p = (seed ? 0 : 1) + tid; p < 1 + np; p += nt) {
    if ((unsigned long long)p > *b1) break;
    const int32_t w = p == 0 ? x : row_at(g, x, p - 1);
    if (w >= 0 && eligible(g, it, w, n_seeds, removed)) at_min(b1, (unsigned long long)p);
  }
  CTA_SYNC();
  const unsigned long long best = *b1;
  if (best != kNone) {
    const int64_t p = (int64_t)best;
    return p == 0 ? x : row_at(g, x, p - 1);
  }
  if (!seed) return -1;
  // rows of the row's elements: thread per element h (in row order), its
  // row scanned in order; the first (h position, inner position) wins.
  // Chunks share b2, so each takes two barriers: every thread reads b2
  // before the next chunk may write it.
  for (int64_t h0 = 0; h0 < np; h0 += nt) {
    const int64_t hp = h0 + tid;
    if (hp < np) {
      const int32_t h = row_at(g, x, hp);
      if (h >= 0) {
        const int64_t nq = row_positions(g, h);
        for (int64_t q = 0; q < nq; ++q) {
          const unsigned long long key = ((unsigned long long)hp << 32) | (unsigned long long)q;
          if (key > *b2) break;
          const int32_t w = row_at(g, h, q);
          if (w >= 0 && eligible(g, it, w, n_seeds, removed)) {
            at_min(b2, key);
            break;
          }
        }
      }
    }
    CTA_SYNC();
    const unsigned long long best2 = *b2;
    CTA_SYNC();
    if (best2 != kNone) {
      const int32_t h = row_at(g, x, (int64_t)(best2 >> 32));
      return row_at(g, h, (int64_t)(best2 & 0xffffffffull));
    }
  }
  return -1;
}

// Any member other than `except` in the packed row of rows[ri].
// Block-cooperative; fd is a shared flag holding 0 on entry (the caller
// resets it).  Ends with a barrier after which the flag is only read.
CTA_FN bool block_any_member(const View& g, const Item& it, int32_t ri, int64_t n_seeds, int32_t except, int* fd) {
  const int tid = CTA_TID, nt = CTA_NT;
  const int32_t x = it.rows[ri];
  const bool seed = ri < n_seeds;
  if (tid == 0 && seed && x != except && member(it.mis, x)) *fd = 1;
  const int64_t np = row_positions(g, x);
  for (int64_t p = tid; p < np; p += nt) {
    if (*fd) break;
    const int32_t z = row_at(g, x, p);
    if (z < 0) continue;
    bool f = z != except && member(it.mis, z);
    if (!f && seed) f = row_until(g, z, [&](int32_t w) { return w != except && member(it.mis, w); });
    if (f) *fd = 1;
  }
  CTA_SYNC();
  return *fd != 0;
}

// ---- the whole batch -------------------------------------------------------------------

CTA_FN void run_item(const Item& it, int32_t* hist, int64_t* sh) {
  const int tid = CTA_TID, nt = CTA_NT;
  const int64_t m = it.m;
  const int32_t n = it.n;
  if (tid == 0) it.out[kOutT0] = (int64_t)now_ns();

  const View g = apply_overlay(it, hist, sh);

  // Previous occurrence of each endpoint slot (slot 2t = u[t], 2t+1 = v[t]).
  const int nbits = bits_for(n - 1 > 1 ? n - 1 : 1);
  const int64_t ns = 2 * m;
  for (int64_t j = tid; j < ns; j += nt) {
    const int32_t x = (j & 1) ? it.v[j >> 1] : it.u[j >> 1];
    it.k0[j] = ((uint64_t)x << 32) | (uint64_t)j;
    it.v0[j] = (uint32_t)j;
  }
  CTA_SYNC();
  sort_pairs(it.k0, it.v0, it.k1, it.v1, ns, 32 + nbits, hist, sh);
  for (int64_t i = tid; i < ns; i += nt) {
    const bool same = i > 0 && (it.k0[i - 1] >> 32) == (it.k0[i] >> 32);
    it.prev[it.v0[i]] = same ? (int32_t)(it.k0[i - 1] & 0xffffffffull) : -1;
  }
  CTA_SYNC();

  CTA_SHARED int64_t s_est;
  CTA_SHARED unsigned long long s_cut, s_cnt;
  CTA_SHARED int64_t s_max_csr;
  CTA_SHARED unsigned long long s_win[2], s_b1[2], s_b2[2];
  CTA_SHARED int s_fd[2];
  if (tid == 0) s_max_csr = it.max_csr;
  CTA_SYNC();
  int64_t n_sub = 0, n_seeds_total = 0, n_cands_total = 0, n_clusters = 0, n_processed = 0, n_exact = 0;
  uint32_t epoch = it.epoch;
  int64_t p = 0;
  while (p < m) {
    const int64_t max_csr = s_max_csr;
    // ---- split rule (:490-521): edge q joins while est + add < MAX_CSR_ELEMENTS
    if (tid == 0) {
      s_est = 0;
      s_cut = ~0ull;
    }
    CTA_SYNC();
    const int64_t qmax = (m - p) < kMaxBatchEdges ? m : p + kMaxBatchEdges;
    int64_t q = qmax;
    for (int64_t w0 = p; w0 < qmax; w0 += nt) {
      const int64_t e = w0 + tid;
      int64_t add = 0;
      if (e < qmax) {
        if (it.prev[2 * e] < 2 * p) add += (int64_t)it.deg[it.u[e]] * kEstimateWeight;
        if (it.prev[2 * e + 1] < 2 * p) add += (int64_t)it.deg[it.v[e]] * kEstimateWeight;
      }
      const int64_t incl = block_incl(add, sh);
      const int64_t est0 = s_est;
      if (e < qmax && e > p && est0 + incl >= max_csr) at_min(&s_cut, (unsigned long long)e);
      CTA_SYNC();
      if (s_cut != ~0ull) {
        q = (int64_t)s_cut;
        break;
      }
      if (tid == nt - 1) s_est = est0 + incl;
      CTA_SYNC();
    }
    CTA_SYNC();

    // ---- seeds: endpoints not seen earlier in the sub-batch, slot order
    const int64_t S = scan(
        2 * (q - p), [&](int64_t j) { return (int64_t)(it.prev[2 * p + j] < 2 * p ? 1 : 0); },
        [&](int64_t j, int64_t pos) {
          if (it.prev[2 * p + j] < 2 * p) {
            const int64_t sl = 2 * p + j;
            it.rows[pos] = (sl & 1) ? it.v[sl >> 1] : it.u[sl >> 1];
          }
        },
        sh);
    for (int64_t i = tid; i < S; i += nt) {
      const int32_t s = it.rows[i];
      it.map[s] = (int32_t)i;
      at_or(it.sbits + (s >> 5), 1u << (s & 31));
    }
    CTA_SYNC();
    // ---- hop-1 set and candidate rows (hop-1 vertices that are not seeds, ascending id)
    for (int64_t i = tid; i < S; i += nt)
      row_until(g, it.rows[i], [&](int32_t y) {
        at_or(it.hbits + (y >> 5), 1u << (y & 31));
        return false;
      });
    CTA_SYNC();
    const int64_t W = ((int64_t)n + 31) >> 5;
    const int64_t cap_c = S >= kMaxRows ? 0 : kMaxRows - S;
    const int64_t c_all = scan(
        W, [&](int64_t w) { return (int64_t)popc32(it.hbits[w] & ~it.sbits[w]); },
        [&](int64_t w, int64_t pos) {
          uint32_t bitsw = it.hbits[w] & ~it.sbits[w];
          while (bitsw) {
            const int b = ffs32(bitsw) - 1;
            bitsw &= bitsw - 1;
            if (pos < cap_c) {
              const int32_t c = (int32_t)(w * 32 + b);
              it.rows[S + pos] = c;
              it.map[c] = (int32_t)(S + pos);
            }
            ++pos;
          }
        },
        sh);
    const int64_t C = c_all < cap_c ? c_all : cap_c;
    const int64_t R = S + C;

    // ---- packed sizes and MAX_CSR_ELEMENTS growth (:560-599)
    int64_t loose_part = 0;
    for (int64_t i = tid; i < R; i += nt) {
      const int32_t x = it.rows[i];
      int64_t len = row_len(g, x);
      if (i < S) {
        int64_t acc = 1 + len;
        row_until(g, x, [&](int32_t h) {
          acc += row_len(g, h);
          return false;
        });
        len = acc;
      }
      it.ends[i] = len;
      loose_part += len;
    }
    const int64_t loose = block_sum(loose_part, sh);
    if (loose >= max_csr) {
      // exact 2-hop sizes of the seeds: one seed at a time, its elements
      // marked in a vertex bitmap and the new marks counted
      for (int64_t i = 0; i < S; ++i) {
        const int32_t x = it.rows[i];
        if (tid == 0) s_cnt = 0;
        CTA_SYNC();
        unsigned long long mine = 0;
        auto mark = [&](int32_t y) {
          const uint32_t bit = 1u << (y & 31);
          if (!(at_or(it.xbits + (y >> 5), bit) & bit)) ++mine;
        };
        if (tid == 0) mark(x);
        const int64_t np = row_positions(g, x);
        for (int64_t k = tid; k < np; k += nt) {
          const int32_t y = row_at(g, x, k);
          if (y < 0) continue;
          mark(y);
          row_until(g, y, [&](int32_t z) {
            mark(z);
            return false;
          });
        }
        at_add(&s_cnt, mine);
        CTA_SYNC();
        if (tid == 0) it.ends[i] = (int64_t)s_cnt;
        if (tid == 0) it.xbits[x >> 5] = 0;
        for (int64_t k = tid; k < np; k += nt) {
          const int32_t y = row_at(g, x, k);
          if (y < 0) continue;
          it.xbits[y >> 5] = 0;
          row_until(g, y, [&](int32_t z) {
            it.xbits[z >> 5] = 0;
            return false;
          });
        }
        CTA_SYNC();
      }
      // row end offsets in packing order, then the growth replay: each time a
      // row's end reaches the limit, the limit becomes 1.5x that end
      scan(
          R, [&](int64_t i) { return it.ends[i]; }, [&](int64_t i, int64_t pos) { it.ends[i] = pos + it.ends[i]; },
          sh);
      if (tid == 0) {
        int64_t lim = max_csr;
        int64_t from = 0;
        for (;;) {
          int64_t lo = from, hi = R;  // first row with end >= lim
          while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (it.ends[mid] < lim) lo = mid + 1; else hi = mid;
          }
          if (lo >= R) break;
          lim = (int64_t)((double)(uint64_t)it.ends[lo] * 1.5);
          from = lo + 1;
        }
        s_max_csr = lim;
      }
      ++n_exact;
      CTA_SYNC();
    }

    // ---- clustering read (:219-252): first existing id in row order,
    // against the ids as they were before the kernel
    for (int64_t i = tid; i < R; i += nt) {
      const int32_t x = it.rows[i];
      if (it.cid[x] != -1) {
        it.rowcid[i] = -2;
        continue;
      }
      int32_t found = -1;
      seq_until(g, x, i < S, [&](int32_t y) {
        const int32_t c = it.cid[y];
        if (c != -1) {
          found = c;
          return true;
        }
        return false;
      });
      it.rowcid[i] = found;
    }
    CTA_SYNC();
    // new ids by ascending row index
    const int64_t clusters = scan(
        R, [&](int64_t i) { return (int64_t)(it.rowcid[i] == -1 ? 1 : 0); },
        [&](int64_t i, int64_t pos) {
          if (it.rowcid[i] == -1) it.rowcid[i] = (int32_t)pos;
        },
        sh);
    // ---- clustering write (:253-258): the highest row index writes last
    ++epoch;
    if (epoch > kMaxEpoch) {
      for (int32_t x = tid; x < n; x += nt) it.win[x] = 0;
      CTA_SYNC();
      epoch = 1;
    }
    for (int64_t i = tid; i < R; i += nt) {
      if (it.rowcid[i] < 0) continue;
      const uint32_t tag = (epoch << kTagBits) | (uint32_t)i;
      seq_until(g, it.rows[i], i < S, [&](int32_t y) {
        at_max(it.win + y, tag);
        return false;
      });
    }
    CTA_SYNC();
    // every element tagged in this epoch takes its winner's id: a sweep of
    // the tag array when that is shorter than the rows (loose is their
    // length), else a second walk of the rows
    if ((int64_t)n <= loose) {
      for (int32_t y = tid; y < n; y += nt) {
        const uint32_t w = it.win[y];
        if ((w >> kTagBits) == epoch) it.cid[y] = it.rowcid[w & kTagMask];
      }
    } else {
      for (int64_t i = tid; i < R; i += nt) {
        if (it.rowcid[i] < 0) continue;
        seq_until(g, it.rows[i], i < S, [&](int32_t y) {
          it.cid[y] = it.rowcid[it.win[y] & kTagMask];
          return false;
        });
      }
    }
    CTA_SYNC();

    // ---- assignment (:261-275): cid(src) if set, else cid(dst); lists in
    // ascending cluster id, each in descending edge index
    const int64_t limit = clusters < kMaxBatchEdges ? clusters : kMaxBatchEdges;
    if (tid == 0) s_cnt = 0;
    CTA_SYNC();
    for (int64_t t = p + tid; t < q; t += nt) {
      int32_t c = it.cid[it.u[t]];
      if (c == -1) c = it.cid[it.v[t]];
      if (c < 0 || (int64_t)c >= limit) continue;
      const unsigned long long slot = at_add(&s_cnt, 1ull);
      it.k0[slot] = ((uint64_t)c << 32) | (uint64_t)(0xffffffffu - (uint32_t)(t - p));
      it.v0[slot] = (uint32_t)t;
    }
    CTA_SYNC();
    const int64_t P = (int64_t)s_cnt;
    CTA_SYNC();
    sort_pairs(it.k0, it.v0, it.k1, it.v1, P, 32 + bits_for(limit > 0 ? limit : 1), hist, sh);

    // ---- repair (:277-349): the edges in that order, one after another.
    // Edges that change nothing are skipped a window at a time: every
    // thread tests one edge against the membership, and the first edge
    // that acts is applied.  Three barriers per applied edge -- the
    // window's, the evaluation's, the commit's.  The shared slots are
    // double-buffered so that no slot is reset while another thread may
    // still read it: windows alternate between two first-hit slots (an
    // unused one stays kNone; the one that hit is reset after the commit
    // barrier), and applied edges alternate between two sets of result
    // slots (the set of the next edge is reset before the commit barrier).
    if (tid == 0) {
      s_win[0] = s_win[1] = kNone;
      s_b1[0] = s_b1[1] = s_b2[0] = s_b2[1] = kNone;
      s_fd[0] = s_fd[1] = 0;
    }
    CTA_SYNC();
    int64_t k = 0;
    int wp = 0, ap = 0;
    for (;;) {
      unsigned long long f = kNone;
      int hb = 0;
      for (int64_t w0 = k; w0 < P; w0 += nt) {
        const int64_t e = w0 + tid;
        if (e < P) {
          const uint32_t t = it.v0[e];
          const bool ma = member(it.mis, it.u[t]), mb = member(it.mis, it.v[t]);
          const bool act = it.ins[t] ? (ma && mb) : (ma != mb);
          if (act) at_min(&s_win[wp], (unsigned long long)e);
        }
        CTA_SYNC();
        f = s_win[wp];
        hb = wp;
        wp ^= 1;
        if (f != kNone) break;
      }
      if (f == kNone) break;
      // every thread derives the rule of edge f from the same membership
      const uint32_t t = it.v0[f];
      const int32_t a = it.u[t], b = it.v[t];
      int32_t r = -1, w = -1, y = -1;
      bool any = true, evaluated = false;
      if (it.ins[t]) {
        r = a > b ? a : b;
        const int32_t ri = it.map[r];
        if (ri >= 0) {
          w = block_first_eligible(g, it, ri, S, r, &s_b1[ap], &s_b2[ap]);
          evaluated = true;
        }
      } else {
        const bool ma = member(it.mis, a);
        y = ma ? b : a;
        const int32_t keep = ma ? a : b;
        const int32_t ri = it.map[y];
        if (ri >= 0) {
          any = block_any_member(g, it, ri, S, keep, &s_fd[ap]);
          evaluated = true;
        } else {
          any = false;
        }
      }
      // the evaluations end with a barrier; without one, this barrier makes
      // every thread derive the rule before the commit changes the membership
      if (!evaluated) CTA_SYNC();
      if (tid == 0) {
        if (r >= 0) {
          it.mis[r] = 0;
          if (w >= 0) it.mis[w] = 1;
        } else if (!any) {
          it.mis[y] = 1;
        }
        s_b1[ap ^ 1] = kNone;
        s_b2[ap ^ 1] = kNone;
        s_fd[ap ^ 1] = 0;
      }
      ap ^= 1;
      CTA_SYNC();
      if (tid == 0) s_win[hb] = kNone;
      k = (int64_t)f + 1;
    }
    CTA_SYNC();

    // ---- clear (:351-358): mapped vertices only; marks for the next sub-batch
    for (int64_t i = tid; i < R; i += nt) {
      const int32_t x = it.rows[i];
      it.cid[x] = -1;
      it.map[x] = -1;
    }
    for (int64_t i = tid; i < S; i += nt) {
      const int32_t x = it.rows[i];
      it.sbits[x >> 5] = 0;
      row_until(g, x, [&](int32_t y) {
        it.hbits[y >> 5] = 0;
        return false;
      });
    }
    CTA_SYNC();
    ++n_sub;
    n_seeds_total += S;
    n_cands_total += C;
    n_clusters += clusters;
    n_processed += P;
    p = q;
  }
  if (tid == 0) {
    it.out[kOutMaxCsr] = s_max_csr;
    it.out[kOutSubBatches] = n_sub;
    it.out[kOutSeeds] = n_seeds_total;
    it.out[kOutCands] = n_cands_total;
    it.out[kOutClusters] = n_clusters;
    it.out[kOutProcessed] = n_processed;
    it.out[kOutExactSizes] = n_exact;
    it.out[kOutEpoch] = epoch;
    it.out[kOutStatus] = 0;
    it.out[kOutT1] = (int64_t)now_ns();
  }
  CTA_SYNC();
}

}  // namespace cta
}  // namespace mf
