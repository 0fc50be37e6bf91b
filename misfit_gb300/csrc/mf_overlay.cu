// mf_overlay.cu -- device-resident base CSR + delta overlay.
//
// The reference keeps the overlay as hash maps of vectors and sets on the
// host (core/FlashGraph.h:172-276).  Here:
//   * a tombstone of (x, y) clears the live bits of every copy of y in the
//     base row of x (and of x in the row of y) and counts into rcnt[x],
//     rcnt[y] -- the size of removed_adj[x] that DeltaOverlay::degree uses;
//   * added neighbours live in a CSR (aoff/aadj) that keeps each vertex's
//     entries in insertion order; it is rebuilt after every batch from the
//     surviving entries followed by the new ones in batch order.
// A batch is applied in parallel by grouping its updates per unordered pair:
// different pairs touch disjoint overlay entries, so only the updates of one
// pair have to run in batch order (one thread walks them through the
// three-state machine none / added / tombstoned that insertEdge, removeEdge,
// un_tombstone and forget_delta_edge implement, core/FlashGraph.h:196-275).
#include <algorithm>
#include <mutex>

#include "mf_internal.cuh"

namespace mf {

namespace {

constexpr int kTB = 256;

inline unsigned grid_for(int64_t n, int per = kTB) {
  int64_t g = (n + per - 1) / per;
  if (g < 1) g = 1;
  if (g > (1 << 30)) g = 1 << 30;
  return (unsigned)g;
}

__global__ void k_base_degree(const int64_t* nindex, int32_t n, int32_t* deg) {
  int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x < n) deg[x] = (int32_t)(nindex[x + 1] - nindex[x]);
}

// Rows non-decreasing?  (Sorted rows allow binary search for a neighbour.)
// Load-balanced over all entries: each entry compares with its predecessor
// in the same row.  flags[0] cleared on a descent.
__global__ void k_check_sorted(GraphView g, const int32_t* list, const int64_t* offs, int32_t n, int* ok) {
  lb_rows_pos(g, list, offs, n, 0, [&](int64_t, int32_t x, int32_t y, int64_t j) {
    if (j > 0 && g.nlist[g.nindex[x] + j - 1] > y) atomicAnd(ok, 0);
  });
}

// Every entry x -> y has its reverse y -> x (rows sorted: binary search).
__global__ void k_check_symmetric(GraphView g, const int32_t* list, const int64_t* offs, int32_t n, int* ok) {
  lb_rows(g, list, offs, n, [&](int64_t, int32_t x, int32_t y) {
    int64_t lo = g.nindex[y], hi = g.nindex[y + 1];
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (g.nlist[mid] < x) lo = mid + 1; else hi = mid;
    }
    if (lo >= g.nindex[y + 1] || g.nlist[lo] != x) atomicAnd(ok, 0);
  });
}

__global__ void k_iota_n(int32_t* out, int32_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (int32_t)i;
}

__global__ void k_base_positions(const int64_t* nindex, int32_t n, int64_t* out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = nindex[i + 1] - nindex[i];
}

__global__ void k_check_ids(const int32_t* nlist, int64_t nnz, int32_t n, int* ok) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int32_t y = nlist[k];
    if (y < 0 || y >= n) { atomicAnd(ok, 0); return; }
  }
}

__global__ void k_check_index(const int64_t* nindex, int32_t n, int64_t nnz, int* ok) {
  int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x > n) return;
  const int64_t a = nindex[x];
  if (a < 0 || a > nnz || (x < n && nindex[x + 1] < a) || (x == 0 && a != 0)) atomicAnd(ok, 0);
}

// Copies of y in the base row of x, split by live/tombstoned.
__device__ void base_copies(const GraphView& g, bool sorted, int32_t x, int32_t y, int32_t* nlive, int32_t* ndead) {
  int32_t l = 0, d = 0;
  int64_t b = g.nindex[x], e = g.nindex[x + 1];
  if (sorted) {
    int64_t lo = b, hi = e;
    while (lo < hi) {
      int64_t mid = (lo + hi) >> 1;
      if (g.nlist[mid] < y) lo = mid + 1; else hi = mid;
    }
    for (int64_t k = lo; k < e && g.nlist[k] == y; ++k) {
      if (live_at(g.live, k)) ++l; else ++d;
    }
  } else {
    for (int64_t k = b; k < e; ++k)
      if (g.nlist[k] == y) { if (live_at(g.live, k)) ++l; else ++d; }
  }
  *nlive = l;
  *ndead = d;
}

__device__ void base_mark(const GraphView& g, uint32_t* live, bool sorted, int32_t x, int32_t y, bool on) {
  int64_t b = g.nindex[x], e = g.nindex[x + 1];
  int64_t k = b;
  if (sorted) {
    int64_t lo = b, hi = e;
    while (lo < hi) {
      int64_t mid = (lo + hi) >> 1;
      if (g.nlist[mid] < y) lo = mid + 1; else hi = mid;
    }
    k = lo;
  }
  for (; k < e; ++k) {
    const int32_t z = g.nlist[k];
    if (sorted && z != y) break;
    if (z != y) continue;
    const uint32_t bit = 1u << (k & 31);
    if (on) atomicOr(live + (k >> 5), bit); else atomicAnd(live + (k >> 5), ~bit);
  }
}

__device__ int64_t added_find(const GraphView& g, int32_t x, int32_t y) {
  for (int64_t k = g.aoff[x]; k < g.aoff[x + 1]; ++k)
    if (g.aadj[k] == y) return k;
  return -1;
}

__global__ void k_pair_keys(const int32_t* u, const int32_t* v, int64_t m, int nbits, uint64_t* keys, uint32_t* vals) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const uint64_t a = (uint64_t)min(u[i], v[i]), b = (uint64_t)max(u[i], v[i]);
  keys[i] = (a << nbits) | b;
  vals[i] = (uint32_t)i;
}

__global__ void k_init_acnt(const int64_t* aoff, int32_t n, int32_t* acnt) {
  int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x < n) acnt[x] = (int32_t)(aoff[x + 1] - aoff[x]);
}

enum : int { kStN = 0, kStA = 1, kStR = 2 };

// One thread per run of equal pair keys (the updates of one unordered pair
// in batch order).  counters[0] = appended entries, counters[1] = killed.
__global__ void k_apply_pairs(GraphView g, uint32_t* live, int32_t* dead, int32_t* rcnt, bool sorted,
                              const uint64_t* keys, const uint32_t* vals, int64_t m, int nbits,
                              const int32_t* u, const int32_t* v, const uint8_t* ins,
                              int32_t* acnt, uint8_t* akill, uint64_t* app_keys, uint32_t* app_vals,
                              int64_t* counters) {
  int64_t j0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j0 >= m) return;
  if (j0 > 0 && keys[j0 - 1] == keys[j0]) return;  // not the head of a run
  const uint64_t key = keys[j0];
  const int32_t a = (int32_t)(key >> nbits);
  const int32_t b = (int32_t)(key & ((1ull << nbits) - 1));
  const int64_t pos_ab = added_find(g, a, b);
  const int64_t pos_ba = added_find(g, b, a);
  int32_t live_ab, dead_ab, live_ba, dead_ba;
  base_copies(g, sorted, a, b, &live_ab, &dead_ab);
  base_copies(g, sorted, b, a, &live_ba, &dead_ba);
  const bool in_base_ab = live_ab + dead_ab > 0, in_base_ba = live_ba + dead_ba > 0;
  const int st0 = (pos_ab >= 0 || pos_ba >= 0) ? kStA : ((dead_ab + dead_ba) > 0 ? kStR : kStN);
  int st = st0;
  bool appended = false, old_killed = false;
  uint32_t last_seq = 0;
  for (int64_t j = j0; j < m && keys[j] == key; ++j) {
    const uint32_t i = vals[j];
    const int32_t x = u[i];
    const bool base_xy = (x == a) ? in_base_ab : in_base_ba;
    const bool adj = st == kStA || (st == kStN && base_xy);
    if (ins[i] && !adj) {
      if (st == kStR) st = kStN;
      else { st = kStA; appended = true; last_seq = i; }
    } else if (!ins[i] && adj) {
      if (st == kStA) {
        st = kStN;
        if (appended) appended = false; else old_killed = true;
      } else {
        st = kStR;
      }
    }
  }
  // tombstone changes
  if ((st0 == kStR) != (st == kStR)) {
    const bool on = st0 == kStR;  // untombstone -> set live again
    base_mark(g, live, sorted, a, b, on);
    base_mark(g, live, sorted, b, a, on);
    const int32_t sgn = on ? -1 : 1;
    atomicAdd(rcnt + a, sgn);
    atomicAdd(rcnt + b, sgn);
    atomicAdd(dead + a, sgn * (live_ab + dead_ab));
    atomicAdd(dead + b, sgn * (live_ba + dead_ba));
  }
  if (old_killed) {
    if (pos_ab >= 0) { akill[pos_ab] = 1; atomicSub(acnt + a, 1); }
    if (pos_ba >= 0) { akill[pos_ba] = 1; atomicSub(acnt + b, 1); }
    atomicAdd((unsigned long long*)(counters + 1), 2ull);
  }
  if (appended) {
    const unsigned long long slot = atomicAdd((unsigned long long*)counters, 2ull);
    app_keys[slot] = ((uint64_t)a << 32) | last_seq;
    app_vals[slot] = (uint32_t)b;
    app_keys[slot + 1] = ((uint64_t)b << 32) | last_seq;
    app_vals[slot + 1] = (uint32_t)a;
    atomicAdd(acnt + a, 1);
    atomicAdd(acnt + b, 1);
  }
}

__global__ void k_move_survivors(const int64_t* aoff, const int32_t* aadj, const int32_t* aown,
                                 const uint8_t* akill, const int64_t* kp, int64_t a_total,
                                 const int64_t* noff, int32_t* nadj, int32_t* nown) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a_total || akill[j]) return;
  const int32_t x = aown[j];
  const int64_t s = aoff[x];
  const int64_t r = (j - s) - (kp[j] - kp[s]);
  const int64_t pos = noff[x] + r;
  nadj[pos] = aadj[j];
  nown[pos] = x;
}

__global__ void k_place_appends(const uint64_t* keys, const uint32_t* vals, int64_t cnt,
                                const int64_t* noff, int32_t* nadj, int32_t* nown) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= cnt) return;
  const uint64_t owner = keys[k] >> 32;
  int64_t lo = 0, hi = k;  // first index with this owner
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if ((keys[mid] >> 32) < owner) lo = mid + 1; else hi = mid;
  }
  int64_t lo2 = k + 1, hi2 = cnt;  // one past the last index with this owner
  while (lo2 < hi2) {
    int64_t mid = (lo2 + hi2) >> 1;
    if ((keys[mid] >> 32) <= owner) lo2 = mid + 1; else hi2 = mid;
  }
  const int32_t x = (int32_t)owner;
  const int64_t pos = noff[x + 1] - (lo2 - lo) + (k - lo);
  nadj[pos] = (int32_t)vals[k];
  nown[pos] = x;
}

__global__ void k_degrees(const int64_t* nindex, const int32_t* rcnt, const int64_t* aoff, int32_t n, int32_t* deg) {
  int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x < n) deg[x] = (int32_t)((nindex[x + 1] - nindex[x]) - rcnt[x] + (aoff[x + 1] - aoff[x]));
}

// isAdjacent (core/FlashGraph.h:291-301) for every update.
__global__ void k_flags(GraphView g, bool sorted, const int32_t* u, const int32_t* v, int64_t m, uint8_t* ins) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const int32_t x = u[i], y = v[i];
  bool adj = added_find(g, x, y) >= 0;
  if (!adj) {
    int32_t l, d;
    base_copies(g, sorted, x, y, &l, &d);
    adj = l > 0;
  }
  ins[i] = adj ? 0 : 1;
}

// k_flags with the endpoint check folded in, for flag_updates_noalloc: a pair
// with an endpoint outside [0, n) or u == v is counted into *bad and gets no
// flag (the host then reports the batch as invalid and copies nothing out).
__global__ void k_flags_checked(GraphView g, bool sorted, const int32_t* u, const int32_t* v, int64_t m,
                                uint8_t* ins, unsigned long long* bad) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const int32_t x = u[i], y = v[i];
  if (x < 0 || x >= g.n || y < 0 || y >= g.n || x == y) {
    atomicAdd(bad, 1ull);
    return;
  }
  bool adj = added_find(g, x, y) >= 0;
  if (!adj) {
    int32_t l, d;
    base_copies(g, sorted, x, y, &l, &d);
    adj = l > 0;
  }
  ins[i] = adj ? 0 : 1;
}

// ---- compaction --------------------------------------------------------------

__global__ void k_compact_check(GraphView g, const int32_t* deg, int64_t* counters) {
  int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= g.n) return;
  const int32_t d = deg[x];
  if (d < 0) atomicAdd((unsigned long long*)(counters + 0), 1ull);
  else if ((int64_t)d != row_len(g, x)) atomicAdd((unsigned long long*)(counters + 1), 1ull);
}

__global__ void k_compact_gather(GraphView g, const int64_t* noff, int32_t* out) {
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= g.n) return;
  const int32_t x = (int32_t)warp;
  int64_t o = noff[x];
  const int64_t b = g.nindex[x], e = g.nindex[x + 1];
  const bool filt = g.dead[x] != 0;
  for (int64_t k0 = b; k0 < e; k0 += 32) {
    const int64_t k = k0 + lane;
    const bool ok = k < e && (!filt || live_at(g.live, k));
    const unsigned msk = __ballot_sync(0xffffffffu, ok);
    if (ok) out[o + __popc(msk & ((1u << lane) - 1u))] = g.nlist[k];
    o += __popc(msk);
  }
  for (int64_t k0 = g.aoff[x]; k0 < g.aoff[x + 1]; k0 += 32) {
    const int64_t k = k0 + lane;
    if (k < g.aoff[x + 1]) out[o + lane] = g.aadj[k];
    o += min((int64_t)32, g.aoff[x + 1] - k0);
  }
}

// ---- greedy MIS in vertex order ------------------------------------------------
// x joins iff no lower-id neighbour joined; decided in rounds, each vertex
// settling once all its lower-id neighbours have settled.
__global__ void k_greedy_round(GraphView g, bool sorted, uint8_t* st, int64_t* counters) {
  int64_t xi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (xi >= g.n) return;
  const int32_t x = (int32_t)xi;
  if (st[x] != 0) return;
  bool pending = false, blocked = false;
  const int64_t b = g.nindex[x], e = g.nindex[x + 1];
  const bool filt = g.dead[x] != 0;
  for (int64_t k = b; k < e && !blocked; ++k) {
    const int32_t y = g.nlist[k];
    if (sorted && y >= x) break;
    if (y >= x || (filt && !live_at(g.live, k))) continue;
    const uint8_t s = st[y];
    if (s == 1) blocked = true; else if (s == 0) pending = true;
  }
  for (int64_t k = g.aoff[x]; k < g.aoff[x + 1] && !blocked; ++k) {
    const int32_t y = g.aadj[k];
    if (y >= x) continue;
    const uint8_t s = st[y];
    if (s == 1) blocked = true; else if (s == 0) pending = true;
  }
  if (blocked) st[x] = 2;
  else if (!pending) st[x] = 1;
  else atomicAdd((unsigned long long*)counters, 1ull);
}

// ---- exact-MIS mode (no reference counterpart) -----------------------------------
// After a batch's repair: a member with a smaller-id member neighbour leaves
// (decided on the set the repair left), then the vertices with no member
// neighbour are completed in ascending id by the greedy rounds (state 1 in,
// 2 out, 0 undecided; non-members next to a member start out).

__global__ void k_exact_leave(GraphView g, bool sorted, const uint8_t* mis, uint8_t* leave) {
  const int64_t xi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (xi >= g.n) return;
  const int32_t x = (int32_t)xi;
  bool found = false;
  if (mis[x] & 1) {
    const int64_t b = g.nindex[x], e = g.nindex[x + 1];
    const bool filt = g.dead[x] != 0;
    for (int64_t k = b; k < e && !found; ++k) {
      const int32_t y = g.nlist[k];
      if (sorted && y >= x) break;
      if (y >= x || (filt && !live_at(g.live, k))) continue;
      found = (mis[y] & 1) != 0;
    }
    for (int64_t k = g.aoff[x]; k < g.aoff[x + 1] && !found; ++k) {
      const int32_t y = g.aadj[k];
      found = y < x && (mis[y] & 1) != 0;
    }
  }
  leave[x] = found ? 1 : 0;
}

__global__ void k_exact_init(GraphView g, const uint8_t* mis, const uint8_t* leave, uint8_t* st) {
  const int64_t xi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (xi >= g.n) return;
  const int32_t x = (int32_t)xi;
  auto member = [&](int32_t y) { return (mis[y] & 1) != 0 && leave[y] == 0; };
  if (member(x)) {
    st[x] = 1;
    return;
  }
  const bool covered = thread_row_until(g, x, [&](int32_t y) { return member(y); });
  st[x] = covered ? 2 : 0;
}

__global__ void k_exact_out(const uint8_t* st, int32_t n, uint8_t* mis) {
  const int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x < n) mis[x] = st[x] == 1 ? 1 : 0;
}

__global__ void k_greedy_out(const uint8_t* st, int32_t n, uint8_t* out) {
  int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x < n) out[x] = st[x] == 1 ? 1 : 0;
}

__global__ void k_check_mis(GraphView g, const uint8_t* mis, int64_t* counters) {
  int64_t xi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (xi >= g.n) return;
  const int32_t x = (int32_t)xi;
  const bool in = mis[x] != 0;
  bool covered = in;
  int64_t viol = 0;
  thread_row_until(g, x, [&](int32_t y) {
    if (mis[y]) {
      covered = true;
      if (in && x < y) ++viol;
    }
    return false;
  });
  if (viol) atomicAdd((unsigned long long*)(counters + 0), (unsigned long long)viol);
  if (!covered) atomicAdd((unsigned long long*)(counters + 1), 1ull);
}

}  // namespace

void upload_base(mf_ctx* c, int32_t n, const int64_t* nindex, const int32_t* nlist, int64_t nnz) {
  cudaStream_t s = c->stream;
  c->n = n;
  c->nnz = nnz;
  c->nindex.reserve((int64_t)n + 1);
  c->nlist.reserve(nnz + kNlistPad);
  if (nindex) MF_CUDA(cudaMemcpyAsync(c->nindex.p, nindex, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyHostToDevice, s));
  if (nlist && nnz > 0) MF_CUDA(cudaMemcpyAsync(c->nlist.p, nlist, sizeof(int32_t) * (size_t)nnz, cudaMemcpyHostToDevice, s));
  const int64_t words = (nnz + 31) / 32;
  c->live.reserve(words);
  MF_CUDA(cudaMemsetAsync(c->live.p, 0xFF, sizeof(uint32_t) * (size_t)std::max<int64_t>(words, 1), s));
  c->dead.reserve(n);
  c->rcnt.reserve(n);
  c->deg.reserve(n);
  c->aoff.reserve((int64_t)n + 1);
  c->mis.reserve(n);
  c->cid.reserve(n);
  MF_CUDA(cudaMemsetAsync(c->dead.p, 0, sizeof(int32_t) * (size_t)n, s));
  MF_CUDA(cudaMemsetAsync(c->rcnt.p, 0, sizeof(int32_t) * (size_t)n, s));
  MF_CUDA(cudaMemsetAsync(c->aoff.p, 0, sizeof(int64_t) * ((size_t)n + 1), s));
  MF_CUDA(cudaMemsetAsync(c->mis.p, 0, (size_t)n, s));
  MF_CUDA(cudaMemsetAsync(c->cid.p, 0xFF, sizeof(int32_t) * (size_t)n, s));
  c->a_total = 0;
  alloc_vertex_scratch(c);
  if (n > 0) {
    MF_K(k_base_degree<<<grid_for(n), kTB, 0, s>>>(c->nindex.p, n, c->deg.p));
  }
  // validate and detect sorted rows
  MF_CUDA(cudaMemsetAsync(c->counters.p, 0xFF, sizeof(int64_t) * 4, s));
  int* okp = reinterpret_cast<int*>(c->counters.p);
  MF_K(k_check_index<<<grid_for((int64_t)n + 1), kTB, 0, s>>>(c->nindex.p, n, nnz, okp));
  if (nnz > 0) MF_K(k_check_ids<<<grid_for(std::min<int64_t>(nnz, (int64_t)1 << 22)), kTB, 0, s>>>(c->nlist.p, nnz, n, okp + 1));
  MF_CUDA(cudaStreamSynchronize(s));
  int ok[2] = {0, 0};
  MF_CUDA(cudaMemcpy(ok, okp, sizeof(ok), cudaMemcpyDeviceToHost));
  if (!ok[0]) MF_FAIL(MF_EFORMAT, "nindex is not a valid offset array (non-monotone or outside [0, entries])");
  if (!ok[1]) MF_FAIL(MF_EFORMAT, "nlist holds a vertex id outside [0, nodes)");
  // sorted rows and symmetry (both enable the pull form of the clustering write)
  if (n > 0) {
    DBuf<int32_t> all;
    DBuf<int64_t> offs;
    all.reserve(n);
    offs.reserve(2 * (int64_t)n + 1);
    MF_K(k_iota_n<<<grid_for(n), kTB, 0, s>>>(all.p, n));
    MF_K(k_base_positions<<<grid_for(n), kTB, 0, s>>>(c->nindex.p, n, offs.p + n + 1));
    scan_exclusive_i64(offs.p + n + 1, offs.p, n, c->ws, s);
    int sms = 0;
    MF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
    MF_K(k_check_sorted<<<(unsigned)(sms * 8), kTB, 0, s>>>(c->view(), all.p, offs.p, n, okp + 2));
    MF_CUDA(cudaMemcpyAsync(ok, okp + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
    MF_CUDA(cudaStreamSynchronize(s));
    c->rows_sorted = ok[0] != 0;
    c->symmetric = false;
    if (c->rows_sorted) {
      MF_K(k_check_symmetric<<<(unsigned)(sms * 8), kTB, 0, s>>>(c->view(), all.p, offs.p, n, okp + 3));
      MF_CUDA(cudaMemcpyAsync(ok, okp + 3, sizeof(int), cudaMemcpyDeviceToHost, s));
      MF_CUDA(cudaStreamSynchronize(s));
      c->symmetric = ok[0] != 0;
    }
    all.release();
    offs.release();
  } else {
    c->rows_sorted = true;
    c->symmetric = true;
  }
  c->max_csr = initial_max_csr(n, c->header_edges);
}

// The n-sized scratch with its initial values: no row mapped (v2i = -1),
// epoch-tagged arrays at epoch 0, plus the device counters.
void alloc_vertex_scratch(mf_ctx* c) {
  cudaStream_t s = c->stream;
  const int32_t n = c->n;
  c->aoff_alt.reserve((int64_t)n + 1);
  c->v2i.reserve(n);
  c->bval.reserve(n);
  c->wval.reserve(n);
  c->f1.reserve(n);
  c->nmark.reserve(n);
  c->nlist_need.reserve(n);
  c->touched.reserve(n);
  c->hlist.reserve(n);
  c->acnt_new.reserve(n);
  if (n > 0) {
    MF_CUDA(cudaMemsetAsync(c->v2i.p, 0xFF, sizeof(int32_t) * (size_t)n, s));
    MF_CUDA(cudaMemsetAsync(c->bval.p, 0, sizeof(uint32_t) * (size_t)n, s));
    MF_CUDA(cudaMemsetAsync(c->wval.p, 0, sizeof(uint32_t) * (size_t)n, s));
    MF_CUDA(cudaMemsetAsync(c->nmark.p, 0, sizeof(uint32_t) * (size_t)n, s));
  }
  c->epoch = 0;
  c->counters.reserve(64);
}

void flag_updates(mf_ctx* c, int64_t m) {
  if (m <= 0) return;
  MF_K(k_flags<<<grid_for(m), kTB, 0, c->stream>>>(c->view(), c->rows_sorted, c->bu.p, c->bv.p, m, c->bins.p));
  MF_CUDA(cudaGetLastError());
}

void apply_overlay(mf_ctx* c, int64_t m) {
  if (m <= 0) return;
  cudaStream_t s = c->stream;
  const int nbits = bits_for(std::max<int32_t>(c->n - 1, 1));
  c->keys.reserve(2 * m);
  c->vals.reserve(2 * m);
  MF_K(k_pair_keys<<<grid_for(m), kTB, 0, s>>>(c->bu.p, c->bv.p, m, nbits, c->keys.p, c->vals.p));
  radix_sort_pairs(c->keys.p, c->vals.p, m, 2 * nbits, c->ws, s);

  const int64_t cap_new = c->a_total + 2 * m;
  c->akill.reserve(std::max<int64_t>(c->a_total, 1));
  c->app_keys.reserve(2 * m);
  c->app_vals.reserve(2 * m);
  c->aadj_alt.reserve(cap_new);
  c->aown_alt.reserve(cap_new);
  c->aadj.reserve(std::max<int64_t>(c->a_total, 1));
  c->aown.reserve(std::max<int64_t>(c->a_total, 1));
  c->i64a.reserve(std::max<int64_t>(c->a_total, 1) + 1);
  if (c->a_total > 0) MF_CUDA(cudaMemsetAsync(c->akill.p, 0, (size_t)c->a_total, s));
  MF_CUDA(cudaMemsetAsync(c->counters.p, 0, sizeof(int64_t) * 2, s));
  MF_K(k_init_acnt<<<grid_for(c->n), kTB, 0, s>>>(c->aoff.p, c->n, c->acnt_new.p));
  MF_K(k_apply_pairs<<<grid_for(m), kTB, 0, s>>>(c->view(), c->live.p, c->dead.p, c->rcnt.p, c->rows_sorted,
                                            c->keys.p, c->vals.p, m, nbits, c->bu.p, c->bv.p, c->bins.p,
                                            c->acnt_new.p, c->akill.p, c->app_keys.p, c->app_vals.p,
                                            c->counters.p));
  MF_CUDA(cudaGetLastError());
  MF_CUDA(cudaMemcpyAsync(c->h_counters, c->counters.p, sizeof(int64_t) * 2, cudaMemcpyDeviceToHost, s));
  MF_CUDA(cudaStreamSynchronize(s));
  const int64_t appended = c->h_counters[0], killed = c->h_counters[1];
  if (appended == 0 && killed == 0) {
    MF_K(k_degrees<<<grid_for(c->n), kTB, 0, s>>>(c->nindex.p, c->rcnt.p, c->aoff.p, c->n, c->deg.p));
    MF_CUDA(cudaGetLastError());
    return;
  }
  // new offsets
  scan_exclusive_i32(c->acnt_new.p, c->aoff_alt.p, c->n, c->ws, s);
  if (c->a_total > 0) {
    scan_exclusive_u8(c->akill.p, c->i64a.p, c->a_total, c->ws, s);
    MF_K(k_move_survivors<<<grid_for(c->a_total), kTB, 0, s>>>(c->aoff.p, c->aadj.p, c->aown.p, c->akill.p, c->i64a.p,
                                                          c->a_total, c->aoff_alt.p, c->aadj_alt.p, c->aown_alt.p));
  }
  if (appended > 0) {
    radix_sort_pairs(c->app_keys.p, c->app_vals.p, appended, 32 + nbits, c->ws, s);
    MF_K(k_place_appends<<<grid_for(appended), kTB, 0, s>>>(c->app_keys.p, c->app_vals.p, appended, c->aoff_alt.p,
                                                       c->aadj_alt.p, c->aown_alt.p));
  }
  MF_CUDA(cudaGetLastError());
  std::swap(c->aoff, c->aoff_alt);
  std::swap(c->aadj, c->aadj_alt);
  std::swap(c->aown, c->aown_alt);
  c->a_total = c->a_total + appended - killed;
  MF_K(k_degrees<<<grid_for(c->n), kTB, 0, s>>>(c->nindex.p, c->rcnt.p, c->aoff.p, c->n, c->deg.p));
  MF_CUDA(cudaGetLastError());
}

void compact_graph(mf_ctx* c, std::vector<int64_t>& nindex_out, std::vector<int32_t>& nlist_out) {
  cudaStream_t s = c->stream;
  const int32_t n = c->n;
  MF_CUDA(cudaMemsetAsync(c->counters.p, 0, sizeof(int64_t) * 2, s));
  if (n > 0) MF_K(k_compact_check<<<grid_for(n), kTB, 0, s>>>(c->view(), c->deg.p, c->counters.p));
  MF_CUDA(cudaMemcpyAsync(c->h_counters, c->counters.p, sizeof(int64_t) * 2, cudaMemcpyDeviceToHost, s));
  MF_CUDA(cudaStreamSynchronize(s));
  if (c->h_counters[0] > 0) MF_FAIL(MF_ESTATE, "compaction computed a negative degree: delta is inconsistent with the base graph");
  if (c->h_counters[1] > 0) MF_FAIL(MF_ESTATE, "compaction degree mismatch: tombstones without base entries (asymmetric base graph)");
  c->i64b.reserve((int64_t)n + 1);
  scan_exclusive_i32(c->deg.p, c->i64b.p, n, c->ws, s);
  int64_t total = 0;
  MF_CUDA(cudaMemcpyAsync(&total, c->i64b.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  MF_CUDA(cudaStreamSynchronize(s));
  DBuf<int32_t> out;
  out.reserve(std::max<int64_t>(total, 1));
  if (n > 0) MF_K(k_compact_gather<<<grid_for((int64_t)n * 32), kTB, 0, s>>>(c->view(), c->i64b.p, out.p));
  MF_CUDA(cudaGetLastError());
  nindex_out.resize((size_t)n + 1);
  nlist_out.resize((size_t)total);
  MF_CUDA(cudaMemcpyAsync(nindex_out.data(), c->i64b.p, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyDeviceToHost, s));
  if (total > 0) MF_CUDA(cudaMemcpyAsync(nlist_out.data(), out.p, sizeof(int32_t) * (size_t)total, cudaMemcpyDeviceToHost, s));
  MF_CUDA(cudaStreamSynchronize(s));
  out.release();
}

void greedy_mis(mf_ctx* c, uint8_t* d_out) {
  cudaStream_t s = c->stream;
  const int32_t n = c->n;
  if (n <= 0) return;
  DBuf<uint8_t> st;
  st.reserve(n);
  MF_CUDA(cudaMemsetAsync(st.p, 0, (size_t)n, s));
  for (int round = 0;; ++round) {
    MF_CUDA(cudaMemsetAsync(c->counters.p, 0, sizeof(int64_t), s));
    MF_K(k_greedy_round<<<grid_for(n), kTB, 0, s>>>(c->view(), c->rows_sorted, st.p, c->counters.p));
    MF_CUDA(cudaMemcpyAsync(c->h_counters, c->counters.p, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    MF_CUDA(cudaStreamSynchronize(s));
    if (c->h_counters[0] == 0) break;
    if (round > n + 2) MF_FAIL(MF_ESTATE, "greedy MIS did not settle");
  }
  MF_K(k_greedy_out<<<grid_for(n), kTB, 0, s>>>(st.p, n, d_out));
  MF_CUDA(cudaStreamSynchronize(s));
  st.release();
}

void exact_fixup(mf_ctx* c) {
  cudaStream_t s = c->stream;
  const int32_t n = c->n;
  if (n <= 0) return;
  c->xst.reserve(n);
  c->xleave.reserve(n);
  MF_K(k_exact_leave<<<grid_for(n), kTB, 0, s>>>(c->view(), c->rows_sorted, c->mis.p, c->xleave.p));
  MF_K(k_exact_init<<<grid_for(n), kTB, 0, s>>>(c->view(), c->mis.p, c->xleave.p, c->xst.p));
  for (int round = 0;; ++round) {
    MF_CUDA(cudaMemsetAsync(c->counters.p, 0, sizeof(int64_t), s));
    MF_K(k_greedy_round<<<grid_for(n), kTB, 0, s>>>(c->view(), c->rows_sorted, c->xst.p, c->counters.p));
    MF_CUDA(cudaMemcpyAsync(c->h_counters, c->counters.p, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    MF_CUDA(cudaStreamSynchronize(s));
    if (c->h_counters[0] == 0) break;
    if (round > n + 2) MF_FAIL(MF_ESTATE, "exact-MIS completion did not settle");
  }
  MF_K(k_exact_out<<<grid_for(n), kTB, 0, s>>>(c->xst.p, n, c->mis.p));
  MF_CUDA(cudaGetLastError());
}

void check_mis(mf_ctx* c, int64_t* viol, int64_t* uncovered) {
  cudaStream_t s = c->stream;
  MF_CUDA(cudaMemsetAsync(c->counters.p, 0, sizeof(int64_t) * 2, s));
  if (c->n > 0) MF_K(k_check_mis<<<grid_for(c->n), kTB, 0, s>>>(c->view(), c->mis.p, c->counters.p));
  MF_CUDA(cudaMemcpyAsync(c->h_counters, c->counters.p, sizeof(int64_t) * 2, cudaMemcpyDeviceToHost, s));
  MF_CUDA(cudaStreamSynchronize(s));
  *viol = c->h_counters[0];
  *uncovered = c->h_counters[1];
}

void rebase(mf_ctx* c) {
  std::vector<int64_t> ni;
  std::vector<int32_t> nl;
  compact_graph(c, ni, nl);
  // keep membership and cluster ids; the base becomes the compacted graph
  DBuf<uint8_t> mis_keep;
  DBuf<int32_t> cid_keep;
  cudaStream_t s = c->stream;
  const int32_t n = c->n;
  mis_keep.reserve(std::max(n, 1));
  cid_keep.reserve(std::max(n, 1));
  MF_CUDA(cudaMemcpyAsync(mis_keep.p, c->mis.p, (size_t)n, cudaMemcpyDeviceToDevice, s));
  MF_CUDA(cudaMemcpyAsync(cid_keep.p, c->cid.p, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToDevice, s));
  c->nlist.release();
  c->live.release();
  c->header_edges = (uint64_t)nl.size();
  const int64_t keep_max = c->max_csr;
  upload_base(c, n, ni.data(), nl.data(), (int64_t)nl.size());
  c->max_csr = keep_max;
  MF_CUDA(cudaMemcpyAsync(c->mis.p, mis_keep.p, (size_t)n, cudaMemcpyDeviceToDevice, s));
  MF_CUDA(cudaMemcpyAsync(c->cid.p, cid_keep.p, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToDevice, s));
  MF_CUDA(cudaStreamSynchronize(s));
  mis_keep.release();
  cid_keep.release();
}

}  // namespace mf

// ---- update flags without allocation ------------------------------------------
// mf_flag_updates stages the endpoints in the context's buffers, which grow
// to the largest batch seen (cudaFree of the old buffer + cudaMalloc).  This
// variant stages them in one fixed device array instead, so that it never
// allocates: every call on a device uses the same array, found once per
// device with cudaGetSymbolAddress.
//
// Layout of the array (byte offsets, each part 256-byte aligned):
//   [0, 256)                     invalid-pair counter (u64; zeroed every call)
//   [256, 256 + 4K)              u endpoints (int32, K = MF_NOALLOC_MAX_UPDATES)
//   [256 + 4K, 256 + 8K)         v endpoints
//   [256 + 8K, 256 + 9K)         flags (u8)
// K = 65536 gives 590,080 bytes.
namespace {
constexpr size_t kNaCounterBytes = 256;
constexpr size_t kNaEndpointBytes = sizeof(int32_t) * (size_t)MF_NOALLOC_MAX_UPDATES;
constexpr size_t kNaScratchBytes = kNaCounterBytes + 2 * kNaEndpointBytes + (size_t)MF_NOALLOC_MAX_UPDATES;
constexpr int kNaMaxDevices = 64;
static_assert(kNaEndpointBytes % 256 == 0, "each part of the scratch starts on a 256-byte boundary");
}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaScratchBytes];

namespace mf {
namespace {

std::mutex g_na_mutex;
unsigned char* g_na_base[kNaMaxDevices] = {};

// Device address of the scratch array on the current device (which must be
// `device`).  The first call for a device looks it up; later calls read the
// table.
unsigned char* noalloc_scratch(int device) {
  if (device < 0 || device >= kNaMaxDevices) MF_FAIL(MF_ELIMIT, "device id beyond the no-allocation table (64)");
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (g_na_base[device] == nullptr) {
    void* p = nullptr;
    MF_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    if (p == nullptr) MF_FAIL(MF_ECUDA, "cudaGetSymbolAddress returned a null scratch address");
    g_na_base[device] = static_cast<unsigned char*>(p);
  }
  return g_na_base[device];
}

}  // namespace

// Looks the scratch address up again for `device` (current on the calling
// thread).  Contexts call this when they are created, so that a device
// whose primary context was reset and re-created gets the new address.
void noalloc_refresh(int device) {
  if (device < 0 || device >= kNaMaxDevices) return;
  void* p = nullptr;
  MF_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
  std::lock_guard<std::mutex> lock(g_na_mutex);
  g_na_base[device] = static_cast<unsigned char*>(p);
}

void flag_updates_noalloc(mf_ctx* c, const int32_t* u, const int32_t* v, int64_t m, uint8_t* ins_out) {
  if (m > (int64_t)MF_NOALLOC_MAX_UPDATES)
    MF_FAIL(MF_ELIMIT, "mf_flag_updates_noalloc takes at most 65536 updates per call");
  unsigned char* base = noalloc_scratch(c->device);
  if (m <= 0) return;
  cudaStream_t s = c->stream;
  auto* bad = reinterpret_cast<unsigned long long*>(base);
  auto* du = reinterpret_cast<int32_t*>(base + kNaCounterBytes);
  auto* dv = reinterpret_cast<int32_t*>(base + kNaCounterBytes + kNaEndpointBytes);
  auto* dins = base + kNaCounterBytes + 2 * kNaEndpointBytes;
  // the counter is the only part read before it is written
  MF_CUDA(cudaMemsetAsync(bad, 0, sizeof(unsigned long long), s));
  MF_CUDA(cudaMemcpyAsync(du, u, sizeof(int32_t) * (size_t)m, cudaMemcpyHostToDevice, s));
  MF_CUDA(cudaMemcpyAsync(dv, v, sizeof(int32_t) * (size_t)m, cudaMemcpyHostToDevice, s));
  MF_K(k_flags_checked<<<grid_for(m), kTB, 0, s>>>(c->view(), c->rows_sorted, du, dv, m, dins, bad));
  MF_CUDA(cudaGetLastError());
  unsigned long long nbad = 0;
  MF_CUDA(cudaMemcpyAsync(&nbad, bad, sizeof(nbad), cudaMemcpyDeviceToHost, s));
  MF_CUDA(cudaStreamSynchronize(s));
  if (nbad != 0) MF_FAIL(MF_EINVAL, "update endpoints must be distinct vertex ids in [0, n)");
  MF_CUDA(cudaMemcpyAsync(ins_out, dins, (size_t)m, cudaMemcpyDeviceToHost, s));
  MF_CUDA(cudaStreamSynchronize(s));
}

}  // namespace mf
