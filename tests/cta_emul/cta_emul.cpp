// cta_emul.cpp -- runs the batched form's one-CTA engine (misfit_gb300/csrc/
// mf_cta.cuh) on the CPU.  TEST INFRASTRUCTURE ONLY: it lets the CPU test
// suite compare the engine's logic, stage by stage semantics included, with
// the oracle without a GPU.  The library never uses it; on a GPU the same
// source runs as the persistent kernel in mf_batched.cu.
//
// One CTA of nt threads is emulated by nt OS threads: __syncthreads is a
// pthread barrier, __shared__ variables are function-static, atomics are the
// compiler's __atomic builtins.  The graph state has the device layout of an
// mf_ctx (base CSR, live bits, dead/rcnt counts, added CSR with owners,
// degrees, membership, cluster ids) plus the engine's kept vertex scratch.
#include <pthread.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <thread>
#include <vector>

#include "../../misfit_gb300/csrc/mf_cta.cuh"

namespace mf {
namespace cta {
thread_local int emul_tid = 0;
int emul_nt = 1;
static pthread_barrier_t g_barrier;
void emul_sync() { pthread_barrier_wait(&g_barrier); }
}  // namespace cta
}  // namespace mf

namespace {
int64_t initial_max_csr(int32_t n, uint64_t edges) {
  double avg = n > 0 ? (double)edges / n : 1.0;
  int64_t est = (int64_t)(1048576 * 2.0 * avg * avg);
  int64_t v = est > 0 ? std::min<int64_t>(800000000LL, est) : 50000000LL;
  return std::max<int64_t>(v, 1000000LL);
}
}  // namespace

struct eg {
  int32_t n = 0;
  int64_t nnz = 0;
  bool sorted = true;
  std::vector<int64_t> nindex;
  std::vector<int32_t> nlist;
  std::vector<uint32_t> live;
  std::vector<int32_t> dead, rcnt, deg;
  std::vector<int64_t> aoff{0};
  std::vector<int32_t> aadj, aown;
  int64_t a_total = 0;
  std::vector<uint8_t> mis;
  std::vector<int32_t> cid;
  std::vector<uint32_t> win;
  std::vector<int32_t> map;
  std::vector<uint32_t> hbits, sbits, xbits;
  uint32_t epoch = 0;
  int64_t max_csr = 0;
  int64_t last[mf::cta::kOutWords] = {};
};

extern "C" {

eg* eg_create(int32_t n, const int64_t* nindex, const int32_t* nlist) {
  eg* g = new eg();
  g->n = n;
  g->nindex.assign(nindex, nindex + n + 1);
  g->nnz = g->nindex[n];
  g->nlist.assign(nlist, nlist + g->nnz);
  for (int32_t x = 0; x < n && g->sorted; ++x)
    for (int64_t k = g->nindex[x] + 1; k < g->nindex[x + 1]; ++k)
      if (g->nlist[k - 1] > g->nlist[k]) { g->sorted = false; break; }
  g->live.assign((size_t)((g->nnz + 31) / 32) + 1, 0xffffffffu);
  g->dead.assign(n, 0);
  g->rcnt.assign(n, 0);
  g->deg.resize(n);
  for (int32_t x = 0; x < n; ++x) g->deg[x] = (int32_t)(g->nindex[x + 1] - g->nindex[x]);
  g->aoff.assign((size_t)n + 1, 0);
  g->mis.assign(n, 0);
  g->cid.assign(n, -1);
  g->win.assign(n, 0);
  g->map.assign(n, -1);
  const size_t w = (size_t)(n + 31) / 32 + 1;
  g->hbits.assign(w, 0);
  g->sbits.assign(w, 0);
  g->xbits.assign(w, 0);
  g->max_csr = initial_max_csr(n, (uint64_t)g->nnz);
  return g;
}

void eg_destroy(eg* g) { delete g; }
void eg_set_mis(eg* g, const uint8_t* mis) {
  for (int32_t i = 0; i < g->n; ++i) {
    g->mis[i] = mis[i] ? 1 : 0;
    g->cid[i] = -1;
  }
}
void eg_get_mis(const eg* g, uint8_t* out) { std::memcpy(out, g->mis.data(), g->n); }
void eg_get_cid(const eg* g, int32_t* out) { std::memcpy(out, g->cid.data(), sizeof(int32_t) * g->n); }
void eg_degrees(const eg* g, int32_t* out) { std::memcpy(out, g->deg.data(), sizeof(int32_t) * g->n); }
int64_t eg_max_csr(const eg* g) { return g->max_csr; }
void eg_set_max_csr(eg* g, int64_t v) { g->max_csr = v; }
const int64_t* eg_last(const eg* g) { return g->last; }

int64_t eg_row(const eg* g, int32_t x, int32_t* out, int64_t cap) {
  int64_t len = 0;
  for (int64_t k = g->nindex[x]; k < g->nindex[x + 1]; ++k)
    if ((g->live[k >> 5] >> (k & 31)) & 1u) {
      if (len < cap) out[len] = g->nlist[k];
      ++len;
    }
  for (int64_t k = g->aoff[x]; k < g->aoff[x + 1]; ++k) {
    if (len < cap) out[len] = g->aadj[k];
    ++len;
  }
  return len;
}

// One batch through the engine with nt emulated threads; returns the number
// of sub-batches.
int64_t eg_apply(eg* g, const int32_t* u, const int32_t* v, const uint8_t* ins, int64_t m, int nt) {
  using namespace mf::cta;
  if (m <= 0) return 0;
  const int64_t s2 = 2 * m + 1;
  const int64_t rows = 2 * m + g->n + 1;
  std::vector<uint64_t> k0(s2), k1(s2), ak(s2);
  std::vector<uint32_t> v0(s2), v1(s2), av(s2);
  std::vector<int32_t> prev(s2), rowsv(rows), rowcid(rows), acnt(g->n + 1);
  std::vector<int64_t> ends(rows + 1), kp(g->a_total + 2), aoff_new(g->n + 1);
  std::vector<uint8_t> akill(g->a_total + 1);
  std::vector<int32_t> aadj_new(g->a_total + 2 * m + 1), aown_new(g->a_total + 2 * m + 1);
  std::vector<int32_t> uu(u, u + m), vv(v, v + m);
  std::vector<uint8_t> ii(ins, ins + m);
  int64_t out[kOutWords] = {};
  Item it{};
  it.n = g->n;
  it.sorted = g->sorted ? 1 : 0;
  it.nindex = g->nindex.data();
  it.nlist = g->nlist.data();
  it.live = g->live.data();
  it.dead = g->dead.data();
  it.rcnt = g->rcnt.data();
  it.deg = g->deg.data();
  it.aoff = g->aoff.data();
  it.aadj = g->aadj.data();
  it.aown = g->aown.data();
  it.a_total = g->a_total;
  it.aoff_new = aoff_new.data();
  it.aadj_new = aadj_new.data();
  it.aown_new = aown_new.data();
  it.mis = g->mis.data();
  it.cid = g->cid.data();
  it.u = uu.data();
  it.v = vv.data();
  it.ins = ii.data();
  it.m = m;
  it.max_csr = g->max_csr;
  it.epoch = g->epoch;
  it.win = g->win.data();
  it.map = g->map.data();
  it.hbits = g->hbits.data();
  it.sbits = g->sbits.data();
  it.xbits = g->xbits.data();
  it.k0 = k0.data();
  it.v0 = v0.data();
  it.k1 = k1.data();
  it.v1 = v1.data();
  it.ak = ak.data();
  it.av = av.data();
  it.prev = prev.data();
  it.rows = rowsv.data();
  it.rowcid = rowcid.data();
  it.ends = ends.data();
  it.acnt = acnt.data();
  it.akill = akill.data();
  it.kp = kp.data();
  it.out = out;

  std::vector<int64_t> sh(kMaxThreads);
  std::vector<int32_t> hist((size_t)kBuckets * kMaxThreads);
  emul_nt = nt;
  pthread_barrier_init(&g_barrier, nullptr, (unsigned)nt);
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t)
    th.emplace_back([&, t] {
      emul_tid = t;
      run_item(it, hist.data(), sh.data());
    });
  for (auto& t : th) t.join();
  pthread_barrier_destroy(&g_barrier);

  if (out[kOutSwapped]) {
    const int64_t at = out[kOutATotal];
    g->aoff = aoff_new;
    g->aadj.assign(aadj_new.begin(), aadj_new.begin() + at);
    g->aown.assign(aown_new.begin(), aown_new.begin() + at);
  }
  g->a_total = out[kOutATotal];
  g->max_csr = out[kOutMaxCsr];
  g->epoch = (uint32_t)out[kOutEpoch];
  std::memcpy(g->last, out, sizeof(out));
  return out[kOutSubBatches];
}

}  // extern "C"
