// mf_batched.cu -- the batched form: one update batch for each of many graphs
// in one step (mf_apply_batches).
//
// Batches that one CTA can carry run in a single persistent kernel: the
// host stages every such batch and an item table (device pointers of each
// graph's state and scratch) in one pinned buffer, and one step -- the
// upload, the reset of the work-queue head, the kernel and the read-back
// of the per-graph results -- is captured as a CUDA graph and launched.
// Each CTA of the kernel takes the next item from the queue (items sorted
// by estimated cost, largest first, so the long ones start early) and runs
// the whole path for that graph (mf_cta.cuh).  The other batches go through
// the multi-launch path on their own contexts' streams while the kernel runs.
//
// The engine works on each context's own device state, so per-graph results
// equal mf_apply_batch's, and a graph can alternate between the two paths.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "mf_cta.cuh"
#include "mf_internal.cuh"

namespace mf {
namespace {

__global__ void __launch_bounds__(1024, 1) k_batched(const cta::Item* items, int64_t count, int* head) {
  extern __shared__ __align__(16) unsigned char smem[];
  int64_t* sh = reinterpret_cast<int64_t*>(smem);
  int32_t* hist = reinterpret_cast<int32_t*>(sh + blockDim.x);
  __shared__ int s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(head, 1);
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    if (it >= count) return;
    cta::run_item(items[it], hist, sh);
  }
}

constexpr size_t kAlign = 256;
inline size_t align_up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

// Byte layout of a context's kept per-vertex engine scratch.
struct VertLayout {
  size_t win, map, hbits, sbits, xbits, total;
  explicit VertLayout(int32_t n) {
    const size_t w = ((size_t)n + 31) / 32 + 1;
    size_t o = 0;
    win = o; o = align_up(o + 4 * (size_t)n + 4);
    map = o; o = align_up(o + 4 * (size_t)n + 4);
    hbits = o; o = align_up(o + 4 * w);
    sbits = o; o = align_up(o + 4 * w);
    xbits = o; o = align_up(o + 4 * w);
    total = o;
  }
};

// Byte layout of one item's per-batch scratch.
struct WsLayout {
  size_t k0, k1, ak, v0, v1, av, prev, rows, rowcid, ends, acnt, akill, kp, total;
  WsLayout(int32_t n, int64_t m, int64_t a_total) {
    const size_t s2 = 2 * (size_t)m + 1, r = 2 * (size_t)m + (size_t)n + 2;
    size_t o = 0;
    k0 = o; o = align_up(o + 8 * s2);
    k1 = o; o = align_up(o + 8 * s2);
    ak = o; o = align_up(o + 8 * s2);
    v0 = o; o = align_up(o + 4 * s2);
    v1 = o; o = align_up(o + 4 * s2);
    av = o; o = align_up(o + 4 * s2);
    prev = o; o = align_up(o + 4 * s2);
    rows = o; o = align_up(o + 4 * r);
    rowcid = o; o = align_up(o + 4 * r);
    ends = o; o = align_up(o + 8 * (r + 1));
    acnt = o; o = align_up(o + 4 * ((size_t)n + 1));
    akill = o; o = align_up(o + (size_t)a_total + 1);
    kp = o; o = align_up(o + 8 * ((size_t)a_total + 2));
    total = o;
  }
};

// Per-device state of the batched step: its stream, staging and outputs.
struct Engine {
  std::mutex mu;
  bool ready = false;
  int sms = 0;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  DBuf<uint8_t> d_stage;
  DBuf<int64_t> d_out;
  DBuf<int> d_head;
  uint8_t* h_stage = nullptr;
  size_t h_stage_cap = 0;
  int64_t* h_out = nullptr;
  size_t h_out_cap = 0;
};

constexpr int kMaxDevices = 64;
Engine g_engines[kMaxDevices];

void engine_init(Engine& E, int device) {
  if (E.ready) return;
  MF_CUDA(cudaStreamCreateWithFlags(&E.s, cudaStreamNonBlocking));
  MF_CUDA(cudaEventCreate(&E.e0));
  MF_CUDA(cudaEventCreate(&E.e1));
  MF_CUDA(cudaDeviceGetAttribute(&E.sms, cudaDevAttrMultiProcessorCount, device));
  MF_CUDA(cudaFuncSetAttribute(k_batched, cudaFuncAttributeMaxDynamicSharedMemorySize, cta::kSmemBytes));
  E.ready = true;
}

void pinned_reserve(uint8_t** p, size_t* cap, size_t need) {
  if (need <= *cap) return;
  if (*p) cudaFreeHost(*p);
  *p = nullptr;
  *cap = 0;
  note_alloc();
  MF_CUDA(cudaMallocHost(reinterpret_cast<void**>(p), need));
  *cap = need;
}

struct KernelItem {
  int64_t idx;      // position in the caller's arrays
  double cost;
};

}  // namespace
}  // namespace mf

namespace {

using mf::Failure;

void need(bool cond, int status, const char* msg) {
  if (!cond) MF_FAIL(status, msg);
}

mf_batched_opts default_opts() {
  mf_batched_opts o;
  o.block = 512;
  o.ctas_per_sm = 2;
  o.max_cta_updates = 8192;
  o.max_cta_vertices = 1 << 20;
  o.use_graph = 1;
  o.path_threads = 8;
  o.pool_idle_first = 1;
  return o;
}

double host_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// The multi-launch path for the batches above the kernel's limits: each
// one is host-driven (sizes read back between stages), so they run on
// host threads, each graph on its own stream, largest first.  Returns the
// first failure's status (its message in *error).
int run_path_items(mf_ctx* const* ctxs, const int32_t* const* u, const int32_t* const* v, const uint8_t* const* ins,
                   const int64_t* m, std::vector<int64_t> items, int threads, std::string* error) {
  if (items.empty()) return MF_OK;
  std::sort(items.begin(), items.end(), [&](int64_t a, int64_t b) { return m[a] > m[b]; });
  const size_t nt = std::min((size_t)std::max(threads, 1), items.size());
  std::mutex mu;
  size_t next = 0;
  int status = MF_OK;
  auto drive = [&] {
    for (;;) {
      int64_t i;
      {
        std::lock_guard<std::mutex> lk(mu);
        if (next >= items.size()) return;
        i = items[next++];
      }
      const int r = mf_apply_batch(ctxs[i], u[i], v[i], ins[i], m[i]);
      if (r != MF_OK) {
        std::lock_guard<std::mutex> lk(mu);
        if (status == MF_OK) {
          status = r;
          *error = mf_last_error();
        }
      }
    }
  };
  if (nt == 1) {
    drive();
  } else {
    std::vector<std::thread> th;
    for (size_t t = 0; t < nt; ++t) th.emplace_back(drive);
    for (auto& t : th) t.join();
  }
  return status;
}

void apply_batches(mf_ctx* const* ctxs, const int32_t* const* u, const int32_t* const* v, const uint8_t* const* ins,
                   const int64_t* m, int64_t count, const mf_batched_opts& o, mf_batched_stats* st) {
  using namespace mf;
  const double t_start = host_ms();
  need(count >= 0 && (count == 0 || (ctxs && u && v && ins && m)), MF_EINVAL, "bad arguments");
  need(o.block >= 64 && o.block <= cta::kMaxThreads && o.block % 32 == 0, MF_EINVAL,
       "block must be a multiple of 32 in [64, 1024]");
  need(o.ctas_per_sm >= 1 && o.ctas_per_sm <= 32, MF_EINVAL, "ctas_per_sm must be in [1, 32]");
  need(o.max_cta_updates >= 0 && o.max_cta_updates <= cta::kMaxBatchEdges, MF_EINVAL,
       "max_cta_updates must be in [0, 1048576]");
  need(o.path_threads >= 1 && o.path_threads <= 64, MF_EINVAL, "path_threads must be in [1, 64]");
  mf_batched_stats stats{};
  if (count == 0) {
    if (st) *st = stats;
    return;
  }
  const int device = ctxs[0] ? ctxs[0]->device : -1;
  need(device >= 0 && device < kMaxDevices, MF_EINVAL, "null context or device id out of range");
  {
    std::vector<mf_ctx*> seen(ctxs, ctxs + count);
    std::sort(seen.begin(), seen.end());
    need(std::adjacent_find(seen.begin(), seen.end()) == seen.end(), MF_EINVAL, "contexts must be distinct");
  }
  // Check every batch before anything runs.
  for (int64_t i = 0; i < count; ++i) {
    mf_ctx* c = ctxs[i];
    need(c != nullptr, MF_EINVAL, "null context");
    need(c->device == device, MF_EINVAL, "contexts must be on one GPU");
    need(!c->pending, MF_EINVAL, "asynchronous batches are pending; collect them (mf_collect / mf_sync) first");
    need(m[i] >= 0 && (m[i] == 0 || (u[i] && v[i] && ins[i])), MF_EINVAL, "bad batch arrays");
    for (int64_t k = 0; k < m[i]; ++k) {
      const int32_t a = u[i][k], b = v[i][k];
      need(a >= 0 && a < c->n && b >= 0 && b < c->n && a != b, MF_EINVAL,
           "update endpoints out of range or equal");
    }
    stats.updates += m[i];
  }

  std::vector<KernelItem> kitems;
  std::vector<int64_t> path_items;
  for (int64_t i = 0; i < count; ++i) {
    mf_ctx* c = ctxs[i];
    if (m[i] == 0) {
      c->stats = mf_batch_stats{};
      c->stats.packed_total = -1;
      c->stats.row_degree_total = -1;
      c->stats.max_csr = c->max_csr;
      continue;
    }
    const bool fits = m[i] <= o.max_cta_updates && c->n <= o.max_cta_vertices && !c->exact;
    if (fits) {
      const double avg = c->n > 0 ? (double)c->nnz / c->n : 0.0;
      kitems.push_back({i, (double)m[i] * (1.0 + avg) * (1.0 + avg)});
    } else {
      path_items.push_back(i);
    }
  }
  std::sort(kitems.begin(), kitems.end(), [](const KernelItem& a, const KernelItem& b) { return a.cost > b.cost; });
  stats.kernel_items = (int64_t)kitems.size();
  stats.path_items = (int64_t)path_items.size();

  Engine& E = g_engines[device];
  std::unique_lock<std::mutex> lock(E.mu);
  const int64_t k = (int64_t)kitems.size();
  if (k > 0) {
    MF_CUDA(cudaSetDevice(device));
    engine_init(E, device);
    // each context's kept and per-batch scratch, allocated on its stream
    for (const KernelItem& ki : kitems) {
      mf_ctx* c = ctxs[ki.idx];
      g_alloc_stream = c->stream;
      const VertLayout vl(c->n);
      const bool fresh = c->cta_vert.p == nullptr || c->cta_vert.cap < (int64_t)vl.total;
      c->cta_vert.reserve((int64_t)vl.total);
      if (fresh) {
        uint8_t* b = c->cta_vert.p;
        MF_CUDA(cudaMemsetAsync(b + vl.win, 0, vl.map - vl.win, c->stream));
        MF_CUDA(cudaMemsetAsync(b + vl.map, 0xFF, vl.hbits - vl.map, c->stream));
        MF_CUDA(cudaMemsetAsync(b + vl.hbits, 0, vl.total - vl.hbits, c->stream));
        c->cta_epoch = 0;
      }
      const WsLayout wl(c->n, m[ki.idx], c->a_total);
      c->cta_ws.reserve((int64_t)wl.total);
      c->aoff_alt.reserve((int64_t)c->n + 1);
      c->aadj_alt.reserve(c->a_total + 2 * m[ki.idx] + 1);
      c->aown_alt.reserve(c->a_total + 2 * m[ki.idx] + 1);
      c->aadj.reserve(std::max<int64_t>(c->a_total, 1));
      c->aown.reserve(std::max<int64_t>(c->a_total, 1));
      MF_CUDA(cudaEventRecord(c->ev_a, c->stream));
      MF_CUDA(cudaStreamWaitEvent(E.s, c->ev_a, 0));
    }
    g_alloc_stream = nullptr;

    // pinned staging: item table, then every item's u, v (int32) and ins (u8)
    const size_t table = align_up(sizeof(cta::Item) * (size_t)k);
    std::vector<size_t> off_u(k), off_v(k), off_i(k);
    size_t o_b = table;
    for (int64_t j = 0; j < k; ++j) {
      const int64_t mm = m[kitems[j].idx];
      off_u[j] = o_b; o_b = align_up(o_b + 4 * (size_t)mm);
      off_v[j] = o_b; o_b = align_up(o_b + 4 * (size_t)mm);
      off_i[j] = o_b; o_b = align_up(o_b + (size_t)mm);
    }
    pinned_reserve(&E.h_stage, &E.h_stage_cap, o_b);
    {
      uint8_t* hout = reinterpret_cast<uint8_t*>(E.h_out);
      pinned_reserve(&hout, &E.h_out_cap, sizeof(int64_t) * cta::kOutWords * (size_t)k);
      E.h_out = reinterpret_cast<int64_t*>(hout);
    }
    E.d_stage.reserve((int64_t)o_b);
    E.d_out.reserve(cta::kOutWords * k);
    E.d_head.reserve(1);
    uint8_t* ds = E.d_stage.p;
    cta::Item* table_h = reinterpret_cast<cta::Item*>(E.h_stage);
    for (int64_t j = 0; j < k; ++j) {
      const int64_t i = kitems[j].idx;
      mf_ctx* c = ctxs[i];
      const int64_t mm = m[i];
      std::memcpy(E.h_stage + off_u[j], u[i], 4 * (size_t)mm);
      std::memcpy(E.h_stage + off_v[j], v[i], 4 * (size_t)mm);
      std::memcpy(E.h_stage + off_i[j], ins[i], (size_t)mm);
      const VertLayout vl(c->n);
      const WsLayout wl(c->n, mm, c->a_total);
      uint8_t* vb = c->cta_vert.p;
      uint8_t* wb = c->cta_ws.p;
      cta::Item it{};
      it.n = c->n;
      it.sorted = c->rows_sorted ? 1 : 0;
      it.nindex = c->nindex.p;
      it.nlist = c->nlist.p;
      it.live = c->live.p;
      it.dead = c->dead.p;
      it.rcnt = c->rcnt.p;
      it.deg = c->deg.p;
      it.aoff = c->aoff.p;
      it.aadj = c->aadj.p;
      it.aown = c->aown.p;
      it.a_total = c->a_total;
      it.aoff_new = c->aoff_alt.p;
      it.aadj_new = c->aadj_alt.p;
      it.aown_new = c->aown_alt.p;
      it.mis = c->mis.p;
      it.cid = c->cid.p;
      it.u = reinterpret_cast<const int32_t*>(ds + off_u[j]);
      it.v = reinterpret_cast<const int32_t*>(ds + off_v[j]);
      it.ins = ds + off_i[j];
      it.m = mm;
      it.max_csr = c->max_csr;
      it.epoch = c->cta_epoch;
      it.win = reinterpret_cast<uint32_t*>(vb + vl.win);
      it.map = reinterpret_cast<int32_t*>(vb + vl.map);
      it.hbits = reinterpret_cast<uint32_t*>(vb + vl.hbits);
      it.sbits = reinterpret_cast<uint32_t*>(vb + vl.sbits);
      it.xbits = reinterpret_cast<uint32_t*>(vb + vl.xbits);
      it.k0 = reinterpret_cast<uint64_t*>(wb + wl.k0);
      it.k1 = reinterpret_cast<uint64_t*>(wb + wl.k1);
      it.ak = reinterpret_cast<uint64_t*>(wb + wl.ak);
      it.v0 = reinterpret_cast<uint32_t*>(wb + wl.v0);
      it.v1 = reinterpret_cast<uint32_t*>(wb + wl.v1);
      it.av = reinterpret_cast<uint32_t*>(wb + wl.av);
      it.prev = reinterpret_cast<int32_t*>(wb + wl.prev);
      it.rows = reinterpret_cast<int32_t*>(wb + wl.rows);
      it.rowcid = reinterpret_cast<int32_t*>(wb + wl.rowcid);
      it.ends = reinterpret_cast<int64_t*>(wb + wl.ends);
      it.acnt = reinterpret_cast<int32_t*>(wb + wl.acnt);
      it.akill = wb + wl.akill;
      it.kp = reinterpret_cast<int64_t*>(wb + wl.kp);
      it.out = E.d_out.p + cta::kOutWords * j;
      table_h[j] = it;
    }

    const int grid = (int)std::min<int64_t>(k, (int64_t)E.sms * o.ctas_per_sm);
    const size_t smem = (size_t)o.block * (8 + 4 * cta::kBuckets);
    auto enqueue = [&] {
      MF_CUDA(cudaMemcpyAsync(ds, E.h_stage, o_b, cudaMemcpyHostToDevice, E.s));
      MF_CUDA(cudaMemsetAsync(E.d_head.p, 0, sizeof(int), E.s));
      MF_K(k_batched<<<grid, o.block, smem, E.s>>>(reinterpret_cast<const cta::Item*>(ds), k, E.d_head.p));
      MF_CUDA(cudaGetLastError());
      MF_CUDA(cudaMemcpyAsync(E.h_out, E.d_out.p, sizeof(int64_t) * cta::kOutWords * (size_t)k,
                              cudaMemcpyDeviceToHost, E.s));
    };
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    MF_CUDA(cudaEventRecord(E.e0, E.s));
    if (o.use_graph) {
      MF_CUDA(cudaStreamBeginCapture(E.s, cudaStreamCaptureModeThreadLocal));
      try {
        enqueue();
      } catch (...) {
        cudaStreamEndCapture(E.s, &graph);
        if (graph) cudaGraphDestroy(graph);
        throw;
      }
      MF_CUDA(cudaStreamEndCapture(E.s, &graph));
      const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
      if (ie != cudaSuccess) {
        cudaGraphDestroy(graph);
        MF_CUDA(ie);
      }
      const cudaError_t le = cudaGraphLaunch(exec, E.s);
      if (le != cudaSuccess) {
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
        MF_CUDA(le);
      }
    } else {
      enqueue();
    }
    MF_CUDA(cudaEventRecord(E.e1, E.s));

    // the batches above the kernel's limits, on their own streams meanwhile
    std::string path_error;
    const int path_status = run_path_items(ctxs, u, v, ins, m, path_items, o.path_threads, &path_error);
    MF_CUDA(cudaSetDevice(device));
    const cudaError_t se = cudaStreamSynchronize(E.s);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    MF_CUDA(se);
    float kms = 0.f;
    MF_CUDA(cudaEventElapsedTime(&kms, E.e0, E.e1));
    stats.kernel_ms = kms;
    // Every item the kernel completed gets its host-side state first; the
    // items that reported an inconsistency are named afterwards, so that no
    // completed context is left with host state that lags its device state.
    std::vector<int64_t> bad_items;
    for (int64_t j = 0; j < k; ++j) {
      const int64_t i = kitems[j].idx;
      mf_ctx* c = ctxs[i];
      const int64_t* out = E.h_out + cta::kOutWords * j;
      if (out[cta::kOutStatus] != 0) {
        bad_items.push_back(i);
        continue;
      }
      if (out[cta::kOutSwapped]) {
        std::swap(c->aoff, c->aoff_alt);
        std::swap(c->aadj, c->aadj_alt);
        std::swap(c->aown, c->aown_alt);
      }
      c->a_total = out[cta::kOutATotal];
      c->max_csr = out[cta::kOutMaxCsr];
      c->cta_epoch = (uint32_t)out[cta::kOutEpoch];
      c->stats = mf_batch_stats{};
      c->stats.packed_total = -1;
      c->stats.row_degree_total = -1;
      c->stats.updates = m[i];
      c->stats.sub_batches = out[cta::kOutSubBatches];
      c->stats.seeds = out[cta::kOutSeeds];
      c->stats.candidates = out[cta::kOutCands];
      c->stats.clusters = out[cta::kOutClusters];
      c->stats.processed_edges = out[cta::kOutProcessed];
      c->stats.exact_sizes = out[cta::kOutExactSizes];
      c->stats.max_csr = c->max_csr;
      c->stats.device_ms = (double)(out[cta::kOutT1] - out[cta::kOutT0]) / 1e6;
    }
    // MISFIT_GB_BATCHED_DEBUG: the kernel's items of over 20 ms, one line each
    static const bool debug = std::getenv("MISFIT_GB_BATCHED_DEBUG") != nullptr;
    if (debug) {
      int64_t t_first = INT64_MAX;
      for (int64_t j = 0; j < k; ++j) t_first = std::min<int64_t>(t_first, E.h_out[cta::kOutWords * j + cta::kOutT0]);
      for (int64_t j = 0; j < k; ++j) {
        const int64_t* out = E.h_out + cta::kOutWords * j;
        const double ms = (double)(out[cta::kOutT1] - out[cta::kOutT0]) / 1e6;
        if (ms < 20.0) continue;
        const mf_ctx* c = ctxs[kitems[j].idx];
        std::fprintf(stderr, "[misfit_gb] batched item: n %d nnz %lld added %lld lines %lld sub-batches %lld "
                     "exact %lld seeds %lld cands %lld start-ms %.2f ms %.2f (kernel %.2f, items %lld)\n",
                     c->n, (long long)c->nnz, (long long)out[cta::kOutATotal], (long long)m[kitems[j].idx],
                     (long long)out[cta::kOutSubBatches], (long long)out[cta::kOutExactSizes],
                     (long long)out[cta::kOutSeeds], (long long)out[cta::kOutCands],
                     (double)(out[cta::kOutT0] - t_first) / 1e6, ms, (double)kms, (long long)k);
      }
    }
    if (!bad_items.empty()) {
      std::string msg = "batched kernel reported an inconsistent state for batch";
      msg += bad_items.size() > 1 ? "es" : "";
      for (size_t b = 0; b < bad_items.size(); ++b) msg += (b ? ", " : " ") + std::to_string(bad_items[b]);
      msg += "; those contexts must be rebuilt (the other batches completed)";
      if (path_status != MF_OK) msg += "; multi-launch path: " + path_error;
      MF_FAIL(MF_ESTATE, msg);
    }
    if (path_status != MF_OK) MF_FAIL(path_status, path_error);
  } else {
    std::string path_error;
    const int r = run_path_items(ctxs, u, v, ins, m, path_items, o.path_threads, &path_error);
    if (r != MF_OK) MF_FAIL(r, path_error);
  }
  stats.wall_ms = host_ms() - t_start;
  if (st) *st = stats;
}

}  // namespace

extern "C" {

int mf_batched_default_opts(mf_batched_opts* out) {
  if (!out) return MF_EINVAL;
  *out = default_opts();
  return MF_OK;
}

int mf_apply_batches(mf_ctx* const* ctxs, const int32_t* const* u, const int32_t* const* v,
                     const uint8_t* const* ins, const int64_t* m, int64_t count, const mf_batched_opts* opts,
                     mf_batched_stats* stats) {
  struct ClearStream {
    ~ClearStream() { mf::g_alloc_stream = nullptr; }
  } clear;
  try {
    mf::set_error("");
    apply_batches(ctxs, u, v, ins, m, count, opts ? *opts : default_opts(), stats);
    return MF_OK;
  } catch (const Failure& e) {
    return e.status;
  } catch (const std::bad_alloc&) {
    mf::set_error("host allocation failed");
    return MF_ENOMEM;
  } catch (const std::exception& e) {
    mf::set_error(e.what());
    return MF_EINVAL;
  }
}

}  // extern "C"
