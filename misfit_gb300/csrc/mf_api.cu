// mf_api.cu -- extern "C" entry points of libmisfit_gb and the host-side file
// formats (.egr, MIS file, batch folder).
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "mf_internal.cuh"

namespace mf {

namespace {
thread_local std::string g_error;
}

std::atomic<long long> g_launches{0};
std::atomic<long long> g_allocs{0};
thread_local cudaStream_t g_alloc_stream = nullptr;

namespace {
struct KTimes {
  std::mutex mu;
  std::map<std::string, std::pair<long long, double>> by_name;
  ~KTimes() {
    if (by_name.empty()) return;
    std::vector<std::pair<double, std::string>> rows;
    double total = 0.0;
    for (const auto& kv : by_name) {
      rows.emplace_back(kv.second.second, kv.first);
      total += kv.second.second;
    }
    std::sort(rows.rbegin(), rows.rend());
    std::fprintf(stderr, "[misfit_gb] per-kernel host-timed ms (synchronised launches), total %.3f\n", total);
    for (const auto& r : rows)
      std::fprintf(stderr, "  %-28s %9lld %12.3f %6.1f%%\n", r.second.c_str(), by_name[r.second].first, r.first,
                   total > 0 ? 100.0 * r.first / total : 0.0);
  }
};
KTimes g_ktimes;

double ktime_now() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
}  // namespace

bool pdl_on() {
  static const bool on = [] {
    const char* e = std::getenv("MISFIT_GB_PDL");
    return !(e != nullptr && std::strcmp(e, "0") == 0);
  }();
  return on;
}

bool ktime_on() {
  static const bool on = [] {
    const char* e = std::getenv("MISFIT_GB_KTIME");
    return e != nullptr && std::strcmp(e, "1") == 0;
  }();
  return on;
}

double ktime_begin() {
  cudaDeviceSynchronize();
  return ktime_now();
}

void ktime_end(const char* launch_text, double t0) {
  cudaDeviceSynchronize();
  const double dt = ktime_now() - t0;
  std::string name(launch_text);
  const size_t cut = name.find("<<<");
  if (cut != std::string::npos) name.resize(cut);
  while (!name.empty() && (name.back() == ' ' || name.back() == '\n')) name.pop_back();
  std::lock_guard<std::mutex> lock(g_ktimes.mu);
  auto& e = g_ktimes.by_name[name];
  e.first += 1;
  e.second += dt;
}

const char* const kStageNames[kStCount] = {"overlay", "split",  "seeds", "hop1",  "sizes", "cluster_read",
                                           "cluster_write", "assign", "repair", "clear", "exact", "repair_big",
                                           "push_hop", "cluster_read_need", "pull"};

void set_error(const std::string& msg) { g_error = msg; }

void bind_device(const mf_ctx* c) {
  MF_CUDA(cudaSetDevice(c->device));
  g_alloc_stream = c->stream;
}

double now_ms_host() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
const char* get_error() { return g_error.c_str(); }

}  // namespace mf

namespace {

using mf::Failure;

// Runs an entry point: exceptions become status codes, and the thread's
// allocation stream (set by bind) does not outlive the call.
template <class F>
int guarded(F&& f) {
  struct ClearStream {
    ~ClearStream() { mf::g_alloc_stream = nullptr; }
  } clear;
  try {
    mf::set_error("");
    f();
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

void need(bool cond, int status, const char* msg) {
  if (!cond) MF_FAIL(status, msg);
}

void release_all(mf_ctx* c) {
  mf::release_device_state(c);
  if (c->h_counters) cudaFreeHost(c->h_counters);
  c->h_counters = nullptr;
  for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
  c->ev_pool.clear();
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream_b) {
    cudaStreamSynchronize(c->stream_b);
    cudaStreamDestroy(c->stream_b);
  }
  c->stream_b = nullptr;
  if (c->ev_a) cudaEventDestroy(c->ev_a);
  if (c->ev_b) cudaEventDestroy(c->ev_b);
  if (c->stream) cudaStreamDestroy(c->stream);
  c->stream = nullptr;
}

mf_ctx* new_ctx(int gpu) {
  int count = 0;
  MF_CUDA(cudaGetDeviceCount(&count));
  if (gpu < 0 || gpu >= count) MF_FAIL(MF_EINVAL, "gpu id out of range");
  MF_CUDA(cudaSetDevice(gpu));
  mf_ctx* c = new mf_ctx();
  c->device = gpu;
  try {
    mf::noalloc_refresh(gpu);
    if (const char* e = std::getenv("MISFIT_GB_BIG_THRESHOLD")) c->tune.big_threshold = std::max<long long>(0, std::atoll(e));
    if (const char* e = std::getenv("MISFIT_GB_EXACT_CAPS")) {
      long long dn = 0, pr = 0;
      if (std::sscanf(e, "%lld,%lld", &dn, &pr) == 2) {
        c->exact_cap_dense = std::max<long long>(0, dn);
        c->exact_cap_pairs = pr > 0 ? std::max<long long>(4096, pr) : 0;
      }
    }
    MF_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    mf::g_alloc_stream = c->stream;
    // keep freed stream-ordered memory in this process's pool for reuse
    cudaMemPool_t mp;
    if (cudaDeviceGetDefaultMemPool(&mp, gpu) == cudaSuccess) {
      uint64_t keep = ~0ull;
      cudaMemPoolSetAttribute(mp, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    MF_CUDA(cudaEventCreate(&c->ev0));
    MF_CUDA(cudaEventCreate(&c->ev1));
    MF_CUDA(cudaStreamCreateWithFlags(&c->stream_b, cudaStreamNonBlocking));
    MF_CUDA(cudaEventCreateWithFlags(&c->ev_a, cudaEventDisableTiming));
    MF_CUDA(cudaEventCreateWithFlags(&c->ev_b, cudaEventDisableTiming));
    mf::note_alloc();
    MF_CUDA(cudaMallocHost(&c->h_counters, sizeof(int64_t) * 64));
    c->counters.reserve(64);
  } catch (...) {
    release_all(c);
    delete c;
    throw;
  }
  return c;
}

void quiesce(const mf_ctx* c);

// Every entry point that touches a context first waits until the context's
// pipelined batches (mf_apply_batch_async) have finished running, then binds
// its device and stream to the calling thread.
void bind(const mf_ctx* c) {
  quiesce(c);
  MF_CUDA(cudaSetDevice(c->device));
  mf::g_alloc_stream = c->stream;
}

// Inputs of a batch are already in c->bu / c->bv / c->bins.
void run_batch(mf_ctx* c, int64_t m) {
  cudaStream_t s = c->stream;
  c->stats = mf_batch_stats{};
  c->stats.updates = m;
  c->stats.packed_total = -1;
  c->stats.row_degree_total = -1;
  c->traces.clear();
  c->work.reserve(2 * mf::kStCount + 8);
  c->touched_total = 0;
  c->pull_runs = 0;
  MF_CUDA(cudaMemsetAsync(c->work.p, 0, sizeof(unsigned long long) * (2 * mf::kStCount + 8), s));
  MF_CUDA(cudaEventRecord(c->ev0, s));
  if (m > 0) {
    {
      mf::StageScope sc(c, mf::kStOverlay);
      mf::apply_overlay(c, m);
    }
    mf::process_batch(c, m);
    if (c->exact) mf::exact_fixup(c);
  }
  MF_CUDA(cudaEventRecord(c->ev1, s));
  MF_CUDA(cudaEventSynchronize(c->ev1));
  float ms = 0.f;
  MF_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  c->stats.device_ms = ms;
  c->stats.max_csr = c->max_csr;
  for (const auto& mk : c->ev_marks) {
    float t = 0.f;
    if (cudaEventElapsedTime(&t, c->ev_pool[mk.second], c->ev_pool[mk.second + 1]) == cudaSuccess) {
      c->stage_ms[mk.first] += t;
      c->stage_calls[mk.first] += 1;
    }
  }
  c->ev_marks.clear();
  c->ev_used = 0;
  if (c->pull_runs > 0 && c->n >= (1 << 20)) {
    // row entries the pull read per vertex, for the next batch's pull-or-push choice
    unsigned long long visited = 0;
    MF_CUDA(cudaMemcpy(&visited, c->work.p + 2 * mf::kStCount + 2, sizeof(visited), cudaMemcpyDeviceToHost));
    c->pull_visit_ratio = (double)visited / ((double)c->pull_runs * (double)c->n);
  }
  static const bool debug = std::getenv("MISFIT_GB_DEBUG") != nullptr;
  if (debug || c->profile) {
    unsigned long long w[2 * mf::kStCount + 8];
    MF_CUDA(cudaMemcpy(w, c->work.p, sizeof(w), cudaMemcpyDeviceToHost));
    const unsigned long long* x = w + 2 * mf::kStCount;
    // 4 B row entry + 8 B state read and cid write per pushed element (x[3]:
    // the candidate rows of the sub-batches that pushed); x[2] the row
    // entries read by the sub-batches that pulled
    c->stage_bytes[mf::kStPush] += 12.0 * (double)(x[0] + x[3]);
    c->stage_bytes[mf::kStPull] += 4.0 * (double)x[2];
    c->stage_bytes[mf::kStPushHop] += 12.0 * (double)x[1];
    if (debug) {
      std::fprintf(stderr,
                   "[misfit_gb] batch: push elements seed %llu hop %llu cand %llu; pull entries %llu in %lld of %lld "
                   "sub-batches\n",
                   x[0], x[1], x[3], x[2], (long long)c->pull_runs, (long long)c->stats.sub_batches);
      std::fprintf(stderr, "[misfit_gb] first hits: calls %lld rows %lld warp-level %lld chunk-level %lld chunks %lld\n",
                   (long long)c->dbg_first[0], (long long)c->dbg_first[1], (long long)c->dbg_first[2],
                   (long long)c->dbg_first[3], (long long)c->dbg_first[4]);
      for (auto& v : c->dbg_first) v = 0;
    }
  }
  if (c->profile) {
    // algorithmic bytes per stage from the device work counters:
    //   hop1: 4 B row entry + 4 B bitmap OR per element
    //   push: 4 B row entry + 8 B max read-modify-write per element, plus
    //         the cluster-id resolve pass: 4 B tag + 4 B id per vertex
    unsigned long long w[2 * mf::kStCount];
    MF_CUDA(cudaMemcpy(w, c->work.p, sizeof(w), cudaMemcpyDeviceToHost));
    c->stage_bytes[mf::kStHop1] += 8.0 * (double)w[2 * mf::kStHop1];
    c->stage_bytes[mf::kStPush] += 8.0 * (double)c->touched_total;
  }
}

__global__ void k_validate(const int32_t* u, const int32_t* v, int64_t m, int32_t n, unsigned long long* bad) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const int32_t a = u[i], b = v[i];
  if (a < 0 || a >= n || b < 0 || b >= n || a == b) atomicAdd(bad, 1ull);
}

void stage_inputs(mf_ctx* c, const int32_t* u, const int32_t* v, const uint8_t* ins, int64_t m,
                  cudaMemcpyKind kind) {
  cudaStream_t s = c->stream;
  c->bu.reserve(m);
  c->bv.reserve(m);
  c->bins.reserve(m);
  if (m == 0) return;
  MF_CUDA(cudaMemcpyAsync(c->bu.p, u, sizeof(int32_t) * (size_t)m, kind, s));
  MF_CUDA(cudaMemcpyAsync(c->bv.p, v, sizeof(int32_t) * (size_t)m, kind, s));
  if (ins) MF_CUDA(cudaMemcpyAsync(c->bins.p, ins, (size_t)m, kind, s));
  MF_CUDA(cudaMemsetAsync(c->counters.p, 0, sizeof(int64_t), s));
  MF_K(k_validate<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(c->bu.p, c->bv.p, m, c->n,
                                                          reinterpret_cast<unsigned long long*>(c->counters.p)));
  MF_CUDA(cudaMemcpyAsync(c->h_counters, c->counters.p, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  MF_CUDA(cudaStreamSynchronize(s));
  if (c->h_counters[0] != 0) MF_FAIL(MF_EINVAL, "update endpoints must be distinct vertex ids in [0, n)");
}

// ---- the pipelined engine ---------------------------------------------------------
//
// The reference's misfit_async launches batch i+1 before it collects batch i
// (src/misfit_async/misfit_async.cu:826-876): launchBatch does the host-side
// work and queues the device work, syncAndCollect waits for it.  Here every
// stage of a batch runs on the device and the host only orchestrates, so the
// orchestration itself moves off the caller's thread: mf_apply_batch_async
// queues the batch for the context's worker thread and returns at once, the
// worker runs the queued batches one after another on the context's stream
// (so the results are those of mf_apply_batch in the same order), and
// mf_collect waits for the oldest one.  The caller's thread is free between
// the calls, as the reference's host thread is free while its GPU works.

}  // namespace

namespace mf {
struct AsyncJob {
  const int32_t* u = nullptr;
  const int32_t* v = nullptr;
  const uint8_t* ins = nullptr;
  int64_t m = 0;
  bool done = false;
  int status = MF_OK;
  std::string error;
  mf_batch_stats stats{};
};

struct AsyncQueue {
  std::mutex mu;
  std::condition_variable cv;
  std::deque<std::shared_ptr<AsyncJob>> todo;     // queued, not started
  std::deque<std::shared_ptr<AsyncJob>> issued;   // every uncollected batch, oldest first
  bool busy = false;                              // the worker is running a batch
  bool stop = false;
  std::thread worker;
};
}  // namespace mf

namespace {

void async_worker(mf_ctx* c) {
  mf::AsyncQueue& q = *c->aq;
  for (;;) {
    std::shared_ptr<mf::AsyncJob> j;
    {
      std::unique_lock<std::mutex> lk(q.mu);
      q.cv.wait(lk, [&] { return q.stop || !q.todo.empty(); });
      if (q.todo.empty()) return;
      j = q.todo.front();
      q.todo.pop_front();
      q.busy = true;
    }
    const int st = guarded([&] {
      mf::bind_device(c);
      stage_inputs(c, j->u, j->v, j->ins, j->m, cudaMemcpyHostToDevice);
      run_batch(c, j->m);
    });
    {
      std::lock_guard<std::mutex> lk(q.mu);
      j->status = st;
      if (st != MF_OK) j->error = mf::get_error();
      j->stats = c->stats;
      j->done = true;
      q.busy = false;
    }
    q.cv.notify_all();
  }
}

void enqueue_async(mf_ctx* c, const int32_t* u, const int32_t* v, const uint8_t* ins, int64_t m) {
  if (!c->aq) {
    c->aq = new mf::AsyncQueue();
    c->aq->worker = std::thread(async_worker, c);
  }
  auto j = std::make_shared<mf::AsyncJob>();
  j->u = u;
  j->v = v;
  j->ins = ins;
  j->m = m;
  {
    std::lock_guard<std::mutex> lk(c->aq->mu);
    c->aq->todo.push_back(j);
    c->aq->issued.push_back(j);
    c->pending = true;
  }
  c->aq->cv.notify_all();
}

// Waits for the oldest uncollected batch and removes it; null if none.
std::shared_ptr<mf::AsyncJob> collect_oldest(mf_ctx* c) {
  if (!c->aq) return nullptr;
  std::unique_lock<std::mutex> lk(c->aq->mu);
  if (c->aq->issued.empty()) return nullptr;
  std::shared_ptr<mf::AsyncJob> j = c->aq->issued.front();
  c->aq->cv.wait(lk, [&] { return j->done; });
  c->aq->issued.pop_front();
  c->pending = !c->aq->issued.empty();
  return j;
}

// Waits until the worker has nothing queued or running (results stay
// uncollected).
void quiesce(const mf_ctx* c) {
  mf::AsyncQueue* q = c->aq;
  if (!q) return;
  std::unique_lock<std::mutex> lk(q->mu);
  q->cv.wait(lk, [&] { return q->todo.empty() && !q->busy; });
}

void stop_async(mf_ctx* c) {
  if (!c->aq) return;
  quiesce(c);
  {
    std::lock_guard<std::mutex> lk(c->aq->mu);
    c->aq->stop = true;
  }
  c->aq->cv.notify_all();
  if (c->aq->worker.joinable()) c->aq->worker.join();
  delete c->aq;
  c->aq = nullptr;
  c->pending = false;
}

// ---- .egr ----------------------------------------------------------------------

struct EgrHeader {
  int32_t n = 0;
  uint64_t edges = 0;
  bool wide = false;
  size_t header_bytes = 0;
};

EgrHeader read_egr_header(FILE* f, const char* path, size_t file_size) {
  EgrHeader h;
  int32_t e32 = 0;
  need(std::fread(&h.n, 4, 1, f) == 1 && std::fread(&e32, 4, 1, f) == 1, MF_EFORMAT,
       "failed to read the .egr header");
  if (e32 == -1) {
    need(std::fread(&h.edges, 8, 1, f) == 1, MF_EFORMAT, "failed to read the 64-bit edge count");
    h.wide = true;
    h.header_bytes = 16;
  } else {
    need(h.n >= 1 && e32 >= 0, MF_EFORMAT, "invalid .egr header (nodes < 1 or edges < 0)");
    h.edges = (uint64_t)e32;
    h.header_bytes = 8;
  }
  need(h.n >= 0, MF_EFORMAT, "invalid .egr header (negative node count)");
  const size_t need_bytes = h.header_bytes + ((size_t)h.n + 1) * (h.wide ? 8 : 4) + (size_t)h.edges * 4;
  if (need_bytes > file_size)
    MF_FAIL(MF_EFORMAT, std::string("truncated .egr file ") + path);
  return h;
}

mf_ctx* open_egr(const char* path, int gpu) {
  FILE* f = std::fopen(path, "rb");
  if (!f) MF_FAIL(MF_EIO, std::string("could not open ") + path);
  struct stat st;
  if (fstat(fileno(f), &st) != 0) {
    std::fclose(f);
    MF_FAIL(MF_EIO, std::string("fstat failed for ") + path);
  }
  EgrHeader h;
  try {
    h = read_egr_header(f, path, (size_t)st.st_size);
  } catch (...) {
    std::fclose(f);
    throw;
  }
  std::vector<int64_t> nindex((size_t)h.n + 1);
  bool ok;
  if (h.wide) {
    ok = std::fread(nindex.data(), 8, nindex.size(), f) == nindex.size();
  } else {
    std::vector<int32_t> t(nindex.size());
    ok = std::fread(t.data(), 4, t.size(), f) == t.size();
    for (size_t i = 0; ok && i < t.size(); ++i) nindex[i] = t[i];
  }
  if (!ok) {
    std::fclose(f);
    MF_FAIL(MF_EFORMAT, "failed to read nindex");
  }
  mf_ctx* c = nullptr;
  try {
    c = new_ctx(gpu);
    c->header_edges = h.edges;
    // nlist: read through two pinned chunks, copied asynchronously.
    const int64_t nnz = (int64_t)h.edges;
    c->nlist.reserve(nnz + mf::kNlistPad);
    const size_t chunk = (size_t)64 << 20;
    void* pin[2] = {nullptr, nullptr};
    cudaEvent_t done[2];
    mf::note_alloc();
    MF_CUDA(cudaMallocHost(&pin[0], chunk));
    mf::note_alloc();
    MF_CUDA(cudaMallocHost(&pin[1], chunk));
    MF_CUDA(cudaEventCreate(&done[0]));
    MF_CUDA(cudaEventCreate(&done[1]));
    size_t off = 0, total = (size_t)nnz * 4;
    int slot = 0;
    bool rd_ok = true;
    while (off < total) {
      const size_t len = std::min(chunk, total - off);
      MF_CUDA(cudaEventSynchronize(done[slot]));
      if (std::fread(pin[slot], 1, len, f) != len) { rd_ok = false; break; }
      MF_CUDA(cudaMemcpyAsync((char*)c->nlist.p + off, pin[slot], len, cudaMemcpyHostToDevice, c->stream));
      MF_CUDA(cudaEventRecord(done[slot], c->stream));
      off += len;
      slot ^= 1;
    }
    MF_CUDA(cudaStreamSynchronize(c->stream));
    cudaFreeHost(pin[0]);
    cudaFreeHost(pin[1]);
    cudaEventDestroy(done[0]);
    cudaEventDestroy(done[1]);
    std::fclose(f);
    f = nullptr;
    if (!rd_ok) MF_FAIL(MF_EFORMAT, "failed to read nlist");
    mf::upload_base(c, h.n, nindex.data(), nullptr, nnz);
  } catch (...) {
    if (f) std::fclose(f);
    if (c) {
      release_all(c);
      delete c;
    }
    throw;
  }
  return c;
}

int write_egr_int64(const std::string& out_path, int32_t n, const std::vector<int64_t>& nindex,
                    const std::vector<int32_t>& nlist) {
  const std::string tmp = out_path + ".tmp." + std::to_string(getpid());
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) MF_FAIL(MF_EIO, "could not open " + tmp + " for writing");
  const int32_t sentinel = -1;
  const uint64_t total = (uint64_t)nlist.size();
  bool ok = std::fwrite(&n, 4, 1, f) == 1 && std::fwrite(&sentinel, 4, 1, f) == 1 &&
            std::fwrite(&total, 8, 1, f) == 1 &&
            std::fwrite(nindex.data(), 8, nindex.size(), f) == nindex.size() &&
            (nlist.empty() || std::fwrite(nlist.data(), 4, nlist.size(), f) == nlist.size());
  if (ok) ok = std::fflush(f) == 0 && fsync(fileno(f)) == 0;
  std::fclose(f);
  if (!ok) {
    std::remove(tmp.c_str());
    MF_FAIL(MF_EIO, "failed writing " + tmp);
  }
  // Fault injection for the crash-safety test: end the process after the
  // temporary file is complete and flushed, before it replaces out_path --
  // the moment core/flash_compactor.h:88-104 guards against.
  if (const char* x = std::getenv("MISFIT_GB_EXIT_BEFORE_RENAME"))
    if (std::strcmp(x, "1") == 0) std::_Exit(86);
  if (std::rename(tmp.c_str(), out_path.c_str()) != 0) MF_FAIL(MF_EIO, "rename " + tmp + " -> " + out_path + " failed");
  std::string dir = ".";
  const size_t slash = out_path.find_last_of('/');
  if (slash != std::string::npos) dir = out_path.substr(0, slash);
  const int fd = ::open(dir.c_str(), O_RDONLY);
  if (fd >= 0) {
    fsync(fd);
    ::close(fd);
  }
  return 0;
}

}  // namespace

extern "C" {

int mf_version(void) { return 10200; }

const char* mf_status_string(int status) {
  switch (status) {
    case MF_OK: return "ok";
    case MF_EINVAL: return "invalid argument";
    case MF_EIO: return "i/o error";
    case MF_EFORMAT: return "malformed input file";
    case MF_ECUDA: return "CUDA error";
    case MF_ENOMEM: return "out of memory";
    case MF_ESTATE: return "inconsistent graph state";
    case MF_ELIMIT: return "request beyond a fixed limit";
    default: return "unknown status";
  }
}

const char* mf_last_error(void) { return mf::get_error(); }

int mf_open_egr(const char* path, int gpu, mf_ctx** out) {
  return guarded([&] {
    need(path && out, MF_EINVAL, "null argument");
    *out = nullptr;
    *out = open_egr(path, gpu);
  });
}

int mf_open_csr(int32_t n, const int64_t* nindex, const int32_t* nlist, int gpu, mf_ctx** out) {
  return guarded([&] {
    need(out && nindex && n >= 0, MF_EINVAL, "bad CSR arguments");
    *out = nullptr;
    const int64_t nnz = nindex[n];
    need(nnz >= 0 && (nnz == 0 || nlist), MF_EINVAL, "bad CSR arguments");
    mf_ctx* c = new_ctx(gpu);
    try {
      c->header_edges = (uint64_t)nnz;
      mf::upload_base(c, n, nindex, nlist, nnz);
    } catch (...) {
      release_all(c);
      delete c;
      throw;
    }
    *out = c;
  });
}

int mf_close(mf_ctx* c) {
  if (!c) return MF_OK;
  stop_async(c);
  return guarded([&] {
    cudaSetDevice(c->device);
    mf::g_alloc_stream = c->stream;
    if (c->stream) cudaStreamSynchronize(c->stream);
    release_all(c);
    delete c;
  });
}

int mf_num_nodes(const mf_ctx* c, int32_t* n) {
  return guarded([&] {
    need(c && n, MF_EINVAL, "null argument");
    *n = c->n;
  });
}

int mf_num_base_entries(const mf_ctx* c, int64_t* e) {
  return guarded([&] {
    need(c && e, MF_EINVAL, "null argument");
    *e = c->nnz;
  });
}

int mf_set_mis(mf_ctx* c, const uint8_t* mis, int64_t n) {
  return guarded([&] {
    need(c && mis && n == c->n, MF_EINVAL, "membership vector must have n entries");
    bind(c);
    if (n > 0) {
      std::vector<uint8_t> norm((size_t)n);
      for (int64_t i = 0; i < n; ++i) norm[(size_t)i] = mis[i] ? 1 : 0;
      MF_CUDA(cudaMemcpyAsync(c->mis.p, norm.data(), (size_t)n, cudaMemcpyHostToDevice, c->stream));
      MF_CUDA(cudaMemsetAsync(c->cid.p, 0xFF, sizeof(int32_t) * (size_t)n, c->stream));
      MF_CUDA(cudaStreamSynchronize(c->stream));
    }
    MF_CUDA(cudaStreamSynchronize(c->stream));
  });
}

int mf_get_mis(mf_ctx* c, uint8_t* out, int64_t n) {
  return guarded([&] {
    need(c && out && n == c->n, MF_EINVAL, "output must have n entries");
    bind(c);
    if (n > 0) MF_CUDA(cudaMemcpyAsync(out, c->mis.p, (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    MF_CUDA(cudaStreamSynchronize(c->stream));
  });
}

int mf_mis_size(mf_ctx* c, int64_t* count) {
  return guarded([&] {
    need(c && count, MF_EINVAL, "null argument");
    bind(c);
    std::vector<uint8_t> h((size_t)c->n);
    if (c->n > 0) MF_CUDA(cudaMemcpyAsync(h.data(), c->mis.p, (size_t)c->n, cudaMemcpyDeviceToHost, c->stream));
    MF_CUDA(cudaStreamSynchronize(c->stream));
    int64_t k = 0;
    for (uint8_t b : h) k += b != 0;
    *count = k;
  });
}

int mf_greedy_mis(mf_ctx* c, uint8_t* out, int64_t n) {
  return guarded([&] {
    need(c && out && n == c->n, MF_EINVAL, "output must have n entries");
    bind(c);
    mf::DBuf<uint8_t> d;
    d.reserve(std::max<int64_t>(n, 1));
    mf::greedy_mis(c, d.p);
    if (n > 0) MF_CUDA(cudaMemcpy(out, d.p, (size_t)n, cudaMemcpyDeviceToHost));
    d.release();
  });
}

int mf_flag_updates(mf_ctx* c, const int32_t* u, const int32_t* v, int64_t m, uint8_t* ins_out) {
  return guarded([&] {
    need(c && m >= 0 && (m == 0 || (u && v && ins_out)), MF_EINVAL, "bad arguments");
    bind(c);
    stage_inputs(c, u, v, nullptr, m, cudaMemcpyHostToDevice);
    mf::flag_updates(c, m);
    if (m > 0) MF_CUDA(cudaMemcpyAsync(ins_out, c->bins.p, (size_t)m, cudaMemcpyDeviceToHost, c->stream));
    MF_CUDA(cudaStreamSynchronize(c->stream));
  });
}

int mf_flag_updates_noalloc(mf_ctx* c, const int32_t* u, const int32_t* v, int64_t m, uint8_t* ins_out) {
  return guarded([&] {
    need(c && m >= 0 && (m == 0 || (u && v && ins_out)), MF_EINVAL, "bad arguments");
    bind(c);
    mf::flag_updates_noalloc(c, u, v, m, ins_out);
  });
}

int mf_apply_batch(mf_ctx* c, const int32_t* u, const int32_t* v, const uint8_t* ins, int64_t m) {
  return guarded([&] {
    need(c && m >= 0 && (m == 0 || (u && v && ins)), MF_EINVAL, "bad arguments");
    need(!c->pending, MF_EINVAL, "asynchronous batches are pending; collect them (mf_collect / mf_sync) first");
    bind(c);
    stage_inputs(c, u, v, ins, m, cudaMemcpyHostToDevice);
    run_batch(c, m);
  });
}

int mf_apply_batch_device(mf_ctx* c, const int32_t* d_u, const int32_t* d_v, const uint8_t* d_ins, int64_t m) {
  return guarded([&] {
    need(c && m >= 0 && (m == 0 || (d_u && d_v && d_ins)), MF_EINVAL, "bad arguments");
    need(!c->pending, MF_EINVAL, "asynchronous batches are pending; collect them (mf_collect / mf_sync) first");
    bind(c);
    stage_inputs(c, d_u, d_v, d_ins, m, cudaMemcpyDeviceToDevice);
    run_batch(c, m);
  });
}

int mf_apply_batch_async(mf_ctx* c, const int32_t* u, const int32_t* v, const uint8_t* ins, int64_t m) {
  return guarded([&] {
    need(c && m >= 0 && (m == 0 || (u && v && ins)), MF_EINVAL, "bad arguments");
    enqueue_async(c, u, v, ins, m);
  });
}

int mf_collect(mf_ctx* c, mf_batch_stats* out) {
  if (!c) {
    mf::set_error("null context");
    return MF_EINVAL;
  }
  std::shared_ptr<mf::AsyncJob> j = collect_oldest(c);
  if (!j) {
    mf::set_error("no asynchronous batch to collect");
    return MF_EINVAL;
  }
  if (out) *out = j->stats;
  mf::set_error(j->error);
  return j->status;
}

int mf_sync(mf_ctx* c) {
  if (!c) {
    mf::set_error("null context");
    return MF_EINVAL;
  }
  int first = MF_OK;
  std::string err;
  while (std::shared_ptr<mf::AsyncJob> j = collect_oldest(c)) {
    if (first == MF_OK && j->status != MF_OK) {
      first = j->status;
      err = j->error;
    }
  }
  const int st = guarded([&] {
    bind(c);
    MF_CUDA(cudaStreamSynchronize(c->stream));
  });
  if (first != MF_OK) {
    mf::set_error(err);
    return first;
  }
  return st;
}

int mf_get_tuning(mf_ctx* c, mf_tuning* out) {
  return guarded([&] {
    need(c && out, MF_EINVAL, "null argument");
    *out = c->tune;
  });
}

int mf_set_tuning(mf_ctx* c, const mf_tuning* in) {
  return guarded([&] {
    need(c && in, MF_EINVAL, "null argument");
    need(in->pull_long >= 32 && in->heavy_min >= 64 && in->big_threshold >= 0 && in->first_bound >= 8 &&
             in->first_bound <= ((int64_t)1 << 20) && in->cand_push >= 0 && in->cand_push <= 2 &&
             in->pull_sizes >= 0 && in->pull_sizes <= 2,
         MF_EINVAL, "tuning out of range (pull_long >= 32, heavy_min >= 64, big_threshold >= 0, "
                    "8 <= first_bound <= 2^20, cand_push 0..2, pull_sizes 0..2)");
    bind(c);
    c->tune = *in;
  });
}

int mf_last_batch_stats(mf_ctx* c, mf_batch_stats* out) {
  return guarded([&] {
    need(c && out, MF_EINVAL, "null argument");
    *out = c->stats;
  });
}

int mf_get_row(mf_ctx* c, int32_t x, int32_t* out, int64_t cap, int64_t* len) {
  return guarded([&] {
    need(c && len && x >= 0 && x < c->n && (cap == 0 || out), MF_EINVAL, "bad arguments");
    bind(c);
    int64_t nb[2], ab[2];
    int32_t dead = 0;
    MF_CUDA(cudaMemcpy(nb, c->nindex.p + x, sizeof(nb), cudaMemcpyDeviceToHost));
    MF_CUDA(cudaMemcpy(ab, c->aoff.p + x, sizeof(ab), cudaMemcpyDeviceToHost));
    MF_CUDA(cudaMemcpy(&dead, c->dead.p + x, sizeof(dead), cudaMemcpyDeviceToHost));
    std::vector<int32_t> base((size_t)(nb[1] - nb[0]));
    if (!base.empty())
      MF_CUDA(cudaMemcpy(base.data(), c->nlist.p + nb[0], sizeof(int32_t) * base.size(), cudaMemcpyDeviceToHost));
    std::vector<int32_t> row;
    if (dead == 0) {
      row = base;
    } else {
      const int64_t w0 = nb[0] >> 5, w1 = (nb[1] + 31) >> 5;
      std::vector<uint32_t> bits((size_t)(w1 - w0));
      MF_CUDA(cudaMemcpy(bits.data(), c->live.p + w0, sizeof(uint32_t) * bits.size(), cudaMemcpyDeviceToHost));
      for (int64_t k = nb[0]; k < nb[1]; ++k)
        if ((bits[(size_t)((k >> 5) - w0)] >> (k & 31)) & 1u) row.push_back(base[(size_t)(k - nb[0])]);
    }
    std::vector<int32_t> add((size_t)(ab[1] - ab[0]));
    if (!add.empty())
      MF_CUDA(cudaMemcpy(add.data(), c->aadj.p + ab[0], sizeof(int32_t) * add.size(), cudaMemcpyDeviceToHost));
    row.insert(row.end(), add.begin(), add.end());
    *len = (int64_t)row.size();
    for (int64_t i = 0; i < (int64_t)row.size() && i < cap; ++i) out[i] = row[(size_t)i];
  });
}

int mf_get_degrees(mf_ctx* c, int32_t* out, int64_t n) {
  return guarded([&] {
    need(c && out && n == c->n, MF_EINVAL, "output must have n entries");
    bind(c);
    if (n > 0) MF_CUDA(cudaMemcpy(out, c->deg.p, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost));
  });
}

int mf_get_cluster_ids(mf_ctx* c, int32_t* out, int64_t n) {
  return guarded([&] {
    need(c && out && n == c->n, MF_EINVAL, "output must have n entries");
    bind(c);
    MF_CUDA(cudaStreamSynchronize(c->stream));
    if (n > 0) MF_CUDA(cudaMemcpy(out, c->cid.p, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost));
  });
}

int mf_is_adjacent(mf_ctx* c, int32_t u, int32_t v, int* adjacent) {
  return guarded([&] {
    need(c && adjacent && u >= 0 && v >= 0 && u < c->n && v < c->n, MF_EINVAL, "bad arguments");
    bind(c);
    uint8_t ins = 0;
    stage_inputs(c, &u, &v, nullptr, 1, cudaMemcpyHostToDevice);
    mf::flag_updates(c, 1);
    MF_CUDA(cudaMemcpyAsync(&ins, c->bins.p, 1, cudaMemcpyDeviceToHost, c->stream));
    MF_CUDA(cudaStreamSynchronize(c->stream));
    *adjacent = ins ? 0 : 1;
  });
}

int mf_get_max_csr(mf_ctx* c, int64_t* value) {
  return guarded([&] {
    need(c && value, MF_EINVAL, "null argument");
    *value = c->max_csr;
  });
}

int mf_set_max_csr(mf_ctx* c, int64_t value) {
  return guarded([&] {
    need(c && value > 0, MF_EINVAL, "bad arguments");
    c->max_csr = value;
  });
}

int mf_set_exact(mf_ctx* c, int on) {
  return guarded([&] {
    need(c != nullptr, MF_EINVAL, "null context");
    c->exact = on != 0;
  });
}

int mf_check_mis(mf_ctx* c, int64_t* violations, int64_t* uncovered) {
  return guarded([&] {
    need(c && violations && uncovered, MF_EINVAL, "null argument");
    bind(c);
    mf::check_mis(c, violations, uncovered);
  });
}

int mf_compact(mf_ctx* c, const char* out_path, int rebase) {
  return guarded([&] {
    need(c && out_path, MF_EINVAL, "null argument");
    bind(c);
    std::vector<int64_t> ni;
    std::vector<int32_t> nl;
    mf::compact_graph(c, ni, nl);
    write_egr_int64(out_path, c->n, ni, nl);
    if (rebase) mf::rebase(c);
  });
}

int mf_read_mis_file(const char* path, int32_t n, uint8_t* out, int64_t* lines) {
  return guarded([&] {
    need(path && n >= 0 && (n == 0 || out) && lines, MF_EINVAL, "bad arguments");
    std::memset(out, 0, (size_t)n);
    *lines = 0;
    std::ifstream in(path);
    if (!in.is_open()) return;  // the reference starts from an empty set
    std::string line;
    int64_t lineno = 0;
    while (std::getline(in, line)) {
      ++lineno;
      int id;
      try {
        id = std::stoi(line) - 1;
      } catch (...) {
        MF_FAIL(MF_EFORMAT, std::string(path) + ":" + std::to_string(lineno) + ": not an integer");
      }
      if (id >= 0 && id < n) {
        out[id] = 1;
        ++*lines;
      }
    }
  });
}

int mf_write_mis_file(const char* path, const uint8_t* mis, int32_t n) {
  return guarded([&] {
    need(path && n >= 0 && (n == 0 || mis), MF_EINVAL, "bad arguments");
    std::ofstream out(path);
    if (!out.is_open()) MF_FAIL(MF_EIO, std::string("could not open ") + path);
    std::string buf;
    buf.reserve(1 << 20);
    for (int32_t i = 0; i < n; ++i) {
      if (!mis[i]) continue;
      buf += std::to_string(i + 1);
      buf += '\n';
      if (buf.size() > (1 << 20)) {
        out << buf;
        buf.clear();
      }
    }
    out << buf;
    if (!out.good()) MF_FAIL(MF_EIO, std::string("failed writing ") + path);
  });
}

int mf_read_batch_file(const char* path, int32_t n, int32_t** u, int32_t** v, int64_t* m) {
  return guarded([&] {
    need(path && u && v && m, MF_EINVAL, "null argument");
    *u = nullptr;
    *v = nullptr;
    *m = 0;
    std::ifstream in(path);
    if (!in.is_open()) MF_FAIL(MF_EIO, std::string("could not open ") + path);
    std::vector<int32_t> a, b;
    std::string line;
    while (std::getline(in, line)) {
      std::istringstream iss(line);
      int src, dst;
      if (iss >> src >> dst) {
        --src;
        --dst;
        if (src >= 0 && src < n && dst >= 0 && dst < n && src != dst) {
          a.push_back(src);
          b.push_back(dst);
        }
      }
    }
    const size_t cnt = a.size();
    *u = (int32_t*)std::malloc(sizeof(int32_t) * std::max<size_t>(cnt, 1));
    *v = (int32_t*)std::malloc(sizeof(int32_t) * std::max<size_t>(cnt, 1));
    if (!*u || !*v) {
      std::free(*u);
      std::free(*v);
      *u = *v = nullptr;
      MF_FAIL(MF_ENOMEM, "host allocation failed");
    }
    if (cnt) {
      std::memcpy(*u, a.data(), sizeof(int32_t) * cnt);
      std::memcpy(*v, b.data(), sizeof(int32_t) * cnt);
    }
    *m = (int64_t)cnt;
  });
}

int mf_parse_batch_file(mf_ctx* c, const char* path, int32_t** u, int32_t** v, uint8_t** ins, int64_t* m) {
  return guarded([&] {
    need(c && path && u && v && ins && m, MF_EINVAL, "null argument");
    *u = nullptr;
    *v = nullptr;
    *ins = nullptr;
    *m = 0;
    bind(c);
    const int64_t cnt = mf::parse_batch_file_device(c, path);
    if (cnt > 0) mf::flag_updates(c, cnt);
    const size_t k = (size_t)std::max<int64_t>(cnt, 1);
    *u = (int32_t*)std::malloc(sizeof(int32_t) * k);
    *v = (int32_t*)std::malloc(sizeof(int32_t) * k);
    *ins = (uint8_t*)std::malloc(k);
    if (!*u || !*v || !*ins) {
      std::free(*u);
      std::free(*v);
      std::free(*ins);
      *u = *v = nullptr;
      *ins = nullptr;
      MF_FAIL(MF_ENOMEM, "host allocation failed");
    }
    if (cnt > 0) {
      MF_CUDA(cudaMemcpyAsync(*u, c->bu.p, sizeof(int32_t) * (size_t)cnt, cudaMemcpyDeviceToHost, c->stream));
      MF_CUDA(cudaMemcpyAsync(*v, c->bv.p, sizeof(int32_t) * (size_t)cnt, cudaMemcpyDeviceToHost, c->stream));
      MF_CUDA(cudaMemcpyAsync(*ins, c->bins.p, (size_t)cnt, cudaMemcpyDeviceToHost, c->stream));
      MF_CUDA(cudaStreamSynchronize(c->stream));
    }
    *m = cnt;
  });
}

int mf_list_batch_files(const char* folder, char** names, int64_t* count) {
  return guarded([&] {
    need(folder && names && count, MF_EINVAL, "null argument");
    *names = nullptr;
    *count = 0;
    std::vector<std::pair<int, std::string>> files;
    std::error_code ec;
    for (const auto& e : std::filesystem::directory_iterator(folder, ec)) {
      if (!e.is_regular_file()) continue;
      int key;
      try {
        key = std::stoi(e.path().stem().string());
      } catch (...) {
        MF_FAIL(MF_EFORMAT, "batch file name without an integer stem: " + e.path().filename().string());
      }
      files.emplace_back(key, e.path().filename().string());
    }
    if (ec) MF_FAIL(MF_EIO, std::string("could not list ") + folder);
    std::stable_sort(files.begin(), files.end(), [](const auto& x, const auto& y) {
      return x.first != y.first ? x.first < y.first : x.second < y.second;
    });
    std::string joined;
    for (const auto& f : files) joined += f.second + "\n";
    char* buf = (char*)std::malloc(joined.size() + 1);
    if (!buf) MF_FAIL(MF_ENOMEM, "host allocation failed");
    std::memcpy(buf, joined.data(), joined.size());
    buf[joined.size()] = 0;
    *names = buf;
    *count = (int64_t)files.size();
  });
}

void mf_free(void* p) { std::free(p); }

const char* mf_stage_name(int stage) {
  return (stage >= 0 && stage < mf::kStCount) ? mf::kStageNames[stage] : nullptr;
}

int mf_profile_enable(mf_ctx* c, int on) {
  return guarded([&] {
    need(c != nullptr && on >= 0 && on <= 6 && (on & 3) != 3, MF_EINVAL, "bad arguments");
    c->profile = on;
  });
}

int mf_profile_reset(mf_ctx* c) {
  return guarded([&] {
    need(c != nullptr, MF_EINVAL, "null context");
    for (int i = 0; i < mf::kStCount; ++i) {
      c->stage_ms[i] = 0;
      c->stage_calls[i] = 0;
      c->stage_bytes[i] = 0;
    }
  });
}

int mf_profile_read(mf_ctx* c, double* ms, int64_t* calls, double* bytes, int cap) {
  return guarded([&] {
    need(c && ms && calls && cap >= 0, MF_EINVAL, "bad arguments");
    for (int i = 0; i < mf::kStCount && i < cap; ++i) {
      ms[i] = c->stage_ms[i];
      calls[i] = c->stage_calls[i];
      if (bytes) bytes[i] = c->stage_bytes[i];
    }
  });
}

int64_t mf_kernel_launches(void) { return (int64_t)mf::g_launches.load(); }
int64_t mf_allocations(void) { return (int64_t)mf::g_allocs.load(); }

int mf_trace_enable(mf_ctx* c, int on) {
  return guarded([&] {
    need(c != nullptr, MF_EINVAL, "null context");
    c->trace = on != 0;
  });
}

int mf_trace_count(mf_ctx* c, int64_t* count) {
  return guarded([&] {
    need(c && count, MF_EINVAL, "null argument");
    *count = (int64_t)c->traces.size();
  });
}

int mf_trace_get(mf_ctx* c, int64_t index, int field, void* out, int64_t cap, int64_t* len) {
  return guarded([&] {
    need(c && len, MF_EINVAL, "null argument");
    need(index >= 0 && index < (int64_t)c->traces.size(), MF_EINVAL, "trace index out of range");
    const SubBatchTrace& t = c->traces[(size_t)index];
    auto put = [&](const void* src, int64_t cnt, size_t elem) {
      *len = cnt;
      if (out && cap > 0) std::memcpy(out, src, (size_t)std::min(cnt, cap) * elem);
    };
    switch (field) {
      case 0: put(t.hdr, 10, 8); break;
      case 1: put(t.seeds.data(), (int64_t)t.seeds.size(), 4); break;
      case 2: put(t.cands.data(), (int64_t)t.cands.size(), 4); break;
      case 3: put(t.cid_after.data(), (int64_t)t.cid_after.size(), 4); break;
      case 4: put(t.order.data(), (int64_t)t.order.size(), 4); break;
      case 5: put(t.mis_after.data(), (int64_t)t.mis_after.size(), 1); break;
      case 6: put(t.row_len.data(), (int64_t)t.row_len.size(), 8); break;
      default: MF_FAIL(MF_EINVAL, "unknown trace field");
    }
  });
}

}  // extern "C"
