// mf_pool.cu -- the serving form: many resident graphs, continuous admission.
//
// No counterpart in the reference, which processes one graph per process.
// A pool owns graph contexts on one GPU and a set of host worker threads:
//   * every graph keeps its base CSR, delta overlay, membership and cluster
//     ids; batches submitted for a graph run in submission order, one at a
//     time, while batches of different graphs run concurrently on their own
//     CUDA streams (one worker thread drives one graph's batch);
//   * admission is by HBM budget: before a graph runs, idle resident graphs
//     are evicted least-recently-used first until its footprint fits;
//   * eviction copies the graph's state to pinned host memory and frees all
//     of its device buffers; restore copies it back.  The state is restored
//     bit for bit (tombstone positions and added-entry order decide later
//     rows), so a graph's results do not depend on how often it moved.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "mf_internal.cuh"

namespace mf {

namespace {

template <class T>
void save(PinnedSnapshot& snap, const DBuf<T>& b, int64_t count, cudaStream_t s) {
  const size_t bytes = sizeof(T) * (size_t)count;
  snap.parts.push_back({snap.used, bytes});
  if (bytes > 0) MF_CUDA(cudaMemcpyAsync(snap.host + snap.used, b.p, bytes, cudaMemcpyDeviceToHost, s));
  snap.used += (bytes + 255) & ~(size_t)255;
}

template <class T>
void load(const PinnedSnapshot& snap, size_t& part, DBuf<T>& b, int64_t count, cudaStream_t s) {
  b.reserve(std::max<int64_t>(count, 1));
  const auto& pr = snap.parts[part++];
  if (pr.second > 0) MF_CUDA(cudaMemcpyAsync(b.p, snap.host + pr.first, pr.second, cudaMemcpyHostToDevice, s));
}

}  // namespace

int64_t snapshot_bytes(const mf_ctx* c) {
  const int64_t n = c->n, words = (c->nnz + 31) / 32;
  auto r = [](int64_t b) { return (b + 255) & ~(int64_t)255; };
  return r(8 * (n + 1)) + r(4 * c->nnz) + r(4 * words) + 3 * r(4 * n) + r(8 * (n + 1)) + 2 * r(4 * c->a_total) +
         r(n) + r(4 * n);
}

void evict(mf_ctx* c, PinnedSnapshot& snap) {
  cudaStream_t s = c->stream;
  MF_CUDA(cudaStreamSynchronize(s));
  const size_t need = (size_t)snapshot_bytes(c);
  if (snap.cap < need) {
    if (snap.host) cudaFreeHost(snap.host);
    snap.host = nullptr;
    snap.cap = 0;
    mf::note_alloc();
    MF_CUDA(cudaMallocHost(&snap.host, need));
    snap.cap = need;
  }
  snap.used = 0;
  snap.parts.clear();
  const int64_t n = c->n, words = (c->nnz + 31) / 32;
  save(snap, c->nindex, n + 1, s);
  save(snap, c->nlist, c->nnz, s);
  save(snap, c->live, words, s);
  save(snap, c->dead, n, s);
  save(snap, c->rcnt, n, s);
  save(snap, c->deg, n, s);
  save(snap, c->aoff, n + 1, s);
  save(snap, c->aadj, c->a_total, s);
  save(snap, c->aown, c->a_total, s);
  save(snap, c->mis, n, s);
  save(snap, c->cid, n, s);
  MF_CUDA(cudaStreamSynchronize(s));
  release_device_state(c);
}

void restore(mf_ctx* c, const PinnedSnapshot& snap) {
  cudaStream_t s = c->stream;
  const int64_t n = c->n, words = (c->nnz + 31) / 32;
  size_t part = 0;
  load(snap, part, c->nindex, n + 1, s);
  c->nlist.reserve(c->nnz + mf::kNlistPad);
  load(snap, part, c->nlist, c->nnz, s);
  load(snap, part, c->live, words, s);
  load(snap, part, c->dead, n, s);
  load(snap, part, c->rcnt, n, s);
  load(snap, part, c->deg, n, s);
  load(snap, part, c->aoff, n + 1, s);
  load(snap, part, c->aadj, c->a_total, s);
  load(snap, part, c->aown, c->a_total, s);
  load(snap, part, c->mis, n, s);
  load(snap, part, c->cid, n, s);
  alloc_vertex_scratch(c);
  MF_CUDA(cudaStreamSynchronize(s));
}

}  // namespace mf

// ---- the pool -------------------------------------------------------------------

namespace {

struct Request {
  int64_t rid = 0;
  int32_t gid = 0;
  std::vector<int32_t> u, v;
  std::vector<uint8_t> ins;
  double t_submit = 0, t_start = 0, t_done = 0;
  int status = MF_OK;
  std::string error;
  bool done = false;
};

struct Graph {
  mf_ctx* ctx = nullptr;
  bool resident = false;
  bool busy = false;           // a worker runs its batch, or it is being moved
  mf::PinnedSnapshot snap;
  int64_t bytes = 0;           // device bytes when last resident
  bool trimmed = false;        // per-batch scratch freed since its last batch
  uint64_t last_use = 0;
  std::deque<Request*> queue;  // in submission order
};

}  // namespace

struct mf_pool {
  int device = 0;
  int64_t budget = 0;
  std::deque<Graph> graphs;    // a deque: references stay valid while graphs are added
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<int32_t> ready;   // graphs with queued batches and no running one
  std::unordered_map<int64_t, Request*> reqs;
  std::vector<std::thread> workers;
  int working = 0;             // workers between taking a request and finishing it
  // batched dispatch (mf_pool_set_batching): small front requests are
  // routed to one dispatcher thread, which applies all of them that are
  // ready in one mf_apply_batches step while later arrivals queue for the
  // next step
  bool batching = false;
  mf_batched_opts bopts{};
  std::deque<int32_t> ready_small;
  std::condition_variable cv_batch;
  std::thread dispatcher;
  bool stop = false;
  int64_t next_rid = 1;
  uint64_t tick = 0;
  int64_t resident_bytes = 0;
  mf_pool_stats st{};

  // Makes room for `need` bytes, least recently used idle graphs first: a
  // graph that still holds per-batch scratch gives that up (no copy), one
  // that does not is evicted to pinned host memory.  Called with the lock
  // held; the moves run with it released (the victim is marked busy).
  void make_room(std::unique_lock<std::mutex>& lk, int64_t need, int32_t self) {
    while (resident_bytes + need > budget) {
      int32_t victim = -1;
      for (int32_t g = 0; g < (int32_t)graphs.size(); ++g) {
        const Graph& gr = graphs[(size_t)g];
        if (g == self || !gr.resident || gr.busy) continue;
        if (victim < 0) { victim = g; continue; }
        const Graph& vb = graphs[(size_t)victim];
        // idle graphs with nothing queued first, then untrimmed ones, then LRU
        const auto rank = [](const Graph& x) { return (x.queue.empty() ? 0 : 2) + (x.trimmed ? 1 : 0); };
        if (rank(gr) < rank(vb) || (rank(gr) == rank(vb) && gr.last_use < vb.last_use)) victim = g;
      }
      if (victim < 0) {
        st.over_budget += 1;  // every resident graph is running: admit anyway
        return;
      }
      Graph& v = graphs[(size_t)victim];
      const bool full = v.trimmed;
      v.busy = true;
      lk.unlock();
      int status = MF_OK;
      int64_t after = 0;
      try {
        mf::bind_device(v.ctx);
        MF_CUDA(cudaStreamSynchronize(v.ctx->stream));
        if (full) {
          mf::evict(v.ctx, v.snap);
        } else {
          mf::release_batch_scratch(v.ctx);
          after = mf::ctx_device_bytes(v.ctx);
        }
      } catch (const mf::Failure& f) {
        status = f.status;
      }
      mf::g_alloc_stream = nullptr;
      lk.lock();
      v.busy = false;
      // mf_pool_drain and mf_pool_get_mis wait on cv_done for "not busy":
      // clearing the flag must wake them, or a waiter that checked while the
      // move ran sleeps forever once the pool goes quiet (the stall of the
      // eviction test: the last request's completion notified, then started
      // this move).
      cv_done.notify_all();
      if (status == MF_OK) {
        if (full) {
          v.resident = false;
          resident_bytes -= v.bytes;
          st.evictions += 1;
        } else {
          resident_bytes -= v.bytes - after;
          v.bytes = after;
          v.trimmed = true;
          st.trims += 1;
        }
      } else {
        st.errors += 1;
      }
      if (!v.queue.empty()) {
        enqueue_ready(victim);
      }
    }
  }

  // Whether a request goes to the batched kernel: within the size and vertex
  // limits and, since one CTA walks the batch's 2-hop neighbourhoods (about
  // lines * (1 + mean degree)^2 positions), on a graph whose current mean
  // degree, overlay included, keeps that walk within the limit's at mean
  // degree 32.  A small graph that takes many insert-heavy requests grows
  // dense (added entries accumulate in its overlay); its requests then go to
  // the workers, whose launches spread the walk over the whole GPU.
  bool small(const Graph& gr, const Request* rq) const {
    const mf_ctx* c = gr.ctx;
    const int64_t lines = (int64_t)rq->u.size();
    if (lines > bopts.max_cta_updates || c->n > bopts.max_cta_vertices || c->exact) return false;
    const double avg = c->n > 0 ? (double)(c->nnz + c->a_total) / (double)c->n : 0.0;
    return (double)lines * (1.0 + avg) * (1.0 + avg) <= (double)bopts.max_cta_updates * 33.0 * 33.0;
  }

  // Whether the dispatcher takes the graph's front request: batching on, the
  // request small, and the graph resident.  A graph evicted to host memory
  // goes to the workers, which restore graphs concurrently; restored inside
  // a step, it would hold up every other graph of the step (and the hot
  // graphs' queues behind them, one request per step).
  bool for_dispatcher(const Graph& gr) const {
    return batching && gr.resident && !gr.queue.empty() && small(gr, gr.queue.front());
  }

  // A graph with a queued batch and none running becomes ready: for the
  // dispatcher (for_dispatcher), else for the workers.  Called with the
  // lock held.
  void enqueue_ready(int32_t gid) {
    const Graph& gr = graphs[(size_t)gid];
    if (for_dispatcher(gr)) {
      ready_small.push_back(gid);
      cv_batch.notify_one();
    } else {
      ready.push_back(gid);
      cv_work.notify_one();
    }
  }

  void dispatch_loop() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
      cv_batch.wait(lk, [&] { return stop || !ready_small.empty(); });
      if (stop && ready_small.empty()) return;
      std::vector<int32_t> group;
      while (!ready_small.empty()) {
        const int32_t g = ready_small.front();
        ready_small.pop_front();
        Graph& x = graphs[(size_t)g];
        if (x.busy || x.queue.empty()) continue;
        if (!for_dispatcher(x)) {
          ready.push_back(g);
          cv_work.notify_one();
          continue;
        }
        x.busy = true;
        group.push_back(g);
      }
      if (group.empty()) continue;
      // idle workers (minus the requests already waiting for them) that can
      // take the whole group, one request each: a worker's plain batch is
      // cheaper than a batched step over so few requests
      const int idle = (int)workers.size() - working - (int)ready.size();
      if (bopts.pool_idle_first && (int)group.size() <= idle) {
        for (const int32_t g : group) {
          graphs[(size_t)g].busy = false;
          ready.push_back(g);
          cv_work.notify_one();
        }
        st.handed_to_workers += (int64_t)group.size();
        continue;
      }
      run_group(lk, group);
    }
  }

  // One batched step over the front requests of `group` (graphs marked busy).
  void run_group(std::unique_lock<std::mutex>& lk, const std::vector<int32_t>& group) {
    // MISFIT_GB_POOL_DEBUG: one line per batched step (sizes and times)
    static const bool debug = std::getenv("MISFIT_GB_POOL_DEBUG") != nullptr;
    const double t_begin = mf::now_ms_host();
    int restored = 0;
    const size_t k = group.size();
    std::vector<int> status(k, MF_OK);
    std::vector<std::string> err(k);
    std::vector<Request*> rqs(k);
    for (size_t j = 0; j < k; ++j) {
      Graph& x = graphs[(size_t)group[j]];
      Request* rq = x.queue.front();
      rqs[j] = rq;
      // the step refuses a whole call with a bad batch in it: check each here
      for (size_t t = 0; t < rq->u.size(); ++t) {
        const int32_t a = rq->u[t], b = rq->v[t];
        if (a < 0 || a >= x.ctx->n || b < 0 || b >= x.ctx->n || a == b) {
          status[j] = MF_EINVAL;
          err[j] = "update endpoints out of range or equal";
          break;
        }
      }
      if (status[j] != MF_OK || x.resident) continue;
      make_room(lk, x.bytes, group[j]);
      lk.unlock();
      try {
        mf::bind_device(x.ctx);
        mf::restore(x.ctx, x.snap);
      } catch (const mf::Failure& f) {
        status[j] = f.status;
        err[j] = mf_last_error();
      }
      mf::g_alloc_stream = nullptr;
      lk.lock();
      if (status[j] == MF_OK) {
        x.resident = true;
        resident_bytes += x.bytes;
        st.restores += 1;
        ++restored;
      }
    }
    std::vector<mf_ctx*> ctxs;
    std::vector<const int32_t*> us, vs;
    std::vector<const uint8_t*> is;
    std::vector<int64_t> ms;
    const double t0 = mf::now_ms_host();
    for (size_t j = 0; j < k; ++j) {
      rqs[j]->t_start = t0;
      if (status[j] != MF_OK) continue;
      ctxs.push_back(graphs[(size_t)group[j]].ctx);
      us.push_back(rqs[j]->u.data());
      vs.push_back(rqs[j]->v.data());
      is.push_back(rqs[j]->ins.data());
      ms.push_back((int64_t)rqs[j]->u.size());
    }
    const mf_batched_opts opts = bopts;
    lk.unlock();
    int rc = MF_OK;
    std::string rerr;
    mf_batched_stats bst{};
    if (!ctxs.empty()) {
      rc = mf_apply_batches(ctxs.data(), us.data(), vs.data(), is.data(), ms.data(), (int64_t)ctxs.size(), &opts,
                            &bst);
      if (rc != MF_OK) rerr = mf_last_error();
    }
    if (debug) {
      int64_t lines = 0;
      for (const int64_t x : ms) lines += x;
      std::fprintf(stderr, "[misfit_gb] pool step: graphs %zu lines %lld restored %d prepare-ms %.2f apply-ms %.2f "
                   "kernel-ms %.2f\n", ctxs.size(), (long long)lines, restored, t0 - t_begin,
                   mf::now_ms_host() - t0, (double)bst.kernel_ms);
    }
    std::vector<int64_t> bytes(k, -1);
    for (size_t j = 0; j < k; ++j)
      if (status[j] == MF_OK && rc == MF_OK) bytes[j] = mf::ctx_device_bytes(graphs[(size_t)group[j]].ctx);
    lk.lock();
    const double t1 = mf::now_ms_host();
    for (size_t j = 0; j < k; ++j) {
      const int32_t gid = group[j];
      Graph& gr = graphs[(size_t)gid];
      Request* rq = rqs[j];
      if (status[j] == MF_OK && rc != MF_OK) {
        status[j] = rc;
        err[j] = rerr;
      }
      rq->t_done = t1;
      rq->status = status[j];
      rq->error = err[j];
      rq->done = true;
      if (bytes[j] >= 0) {
        resident_bytes += bytes[j] - gr.bytes;
        gr.bytes = bytes[j];
      }
      gr.trimmed = false;
      gr.queue.pop_front();
      gr.busy = false;
      --working;
      gr.last_use = ++tick;
      st.completed += 1;
      st.updates += (int64_t)rq->u.size();
      if (status[j] != MF_OK) st.errors += 1;
      if (!gr.queue.empty()) enqueue_ready(gid);
    }
    st.batched_steps += 1;
    st.batched_requests += (int64_t)ctxs.size();
    st.resident_bytes = resident_bytes;
    st.peak_resident_bytes = std::max(st.peak_resident_bytes, resident_bytes);
    cv_done.notify_all();
    if (resident_bytes > budget) make_room(lk, 0, -1);
    st.resident_bytes = resident_bytes;
  }

  void worker() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
      cv_work.wait(lk, [&] { return stop || !ready.empty(); });
      if (stop && ready.empty()) return;
      const int32_t gid = ready.front();
      ready.pop_front();
      Graph& gr = graphs[(size_t)gid];
      if (gr.busy || gr.queue.empty()) continue;
      gr.busy = true;
      ++working;
      Request* rq = gr.queue.front();
      int status = MF_OK;
      std::string err;
      if (!gr.resident) {
        make_room(lk, gr.bytes, gid);
        lk.unlock();
        try {
          mf::bind_device(gr.ctx);
          mf::restore(gr.ctx, gr.snap);
        } catch (const mf::Failure& f) {
          status = f.status;
          err = mf_last_error();
        }
        mf::g_alloc_stream = nullptr;
        lk.lock();
        if (status == MF_OK) {
          gr.resident = true;
          resident_bytes += gr.bytes;
          st.restores += 1;
        }
      }
      rq->t_start = mf::now_ms_host();
      lk.unlock();
      if (status == MF_OK) {
        status = mf_apply_batch(gr.ctx, rq->u.data(), rq->v.data(), rq->ins.data(), (int64_t)rq->u.size());
        if (status != MF_OK) err = mf_last_error();
      }
      const int64_t bytes = status == MF_OK ? mf::ctx_device_bytes(gr.ctx) : gr.bytes;
      lk.lock();
      rq->t_done = mf::now_ms_host();
      rq->status = status;
      rq->error = err;
      rq->done = true;
      resident_bytes += bytes - gr.bytes;
      gr.bytes = bytes;
      gr.trimmed = false;
      gr.queue.pop_front();
      gr.busy = false;
      --working;
      gr.last_use = ++tick;
      st.completed += 1;
      st.updates += (int64_t)rq->u.size();
      if (status != MF_OK) st.errors += 1;
      st.resident_bytes = resident_bytes;
      st.peak_resident_bytes = std::max(st.peak_resident_bytes, resident_bytes);
      if (!gr.queue.empty()) {
        enqueue_ready(gid);
      }
      cv_done.notify_all();
      // the batch may have grown its scratch: back under the budget
      if (resident_bytes > budget) make_room(lk, 0, -1);
      st.resident_bytes = resident_bytes;
    }
  }
};

namespace {

template <class F>
int pool_guarded(F&& f) {
  try {
    mf::set_error("");
    f();
    return MF_OK;
  } catch (const mf::Failure& e) {
    return e.status;
  } catch (const std::bad_alloc&) {
    mf::set_error("host allocation failed");
    return MF_ENOMEM;
  } catch (const std::exception& e) {
    mf::set_error(e.what());
    return MF_EINVAL;
  }
}

void need_arg(bool cond, const char* msg) {
  if (!cond) MF_FAIL(MF_EINVAL, msg);
}

}  // namespace

extern "C" {

int mf_pool_create(int gpu, int64_t hbm_budget, int workers, mf_pool** out) {
  return pool_guarded([&] {
    need_arg(out != nullptr && hbm_budget > 0 && workers >= 1 && workers <= 64, "bad arguments");
    int count = 0;
    MF_CUDA(cudaGetDeviceCount(&count));
    need_arg(gpu >= 0 && gpu < count, "gpu id out of range");
    mf_pool* p = new mf_pool();
    p->device = gpu;
    p->budget = hbm_budget;
    for (int i = 0; i < workers; ++i) p->workers.emplace_back([p] { p->worker(); });
    *out = p;
  });
}

int mf_pool_destroy(mf_pool* p) {
  return pool_guarded([&] {
    need_arg(p != nullptr, "null pool");
    {
      std::lock_guard<std::mutex> lk(p->mu);
      p->stop = true;
    }
    p->cv_work.notify_all();
    p->cv_batch.notify_all();
    for (auto& t : p->workers) t.join();
    if (p->dispatcher.joinable()) p->dispatcher.join();
    for (auto& gr : p->graphs) {
      if (gr.ctx) mf_close(gr.ctx);
      if (gr.snap.host) cudaFreeHost(gr.snap.host);
    }
    for (auto& kv : p->reqs) delete kv.second;  // every request not yet waited for, queued ones included
    delete p;
  });
}

int mf_pool_add_graph(mf_pool* p, int32_t n, const int64_t* nindex, const int32_t* nlist, const uint8_t* mis,
                      int32_t* gid) {
  return pool_guarded([&] {
    need_arg(p && gid && n > 0 && nindex && mis, "bad arguments");
    mf_ctx* c = nullptr;
    int st = mf_open_csr(n, nindex, nlist, p->device, &c);
    if (st != MF_OK) throw mf::Failure{st};
    st = mf_set_mis(c, mis, n);
    if (st != MF_OK) {
      mf_close(c);
      throw mf::Failure{st};
    }
    std::unique_lock<std::mutex> lk(p->mu);
    Graph gr;
    gr.ctx = c;
    gr.resident = true;
    gr.bytes = mf::ctx_device_bytes(c);
    gr.last_use = ++p->tick;
    p->graphs.push_back(std::move(gr));
    const int32_t id = (int32_t)p->graphs.size() - 1;
    p->resident_bytes += p->graphs.back().bytes;
    // over budget: the new graph waits on the host until its first batch
    if (p->resident_bytes > p->budget) {
      Graph& me = p->graphs.back();
      me.busy = true;
      p->resident_bytes -= me.bytes;
      lk.unlock();
      try {
        mf::bind_device(c);
        mf::evict(c, me.snap);
      } catch (...) {
        mf::g_alloc_stream = nullptr;
        lk.lock();
        me.busy = false;   // the graph stays listed as resident; wake any waiter
        p->resident_bytes += me.bytes;
        p->cv_done.notify_all();
        throw;
      }
      mf::g_alloc_stream = nullptr;
      lk.lock();
      me.resident = false;
      me.busy = false;
      p->cv_done.notify_all();
      p->st.evictions += 1;
      if (!me.queue.empty()) {
        p->enqueue_ready(id);
      }
    }
    p->st.graphs = (int64_t)p->graphs.size();
    p->st.resident_bytes = p->resident_bytes;
    p->st.peak_resident_bytes = std::max(p->st.peak_resident_bytes, p->resident_bytes);
    *gid = id;
  });
}

int mf_pool_submit(mf_pool* p, int32_t gid, const int32_t* u, const int32_t* v, const uint8_t* ins, int64_t m,
                   int64_t* rid) {
  return pool_guarded([&] {
    need_arg(p && rid && m >= 0 && (m == 0 || (u && v && ins)), "bad arguments");
    Request* r = new Request();
    r->u.assign(u, u + m);
    r->v.assign(v, v + m);
    r->ins.assign(ins, ins + m);
    r->t_submit = mf::now_ms_host();
    std::lock_guard<std::mutex> lk(p->mu);
    if (gid < 0 || gid >= (int32_t)p->graphs.size()) {
      delete r;
      MF_FAIL(MF_EINVAL, "unknown graph id");
    }
    r->gid = gid;
    r->rid = p->next_rid++;
    Graph& gr = p->graphs[(size_t)gid];
    gr.queue.push_back(r);
    p->reqs[r->rid] = r;
    if (gr.queue.size() == 1 && !gr.busy) {
      p->enqueue_ready(gid);
    }
    *rid = r->rid;
  });
}

int mf_pool_wait(mf_pool* p, int64_t rid, double* latency_ms) {
  int status = MF_OK;
  std::string err;
  const int st = pool_guarded([&] {
    need_arg(p != nullptr, "null pool");
    std::unique_lock<std::mutex> lk(p->mu);
    auto it = p->reqs.find(rid);
    if (it == p->reqs.end()) MF_FAIL(MF_EINVAL, "unknown request id");
    Request* r = it->second;
    p->cv_done.wait(lk, [&] { return r->done; });
    if (latency_ms) *latency_ms = r->t_done - r->t_submit;
    status = r->status;
    err = r->error;
    p->reqs.erase(it);
    delete r;
  });
  if (st != MF_OK) return st;
  if (status != MF_OK) mf::set_error(err);
  return status;
}

int mf_pool_drain(mf_pool* p) {
  return pool_guarded([&] {
    need_arg(p != nullptr, "null pool");
    std::unique_lock<std::mutex> lk(p->mu);
    p->cv_done.wait(lk, [&] {
      for (const auto& gr : p->graphs)
        if (!gr.queue.empty() || gr.busy) return false;
      return true;
    });
  });
}

int mf_pool_get_mis(mf_pool* p, int32_t gid, uint8_t* out, int64_t n) {
  return pool_guarded([&] {
    need_arg(p && out, "bad arguments");
    std::unique_lock<std::mutex> lk(p->mu);
    need_arg(gid >= 0 && gid < (int32_t)p->graphs.size(), "unknown graph id");
    Graph& gr = p->graphs[(size_t)gid];
    p->cv_done.wait(lk, [&] { return gr.queue.empty() && !gr.busy; });
    need_arg(n == gr.ctx->n, "output must have n entries");
    if (gr.resident) {
      const int st = mf_get_mis(gr.ctx, out, n);
      if (st != MF_OK) throw mf::Failure{st};
    } else {
      // membership is the tenth saved part (see mf::evict)
      const auto& pr = gr.snap.parts[9];
      std::copy(gr.snap.host + pr.first, gr.snap.host + pr.first + pr.second, out);
    }
  });
}

int mf_pool_set_budget(mf_pool* p, int64_t hbm_budget) {
  return pool_guarded([&] {
    need_arg(p != nullptr && hbm_budget > 0, "bad arguments");
    std::lock_guard<std::mutex> lk(p->mu);
    p->budget = hbm_budget;
  });
}

int mf_pool_set_batching(mf_pool* p, const mf_batched_opts* opts) {
  return pool_guarded([&] {
    need_arg(p != nullptr, "null pool");
    mf_batched_opts o{};
    if (opts) {
      o = *opts;
      need_arg(o.block >= 64 && o.block <= 1024 && o.block % 32 == 0 && o.ctas_per_sm >= 1 && o.ctas_per_sm <= 32 &&
                   o.max_cta_updates >= 0 && o.max_cta_updates <= mf::kMaxBatchEdges && o.path_threads >= 1 &&
                   o.path_threads <= 64 && (o.pool_idle_first == 0 || o.pool_idle_first == 1),
               "bad batched options");
    }
    std::lock_guard<std::mutex> lk(p->mu);
    p->batching = opts != nullptr;
    p->bopts = o;
    if (p->batching && !p->dispatcher.joinable()) p->dispatcher = std::thread([p] { p->dispatch_loop(); });
    if (!p->batching) {
      while (!p->ready_small.empty()) {
        p->ready.push_back(p->ready_small.front());
        p->ready_small.pop_front();
        p->cv_work.notify_one();
      }
    }
  });
}

int mf_pool_stats_get(mf_pool* p, mf_pool_stats* out) {
  return pool_guarded([&] {
    need_arg(p && out, "bad arguments");
    std::lock_guard<std::mutex> lk(p->mu);
    *out = p->st;
    out->resident_bytes = p->resident_bytes;
  });
}

}  // extern "C"
