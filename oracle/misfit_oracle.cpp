// misfit_oracle.cpp -- CPU oracle for the MISFIT dynamic-MIS path.
//
// TEST INFRASTRUCTURE ONLY: the checker for libmisfit_gb.  Only tests, the
// smoke check and the benchmark's CPU-baseline leg load it.
//
// A plain sequential restatement of the reference engine (src/misfit/misfit.cu
// and core/*.h of anonymous-artifacts/MISFIT) with the racy parts pinned to
// the canonical schedule described in misfit_oracle.h.  Each block cites the
// reference lines it restates.  The overlay uses the same container kinds as
// the reference (hash maps of vectors / sets) so that the CPU baseline timed
// through this file does the same kind of host work the reference does.

#include "misfit_oracle.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include <fcntl.h>
#include <unistd.h>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// src/misfit/misfit.cu:37 (MAX_BATCH_SIZE) and :560 (max_total_rows).
constexpr int64_t kMaxBatchEdges = 1048576;
constexpr int64_t kMaxRows = 2 * kMaxBatchEdges;
// src/misfit/misfit.cu:503-506: hop_limit 2 weighs each new endpoint by 1000.
constexpr int64_t kEstimateWeight = 1000;

struct SubBatchTrace {
  int64_t hdr[10];
  std::vector<int32_t> seeds, cands, cid_after, order;
  std::vector<uint8_t> mis_after;
  std::vector<int64_t> row_len;
};

}  // namespace

struct or_graph {
  int32_t n = 0;
  uint64_t edges = 0;
  std::vector<int64_t> nindex;
  std::vector<int32_t> nlist;
  // DeltaOverlay (core/FlashGraph.h:172-276).
  std::unordered_map<int32_t, std::vector<int32_t>> added;
  std::unordered_map<int32_t, std::unordered_set<int32_t>> removed;
  // DeviceNode {membership, cluster_id} (src/misfit/misfit.cu:129-134).
  std::vector<uint8_t> mis;
  std::vector<int32_t> cid;
  int64_t max_csr = 0;
  bool trace = false;
  bool exact = false;   // exact-MIS mode: fix-up after every batch (no reference counterpart)
  bool serial_clustering = false;   // clustering schedule switch (or_set_serial_clustering)
  std::vector<SubBatchTrace> traces;
};

namespace {

// MAX_CSR_ELEMENTS initial value (src/misfit/misfit.cu:768-772).
int64_t initial_max_csr(int32_t n, uint64_t edges) {
  double avg = n > 0 ? (double)edges / n : 1.0;
  int64_t est = (int64_t)(kMaxBatchEdges * 2.0 * avg * avg);
  int64_t v = est > 0 ? std::min<int64_t>(800000000LL, est) : 50000000LL;
  return std::max<int64_t>(v, 1000000LL);
}

void init_state(or_graph* g) {
  g->mis.assign(g->n, 0);
  g->cid.assign(g->n, -1);
  g->max_csr = initial_max_csr(g->n, g->edges);
}

// HybridGraph::isAdjacent (core/FlashGraph.h:291-301): added list, then the
// tombstone set, then a linear scan of the base row.
bool adjacent(const or_graph* g, int32_t u, int32_t v) {
  auto a = g->added.find(u);
  if (a != g->added.end() && std::find(a->second.begin(), a->second.end(), v) != a->second.end())
    return true;
  auto r = g->removed.find(u);
  if (r != g->removed.end() && r->second.count(v)) return false;
  for (int64_t k = g->nindex[u]; k < g->nindex[u + 1]; ++k)
    if (g->nlist[k] == v) return true;
  return false;
}

// DeltaOverlay::insertEdge / un_tombstone (core/FlashGraph.h:196-203,251-258).
void insert_edge(or_graph* g, int32_t u, int32_t v) {
  auto ru = g->removed.find(u);
  if (ru != g->removed.end() && ru->second.count(v)) {
    ru->second.erase(v);
    auto rv = g->removed.find(v);
    if (rv != g->removed.end()) rv->second.erase(u);
    return;
  }
  g->added[u].push_back(v);
  g->added[v].push_back(u);
}

// DeltaOverlay::removeEdge / forget_delta_edge (core/FlashGraph.h:205-212,260-275).
void remove_edge(or_graph* g, int32_t u, int32_t v) {
  auto au = g->added.find(u);
  if (au != g->added.end()) {
    auto it = std::find(au->second.begin(), au->second.end(), v);
    if (it != au->second.end()) {
      au->second.erase(it);
      auto av = g->added.find(v);
      if (av != g->added.end()) {
        auto jt = std::find(av->second.begin(), av->second.end(), u);
        if (jt != av->second.end()) av->second.erase(jt);
      }
      return;
    }
  }
  g->removed[u].insert(v);
  g->removed[v].insert(u);
}

// DeltaOverlay::neighbors_into (core/FlashGraph.h:214-233).
void row_into(const or_graph* g, int32_t x, std::vector<int32_t>& out) {
  out.clear();
  const int32_t* b = g->nlist.data() + g->nindex[x];
  const int32_t* e = g->nlist.data() + g->nindex[x + 1];
  auto r = g->removed.find(x);
  if (r == g->removed.end() || r->second.empty()) {
    out.insert(out.end(), b, e);
  } else {
    for (const int32_t* p = b; p != e; ++p)
      if (!r->second.count(*p)) out.push_back(*p);
  }
  auto a = g->added.find(x);
  if (a != g->added.end()) out.insert(out.end(), a->second.begin(), a->second.end());
}

// DeltaOverlay::degree (core/FlashGraph.h:235-242): a count, not a row length.
int32_t degree_of(const or_graph* g, int32_t x) {
  int32_t d = (int32_t)(g->nindex[x + 1] - g->nindex[x]);
  auto r = g->removed.find(x);
  if (r != g->removed.end()) d -= (int32_t)r->second.size();
  auto a = g->added.find(x);
  if (a != g->added.end()) d += (int32_t)a->second.size();
  return d;
}

// get_h_hop_neighborhood with hop_limit 2 (src/misfit/misfit.cu:159-202).
// Appends the hop-1 frontier to hop1 when it is non-null.
void two_hop(const or_graph* g, int32_t s, std::vector<char>& visited,
             std::vector<int32_t>& out, std::vector<int32_t>* hop1,
             std::vector<int32_t>& scratch) {
  out.clear();
  std::vector<int32_t> frontier, next;
  visited[s] = 1;
  out.push_back(s);
  frontier.push_back(s);
  for (int hop = 0; hop < 2 && !frontier.empty(); ++hop) {
    for (int32_t cur : frontier) {
      row_into(g, cur, scratch);
      if (hop == 1 && hop1) hop1->push_back(cur);
      for (int32_t y : scratch) {
        if (!visited[y]) {
          visited[y] = 1;
          next.push_back(y);
          out.push_back(y);
        }
      }
    }
    frontier.swap(next);
    next.clear();
  }
  for (int32_t y : out) visited[y] = 0;
}

bool any_member(const or_graph* g, const std::vector<int32_t>& row, int32_t except) {
  for (int32_t z : row)
    if (z != except && g->mis[z]) return true;
  return false;
}

// One sub-batch [p, q) of the batch; seeds/rows already decided by the caller.
struct SubBatch {
  std::vector<int32_t> mapped;              // seeds then candidates
  std::vector<std::vector<int32_t>> rows;   // 2-hop lists, then adjacency rows
  int64_t n_seeds = 0;
};

void run_kernels(or_graph* g, const int32_t* u, const int32_t* v, const uint8_t* ins,
                 int64_t p, int64_t q, SubBatch& sb, SubBatchTrace* tr) {
  const int64_t nrows = (int64_t)sb.mapped.size();
  // build_vertex_map_kernel (src/misfit/misfit.cu:211-217).
  std::unordered_map<int32_t, int64_t> v2i;
  v2i.reserve(nrows * 2 + 1);
  for (int64_t i = 0; i < nrows; ++i) v2i[sb.mapped[i]] = i;

  // vertex_clustering_csr_kernel (src/misfit/misfit.cu:219-259), bulk-synchronous:
  // every row reads the cluster ids as they were before the kernel.
  std::vector<int64_t> rowcid(nrows, -2);  // -2 = row returned early
  int64_t cluster_count = 0;
  if (g->serial_clustering) {
    // Alternative schedule: the rows run one after another, each reading the
    // writes of the rows before it (also a legal run of the racy kernel).
    for (int64_t i = 0; i < nrows; ++i) {
      if (g->cid[sb.mapped[i]] != -1) continue;
      int64_t found = -1;
      for (int32_t y : sb.rows[i])
        if (g->cid[y] != -1) { found = g->cid[y]; break; }
      rowcid[i] = found != -1 ? found : cluster_count++;
      for (int32_t y : sb.rows[i]) g->cid[y] = (int32_t)rowcid[i];
    }
  } else {
    for (int64_t i = 0; i < nrows; ++i) {
      if (g->cid[sb.mapped[i]] != -1) continue;
      int64_t found = -1;
      for (int32_t y : sb.rows[i])
        if (g->cid[y] != -1) { found = g->cid[y]; break; }
      rowcid[i] = found != -1 ? found : cluster_count++;
    }
    // Writes land in row order, so the highest row index writes last.
    for (int64_t i = 0; i < nrows; ++i) {
      if (rowcid[i] == -2) continue;
      for (int32_t y : sb.rows[i]) g->cid[y] = (int32_t)rowcid[i];
    }
  }
  if (tr) tr->cid_after = g->cid;

  // assign_edges_to_clusters_kernel (src/misfit/misfit.cu:261-275): arrival in
  // ascending index, head insertion, so each list runs in descending index.
  const int64_t limit = std::min<int64_t>(cluster_count, kMaxBatchEdges);
  std::vector<std::vector<int64_t>> lists(limit > 0 ? limit : 0);
  for (int64_t t = p; t < q; ++t) {
    int64_t c = -1;
    if (g->cid[u[t]] != -1) c = g->cid[u[t]];
    else if (g->cid[v[t]] != -1) c = g->cid[v[t]];
    if (c != -1 && c < limit) lists[c].push_back(t);
  }

  // process_clusters_csr_kernel (src/misfit/misfit.cu:277-349), clusters in
  // ascending id, each list walked from its head.
  auto row_of = [&](int32_t x) -> const std::vector<int32_t>* {
    auto it = v2i.find(x);
    return it == v2i.end() ? nullptr : &sb.rows[it->second];
  };
  int64_t processed = 0;
  for (int64_t c = 0; c < limit; ++c) {
    for (auto it = lists[c].rbegin(); it != lists[c].rend(); ++it) {
      const int64_t t = *it;
      ++processed;
      if (tr) tr->order.push_back((int32_t)t);
      const int32_t a = u[t], b = v[t];
      const bool ma = g->mis[a], mb = g->mis[b];
      if (ins[t]) {
        if (!(ma && mb)) continue;
        const int32_t r = a > b ? a : b;
        g->mis[r] = 0;
        const std::vector<int32_t>* rr = row_of(r);
        if (!rr) continue;
        for (int32_t w : *rr) {
          if (g->mis[w]) continue;
          const std::vector<int32_t>* rw = row_of(w);
          if (!rw) continue;
          if (!any_member(g, *rw, -1)) { g->mis[w] = 1; break; }
        }
      } else {
        int32_t y, keep;
        if (ma && !mb) { y = b; keep = a; }
        else if (!ma && mb) { y = a; keep = b; }
        else continue;
        const std::vector<int32_t>* ry = row_of(y);
        if (!ry || !any_member(g, *ry, keep)) g->mis[y] = 1;
      }
    }
  }
  if (tr) {
    tr->hdr[6] = cluster_count;
    tr->hdr[7] = processed;
    tr->mis_after = g->mis;
  }
  // clear_cluster_assignments_kernel (src/misfit/misfit.cu:351-358): only the
  // mapped vertices are reset; other row elements keep their ids.
  for (int32_t x : sb.mapped) g->cid[x] = -1;
}

}  // namespace

extern "C" {

or_graph* or_create(int32_t n, const int64_t* nindex, const int32_t* nlist) {
  if (n < 0) return nullptr;
  or_graph* g = new or_graph();
  g->n = n;
  g->nindex.assign(nindex, nindex + n + 1);
  g->edges = (uint64_t)g->nindex[n];
  g->nlist.assign(nlist, nlist + g->nindex[n]);
  init_state(g);
  return g;
}

// FlashGraph::map_file (core/FlashGraph.h:108-169): header int32 nodes, int32
// edges or -1 then int64 edges; nindex int32 or int64; nlist int32.
or_graph* or_open_egr(const char* path) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return nullptr;
  int32_t n = 0, e32 = 0;
  uint64_t edges = 0;
  bool wide = false;
  if (std::fread(&n, 4, 1, f) != 1 || std::fread(&e32, 4, 1, f) != 1) { std::fclose(f); return nullptr; }
  if (e32 == -1) {
    if (std::fread(&edges, 8, 1, f) != 1) { std::fclose(f); return nullptr; }
    wide = true;
  } else {
    if (n < 1 || e32 < 0) { std::fclose(f); return nullptr; }
    edges = (uint64_t)e32;
  }
  if (n < 0) { std::fclose(f); return nullptr; }
  or_graph* g = new or_graph();
  g->n = n;
  g->edges = edges;
  g->nindex.resize((size_t)n + 1);
  bool ok = true;
  if (wide) {
    ok = std::fread(g->nindex.data(), 8, (size_t)n + 1, f) == (size_t)n + 1;
  } else {
    std::vector<int32_t> tmp((size_t)n + 1);
    ok = std::fread(tmp.data(), 4, (size_t)n + 1, f) == (size_t)n + 1;
    for (size_t i = 0; ok && i <= (size_t)n; ++i) g->nindex[i] = tmp[i];
  }
  if (ok) {
    g->nlist.resize(edges);
    ok = std::fread(g->nlist.data(), 4, edges, f) == edges;
  }
  std::fclose(f);
  if (!ok) { delete g; return nullptr; }
  init_state(g);
  return g;
}

void or_destroy(or_graph* g) { delete g; }
int32_t or_num_nodes(const or_graph* g) { return g->n; }
int64_t or_base_entries(const or_graph* g) { return (int64_t)g->edges; }
int64_t or_max_csr(const or_graph* g) { return g->max_csr; }
void or_set_max_csr(or_graph* g, int64_t v) { g->max_csr = v; }
void or_set_exact(or_graph* g, int on) { g->exact = on != 0; }
void or_set_serial_clustering(or_graph* g, int on) { g->serial_clustering = on != 0; }

// setMISFromHost / getMISToHost (src/misfit/misfit.cu:448-462).
void or_set_mis(or_graph* g, const uint8_t* mis) {
  for (int32_t i = 0; i < g->n; ++i) { g->mis[i] = mis[i] ? 1 : 0; g->cid[i] = -1; }
}
void or_get_mis(const or_graph* g, uint8_t* out) { std::memcpy(out, g->mis.data(), g->n); }
void or_get_cluster_ids(const or_graph* g, int32_t* out) {
  std::memcpy(out, g->cid.data(), sizeof(int32_t) * (size_t)g->n);
}

void or_flag_updates(const or_graph* g, const int32_t* u, const int32_t* v, int64_t m, uint8_t* ins_out) {
  for (int64_t i = 0; i < m; ++i) ins_out[i] = adjacent(g, u[i], v[i]) ? 0 : 1;
}
int or_is_adjacent(const or_graph* g, int32_t u, int32_t v) { return adjacent(g, u, v) ? 1 : 0; }

// Exact-MIS mode (no reference counterpart): after the reference's repair,
// (1) every member with a smaller-id member neighbour leaves (decided on the
// set as the repair left it), then (2) the non-members with no member
// neighbour are completed greedily in ascending id.  The result is an
// independent, maximal set.
static void exact_fixup(or_graph* g) {
  std::vector<int32_t> r;
  std::vector<uint8_t> leave((size_t)g->n, 0);
  for (int32_t x = 0; x < g->n; ++x) {
    if (!g->mis[(size_t)x]) continue;
    row_into(g, x, r);
    for (int32_t y : r)
      if (y < x && g->mis[(size_t)y]) { leave[(size_t)x] = 1; break; }
  }
  for (int32_t x = 0; x < g->n; ++x)
    if (leave[(size_t)x]) g->mis[(size_t)x] = 0;
  for (int32_t x = 0; x < g->n; ++x) {
    if (g->mis[(size_t)x]) continue;
    row_into(g, x, r);
    bool covered = false;
    for (int32_t y : r)
      if (g->mis[(size_t)y]) { covered = true; break; }
    if (!covered) g->mis[(size_t)x] = 1;
  }
}

int64_t or_apply_batch(or_graph* g, const int32_t* u, const int32_t* v, const uint8_t* ins, int64_t m) {
  g->traces.clear();
  if (m <= 0) return 0;
  // Batch apply (src/misfit/misfit.cu:708-714): file order, conditional.
  for (int64_t i = 0; i < m; ++i) {
    if (ins[i] && !adjacent(g, u[i], v[i])) insert_edge(g, u[i], v[i]);
    else if (!ins[i] && adjacent(g, u[i], v[i])) remove_edge(g, u[i], v[i]);
  }

  int threads = 1;
#ifdef _OPENMP
  threads = omp_get_max_threads();
#endif
  std::vector<std::vector<char>> visited(threads, std::vector<char>(g->n, 0));
  std::vector<int64_t> seen(g->n, -1);  // sub-batch start that last saw a vertex
  std::vector<uint8_t> hop1_mark(g->n, 0);

  int64_t p = 0, nsub = 0;
  while (p < m) {
    // Greedy split (src/misfit/misfit.cu:490-521).
    std::vector<int32_t> seeds;
    int64_t est = 0, q = p;
    while (q < m && q - p < kMaxBatchEdges) {
      const int32_t a = u[q], b = v[q];
      int64_t add = 0;
      if (seen[a] != p) add += (int64_t)degree_of(g, a) * kEstimateWeight;
      if (seen[b] != p) add += (int64_t)degree_of(g, b) * kEstimateWeight;
      if (q > p && est + add >= g->max_csr) break;
      est += add;
      if (seen[a] != p) { seen[a] = p; seeds.push_back(a); }
      if (seen[b] != p) { seen[b] = p; seeds.push_back(b); }
      ++q;
    }

    // Exact 2-hop lists and hop-1 frontiers (src/misfit/misfit.cu:527-548).
    SubBatch sb;
    sb.n_seeds = (int64_t)seeds.size();
    std::vector<std::vector<int32_t>> lists(seeds.size());
    std::vector<std::vector<int32_t>> hop1(seeds.size());
#pragma omp parallel
    {
      int tid = 0;
#ifdef _OPENMP
      tid = omp_get_thread_num();
#endif
      std::vector<int32_t> scratch;
#pragma omp for schedule(dynamic, 16)
      for (int64_t i = 0; i < (int64_t)seeds.size(); ++i)
        two_hop(g, seeds[i], visited[tid], lists[i], &hop1[i], scratch);
    }
    // Candidate rows: hop-1 vertices that are not seeds (src/misfit/misfit.cu:550-558),
    // in ascending vertex id.
    std::vector<int32_t> cands;
    for (auto& h : hop1)
      for (int32_t x : h)
        if (seen[x] != p && !hop1_mark[x]) { hop1_mark[x] = 1; cands.push_back(x); }
    for (int32_t x : cands) hop1_mark[x] = 0;
    std::sort(cands.begin(), cands.end());

    // Row packing with MAX_CSR_ELEMENTS growth (src/misfit/misfit.cu:560-599).
    int64_t off = 0;
    std::vector<int64_t> row_len;
    auto pack = [&](int32_t x, std::vector<int32_t>&& row) {
      const int64_t len = (int64_t)row.size();
      if (off + len >= g->max_csr)
        g->max_csr = (int64_t)((double)((uint64_t)off + (uint64_t)len) * 1.5);
      off += len;
      row_len.push_back(len);
      sb.mapped.push_back(x);
      sb.rows.push_back(std::move(row));
    };
    for (size_t i = 0; i < seeds.size(); ++i) pack(seeds[i], std::move(lists[i]));
    std::vector<int32_t> packed_cands;
    std::vector<int32_t> scratch;
    for (int32_t c : cands) {
      if ((int64_t)sb.mapped.size() >= kMaxRows) break;
      row_into(g, c, scratch);
      packed_cands.push_back(c);
      pack(c, std::vector<int32_t>(scratch));
    }

    SubBatchTrace* tr = nullptr;
    if (g->trace) {
      g->traces.emplace_back();
      tr = &g->traces.back();
      tr->hdr[0] = p; tr->hdr[1] = q; tr->hdr[2] = sb.n_seeds;
      tr->hdr[3] = (int64_t)packed_cands.size(); tr->hdr[4] = off;
      tr->hdr[5] = g->max_csr; tr->hdr[8] = (int64_t)sb.mapped.size(); tr->hdr[9] = est;
      tr->seeds = seeds;
      tr->cands = packed_cands;
      tr->row_len = row_len;
    }
    run_kernels(g, u, v, ins, p, q, sb, tr);
    p = q;
    ++nsub;
  }
  if (g->exact) exact_fixup(g);
  return nsub;
}

int64_t or_row(const or_graph* g, int32_t x, int32_t* out, int64_t cap) {
  std::vector<int32_t> r;
  row_into(g, x, r);
  for (int64_t i = 0; i < (int64_t)r.size() && i < cap; ++i) out[i] = r[i];
  return (int64_t)r.size();
}

int32_t or_degree(const or_graph* g, int32_t x) { return degree_of(g, x); }

int64_t or_two_hop(const or_graph* g, int32_t s, int32_t* out, int64_t cap) {
  std::vector<char> visited(g->n, 0);
  std::vector<int32_t> list, scratch;
  two_hop(g, s, visited, list, nullptr, scratch);
  for (int64_t i = 0; i < (int64_t)list.size() && i < cap; ++i) out[i] = list[i];
  return (int64_t)list.size();
}

void or_trace_enable(or_graph* g, int on) { g->trace = on != 0; }
int64_t or_trace_count(const or_graph* g) { return (int64_t)g->traces.size(); }

int64_t or_trace_get(const or_graph* g, int64_t i, int field, void* out, int64_t cap) {
  if (i < 0 || i >= (int64_t)g->traces.size()) return -1;
  const SubBatchTrace& t = g->traces[i];
  auto put = [&](const void* src, int64_t count, size_t elem) -> int64_t {
    if (out && cap > 0) std::memcpy(out, src, (size_t)std::min(count, cap) * elem);
    return count;
  };
  switch (field) {
    case 0: return put(t.hdr, 10, 8);
    case 1: return put(t.seeds.data(), (int64_t)t.seeds.size(), 4);
    case 2: return put(t.cands.data(), (int64_t)t.cands.size(), 4);
    case 3: return put(t.cid_after.data(), (int64_t)t.cid_after.size(), 4);
    case 4: return put(t.order.data(), (int64_t)t.order.size(), 4);
    case 5: return put(t.mis_after.data(), (int64_t)t.mis_after.size(), 1);
    case 6: return put(t.row_len.data(), (int64_t)t.row_len.size(), 8);
    default: return -1;
  }
}

// compact_flash_graph (core/flash_compactor.h:20-105): degree formula with a
// negative-degree error, int64-sentinel layout, rows base-minus-tombstones
// then added, temp file + fsync + rename + directory fsync.
int or_compact(const or_graph* g, const char* out_path) {
  const int32_t n = g->n;
  std::vector<uint64_t> idx((size_t)n + 1, 0);
  for (int32_t x = 0; x < n; ++x) {
    int64_t d = degree_of(g, x);
    if (d < 0) return -1;
    idx[x + 1] = idx[x] + (uint64_t)d;
  }
  std::string tmp = std::string(out_path) + ".tmp." + std::to_string(getpid());
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) return -2;
  const int32_t sentinel = -1;
  const uint64_t total = idx[n];
  bool ok = std::fwrite(&n, 4, 1, f) == 1 && std::fwrite(&sentinel, 4, 1, f) == 1 &&
            std::fwrite(&total, 8, 1, f) == 1 &&
            std::fwrite(idx.data(), 8, (size_t)n + 1, f) == (size_t)n + 1;
  std::vector<int32_t> r;
  for (int32_t x = 0; ok && x < n; ++x) {
    row_into(g, x, r);
    if ((uint64_t)r.size() != idx[x + 1] - idx[x]) { ok = false; break; }
    if (!r.empty() && std::fwrite(r.data(), 4, r.size(), f) != r.size()) ok = false;
  }
  if (ok) ok = std::fflush(f) == 0 && fsync(fileno(f)) == 0;
  std::fclose(f);
  if (!ok) { std::remove(tmp.c_str()); return -3; }
  if (std::rename(tmp.c_str(), out_path) != 0) return -4;
  std::string dir = ".";
  std::string op(out_path);
  size_t slash = op.find_last_of('/');
  if (slash != std::string::npos) dir = op.substr(0, slash);
  int fd = ::open(dir.c_str(), O_RDONLY);
  if (fd >= 0) { fsync(fd); ::close(fd); }
  return 0;
}

void or_greedy_mis(int32_t n, const int64_t* nindex, const int32_t* nlist, uint8_t* out) {
  std::vector<uint8_t> blocked(n, 0);
  for (int32_t x = 0; x < n; ++x) {
    out[x] = 0;
    if (blocked[x]) continue;
    out[x] = 1;
    for (int64_t k = nindex[x]; k < nindex[x + 1]; ++k) blocked[nlist[k]] = 1;
  }
}

// The from-scratch alternative to the repair, for the CPU baseline: the batch
// applied to the overlay (src/misfit/misfit.cu:708-714), then the greedy MIS
// of tools/compute_initial_mis.py:151-162 recomputed over the whole current
// graph, single-threaded as that tool is.
void or_apply_overlay(or_graph* g, const int32_t* u, const int32_t* v, const uint8_t* ins, int64_t m) {
  for (int64_t i = 0; i < m; ++i) {
    if (ins[i] && !adjacent(g, u[i], v[i])) insert_edge(g, u[i], v[i]);
    else if (!ins[i] && adjacent(g, u[i], v[i])) remove_edge(g, u[i], v[i]);
  }
}

void or_greedy_current(or_graph* g) {
  std::vector<uint8_t> blocked((size_t)g->n, 0);
  std::vector<int32_t> r;
  for (int32_t x = 0; x < g->n; ++x) {
    g->mis[(size_t)x] = 0;
    if (blocked[(size_t)x]) continue;
    g->mis[(size_t)x] = 1;
    row_into(g, x, r);
    for (int32_t y : r) blocked[(size_t)y] = 1;
  }
}

void or_check_mis(const or_graph* g, int64_t* violations, int64_t* non_maximal) {
  int64_t viol = 0, nonmax = 0;
  std::vector<int32_t> r;
  for (int32_t x = 0; x < g->n; ++x) {
    row_into(g, x, r);
    bool covered = g->mis[x] != 0;
    for (int32_t y : r) {
      if (g->mis[y]) covered = true;
      if (g->mis[x] && g->mis[y] && x < y) ++viol;
    }
    if (!covered) ++nonmax;
  }
  *violations = viol;
  *non_maximal = nonmax;
}

}  // extern "C"
