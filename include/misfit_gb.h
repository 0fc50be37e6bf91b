/*
 * misfit_gb.h -- C ABI of libmisfit_gb, the GB300 implementation of MISFIT's
 * dynamic maximal-independent-set maintenance path.
 *
 * The reference (anonymous-artifacts/MISFIT) has no plugin API: its boundary
 * is the 5-argument CLI plus the .egr / MIS / batch-folder files, and inside
 * the binary the seam is HybridGraph + GPUVertexClusteringGraph +
 * compact_flash_graph.  Each entry point below names the reference interface
 * it replaces (file:line in the reference tree).
 *
 * Conventions:
 *   - every function returns an mf_status (0 = success, negative = error) and
 *     never calls exit(); the reference exits the process on every error
 *     (src/misfit/misfit.cu:28-35, core/FlashGraph.h:110-153);
 *   - mf_last_error() gives a one-line description of the last failure on
 *     the calling thread;
 *   - vertex ids are 0-based int32 (the text formats are 1-based and are
 *     converted by the file helpers, as the reference does);
 *   - a context is bound to one GPU and is not thread-safe: one host thread
 *     drives it.  Host input arrays may be reused as soon as the call that
 *     took them returns, except for mf_apply_batch_async (see there);
 *   - all state (base CSR, delta overlay, membership, cluster ids) lives in
 *     device memory; the library owns every buffer it allocates.
 */
#ifndef MISFIT_GB_H
#define MISFIT_GB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mf_ctx mf_ctx;

typedef enum mf_status {
  MF_OK = 0,
  MF_EINVAL = -1,   /* bad argument (range, size, null pointer) */
  MF_EIO = -2,      /* file could not be opened, read or written */
  MF_EFORMAT = -3,  /* malformed .egr / MIS / batch file */
  MF_ECUDA = -4,    /* CUDA runtime error */
  MF_ENOMEM = -5,   /* device or pinned allocation failed */
  MF_ESTATE = -6,   /* inconsistent graph state (e.g. negative degree) */
  MF_ELIMIT = -7    /* request beyond a documented fixed limit */
} mf_status;

/* Per-batch counters of the last processed batch (host-side copy). */
typedef struct mf_batch_stats {
  int64_t updates;          /* lines in the batch */
  int64_t sub_batches;      /* sub-batches the split rule produced */
  int64_t seeds;            /* mapped seed rows, summed over sub-batches */
  int64_t candidates;       /* mapped candidate rows, summed */
  int64_t clusters;         /* cluster_count, summed (src/misfit/misfit.cu:681) */
  int64_t processed_edges;  /* edges walked by the repair stage */
  int64_t exact_sizes;      /* sub-batches that needed exact 2-hop sizes */
  int64_t max_csr;          /* MAX_CSR_ELEMENTS after the batch */
  int64_t repair_rounds;    /* speculative repair rounds, summed */
  double device_ms;         /* device time of the batch (CUDA events) */
  /* With profiler bit 4 (mf_profile_enable): the exact packed volume of the
   * batch, summed over sub-batches (every seed's 2-hop list length plus every
   * candidate row's length, the elements the reference packs), and the sum
   * of the degrees of the mapped rows.  -1 otherwise. */
  int64_t packed_total;
  int64_t row_degree_total;
} mf_batch_stats;

/* ---- lifetime -------------------------------------------------------- */

/* Version of this ABI (major*10000 + minor*100 + patch).  1.1 added the
 * batched form (mf_apply_batches, mf_batched_*), mf_pool_set_batching and the
 * two batched_* fields at the end of mf_pool_stats.  1.2 added
 * mf_tuning.pull_sizes, mf_batched_opts.pool_idle_first and
 * mf_pool_stats.handed_to_workers, each at the end of its struct. */
int mf_version(void);
const char* mf_status_string(int status);
/* Last error on the calling thread ("" when none). */
const char* mf_last_error(void);

/* Open a .egr file (int32 or int64-sentinel nindex) and stage it into HBM on
 * device `gpu`.  Replaces HybridGraph::open + FlashGraph::map_file
 * (core/FlashGraph.h:108-169,285-289) and the GPUVertexClusteringGraph
 * constructor (src/misfit/misfit.cu:389-421); MAX_CSR_ELEMENTS starts at the
 * reference's estimate (src/misfit/misfit.cu:768-772). */
int mf_open_egr(const char* path, int gpu, mf_ctx** out);

/* Same, from an in-memory CSR (nindex has n+1 entries, copied). */
int mf_open_csr(int32_t n, const int64_t* nindex, const int32_t* nlist, int gpu, mf_ctx** out);

/* Release all device and host resources (~GPUVertexClusteringGraph,
 * src/misfit/misfit.cu:423-439). */
int mf_close(mf_ctx* ctx);

int mf_num_nodes(const mf_ctx* ctx, int32_t* n);
int mf_num_base_entries(const mf_ctx* ctx, int64_t* entries);

/* ---- membership ------------------------------------------------------- */

/* Upload a 0/1 membership vector of n bytes and reset all cluster ids
 * (setMISFromHost, src/misfit/misfit.cu:448-453). */
int mf_set_mis(mf_ctx* ctx, const uint8_t* mis, int64_t n);
/* Download the membership vector (getMISToHost, src/misfit/misfit.cu:455-462). */
int mf_get_mis(mf_ctx* ctx, uint8_t* out, int64_t n);
/* Number of members, counted on the device. */
int mf_mis_size(mf_ctx* ctx, int64_t* count);

/* Greedy MIS of the current graph in ascending vertex order -- the set
 * tools/compute_initial_mis.py:32-43 computes -- written to out[n] (it does
 * not change the context's membership). */
int mf_greedy_mis(mf_ctx* ctx, uint8_t* out, int64_t n);

/* ---- updates --------------------------------------------------------- */

/* is_insertion = !isAdjacent(u, v) against the current graph, one byte per
 * update (core/cli_setup.h:66-82; src/misfit/misfit.cu:812-828 evaluates it
 * for every batch before any batch is applied). */
int mf_flag_updates(mf_ctx* ctx, const int32_t* u, const int32_t* v, int64_t m, uint8_t* ins_out);

/* Largest m that mf_flag_updates_noalloc accepts. */
#define MF_NOALLOC_MAX_UPDATES 65536

/* mf_flag_updates for callers that must not allocate device memory.  This
 * entry point has no counterpart in the reference.
 * mf_flag_updates stages the endpoints in per-context device buffers that
 * grow to the largest batch seen, and growing one means a cudaFree plus a
 * cudaMalloc.  Two kinds of caller cannot accept that:
 *   - a process that has committed the device's memory to its graphs and
 *     overlays, where a growth can fail with MF_ENOMEM part way through a
 *     stream of batches;
 *   - a process with work in flight on other streams of the device, which
 *     the cudaFree waits for.
 * This variant allocates nothing.  Its scratch is one fixed device array of
 * 590,080 bytes (room for MF_NOALLOC_MAX_UPDATES pairs and their flags).
 *   - The first call on a device finds the array's address once
 *     (cudaGetSymbolAddress).  Make that first call, which may have
 *     m = 0, before any stream capture.
 *   - The address is looked up again whenever a context is opened on the
 *     device (mf_open_egr / mf_open_csr, outside any capture).  After a
 *     cudaDeviceReset the cached address is stale: open a new context on
 *     that device before the next call.
 *   - m > MF_NOALLOC_MAX_UPDATES returns MF_ELIMIT and does nothing.
 *   - Each call zeroes the array's invalid-pair counter itself.
 *   - Invalid endpoints return MF_EINVAL without writing ins_out, as in
 *     mf_flag_updates.
 *   - All contexts on one device share the array.  Calls that overlap in
 *     time, from several host threads or on several contexts of one
 *     device, race on it: the caller must serialise them.
 * The flags are the same as those of mf_flag_updates on the same graph. */
int mf_flag_updates_noalloc(mf_ctx* ctx, const int32_t* u, const int32_t* v, int64_t m, uint8_t* ins_out);

/* Process one batch: conditional overlay insert/delete in file order, the
 * sub-batch split, 2-hop neighbourhoods, clustering and MIS repair.
 * Replaces processBatchGPUVertexClustering (src/misfit/misfit.cu:704-730)
 * with GPUVertexClusteringGraph::processBatchWithVertexClustering
 * (:468-692).  u, v: 0-based endpoints, u != v, both < n; ins: the flags.
 * Host arrays; returns when the batch is complete on the device. */
int mf_apply_batch(mf_ctx* ctx, const int32_t* u, const int32_t* v, const uint8_t* ins, int64_t m);

/* Same with device-resident inputs (device pointers, m entries each). */
int mf_apply_batch_device(mf_ctx* ctx, const int32_t* d_u, const int32_t* d_v,
                          const uint8_t* d_ins, int64_t m);

/* The pipelined engine: launchBatch / syncAndCollect of misfit_async
 * (src/misfit_async/misfit_async.cu:484-700, its loop :826-876).
 * mf_apply_batch_async queues the batch for the context's worker thread and
 * returns at once; the worker runs queued batches one after another, in
 * order, with the same results as mf_apply_batch.  The host arrays must stay
 * valid until the batch is collected.  Several batches may be queued (the
 * reference's loop keeps two: batch i+1 is launched before batch i is
 * collected).  Bad pointers or a negative m fail at once; everything else
 * (including invalid endpoints) is reported when the batch is collected.
 * mf_collect waits for the oldest uncollected batch, writes its statistics
 * (out may be NULL) and returns its status and error message.
 * mf_sync collects every queued batch and returns the first failure, if any.
 * While batches are uncollected, mf_apply_batch / mf_apply_batch_device /
 * mf_apply_batches reject the context (MF_EINVAL); every other call on the
 * context first waits until the queued batches have run. */
int mf_apply_batch_async(mf_ctx* ctx, const int32_t* u, const int32_t* v, const uint8_t* ins, int64_t m);
int mf_collect(mf_ctx* ctx, mf_batch_stats* out);
int mf_sync(mf_ctx* ctx);

int mf_last_batch_stats(mf_ctx* ctx, mf_batch_stats* out);

/* Load-balancing settings of one context.  They decide how the work of a
 * sub-batch is spread over kernels and threads, never what it computes:
 * every setting gives the same results (misfit_gb300/autotune.py searches
 * them).  No reference counterpart (the reference's kernels have none).  */
typedef struct mf_tuning {
  int64_t pull_long;      /* rows longer than this take the warp-per-row pass of the
                             candidates' cluster-id pull instead of one thread (default 2048) */
  int64_t heavy_min;      /* least row length of a heavy vertex, whose neighbourhood bitmap the
                             exact 2-hop sizes cache (default 2048; the threshold used is
                             max(heavy_min, n/256)) */
  int64_t big_threshold;  /* hop-2 volume above which the insertion rule's search for the first
                             eligible vertex goes to the grid-wide kernel (default 64) */
  int64_t first_bound;    /* row positions the warp level of the first-cluster-id search covers
                             before long rows go to the chunk level (default 256, at least 8;
                             values below 32, the per-thread probe's length, act as 32) */
  int64_t cand_push;      /* the candidate rows' cluster ids: 1 always pushed from the candidate rows,
                             then finalised per vertex; 2 pulled by every vertex on graphs with
                             symmetric sorted rows (pushed on the others); 0 (default) as 2, except
                             the sub-batches whose candidate rows hold so few entries that the push
                             costs less than half the pull's estimate */
  int64_t pull_sizes;     /* exact 2-hop sizes on symmetric graphs: 0 always by the push form (bit
                             atomics per element of every member's row); 1 (default) the seeds whose
                             neighbourhood volume pays for it by passes over every row, up to 256
                             seeds per pass; 2 every seed to size by those passes */
} mf_tuning;
int mf_get_tuning(mf_ctx* ctx, mf_tuning* out);
int mf_set_tuning(mf_ctx* ctx, const mf_tuning* in);

/* ---- graph queries ----------------------------------------------------- */

/* Row of x in overlay order (base minus tombstones, then added neighbours in
 * insertion order; DeltaOverlay::neighbors_into, core/FlashGraph.h:214-233).
 * Writes min(len, cap) entries and the full length to *len. */
int mf_get_row(mf_ctx* ctx, int32_t x, int32_t* out, int64_t cap, int64_t* len);
/* DeltaOverlay::degree (core/FlashGraph.h:235-242) for all n vertices. */
int mf_get_degrees(mf_ctx* ctx, int32_t* out, int64_t n);
int mf_is_adjacent(mf_ctx* ctx, int32_t u, int32_t v, int* adjacent);
int mf_get_max_csr(mf_ctx* ctx, int64_t* value);
int mf_set_max_csr(mf_ctx* ctx, int64_t value);
int mf_get_cluster_ids(mf_ctx* ctx, int32_t* out, int64_t n);

/* Independence violations (edges with both ends in the set) and uncovered
 * vertices (neither in the set nor adjacent to it) on the current graph. */
int mf_check_mis(mf_ctx* ctx, int64_t* violations, int64_t* uncovered);

/* Exact-MIS mode (on != 0).  No counterpart in the reference, whose repair
 * rules are conservative and can leave violations and uncovered vertices.
 * After each batch's repair: every member with a smaller-id member neighbour
 * leaves, then the vertices with no member neighbour join greedily in
 * ascending id, so the set is independent and maximal afterwards. */
int mf_set_exact(mf_ctx* ctx, int on);

/* ---- compaction -------------------------------------------------------- */

/* Merge base + overlay on the device and write an int64-sentinel .egr via a
 * temporary file, fsync, rename and directory fsync.  With rebase != 0 the
 * merged CSR becomes the new base and the overlay is cleared (the
 * reference's remap + delta.clear(), src/misfit/misfit.cu:919-921).
 * Replaces compact_flash_graph (core/flash_compactor.h:20-105). */
int mf_compact(mf_ctx* ctx, const char* out_path, int rebase);

/* ---- file helpers (host) ----------------------------------------------- */

/* Read a MIS file (1-based ids, one per line; out-of-range ids ignored,
 * src/misfit/misfit.cu:778-791) into out[n]; *lines counts accepted lines. */
int mf_read_mis_file(const char* path, int32_t n, uint8_t* out, int64_t* lines);
/* Write the members of mis[n] 1-based, one per line (src/misfit/misfit.cu:892-907). */
int mf_write_mis_file(const char* path, const uint8_t* mis, int32_t n);

/* Parse a batch file: lines "u v" (1-based); lines that do not start with
 * two integers, out-of-range ids and self-loops are dropped
 * (core/cli_setup.h:66-82).  *u and *v are malloc'd 0-based arrays the
 * caller releases with mf_free. */
int mf_read_batch_file(const char* path, int32_t n, int32_t** u, int32_t** v, int64_t* m);

/* The same parse on the device of ctx, with the same line rules, followed by
 * the flags against the context's current graph (mf_flag_updates): one call
 * replaces parse_batch_file plus its isAdjacent flagging
 * (core/cli_setup.h:66-82).  *u, *v, *ins are malloc'd arrays of *m
 * entries the caller releases with mf_free. */
int mf_parse_batch_file(mf_ctx* ctx, const char* path, int32_t** u, int32_t** v, uint8_t** ins, int64_t* m);
/* Regular files of a folder sorted by the integer value of their stem
 * (core/cli_setup.h:49-59); names joined by '\n' into a malloc'd string. */
int mf_list_batch_files(const char* folder, char** names, int64_t* count);
void mf_free(void* p);

/* ---- profiling ----------------------------------------------------------- */

/* Number of stages the profiler distinguishes. */
#define MF_NUM_STAGES 15
/* Name of stage i (0 <= i < MF_NUM_STAGES), NULL otherwise. */
const char* mf_stage_name(int stage);
/* on = 1: every later batch records CUDA events around each stage on the
 * context's stream; times accumulate until mf_profile_reset.  on = 2: only
 * the k_lb_push_hop launches (the "push_hop" stage) and the candidates'
 * pull (the "pull" stage: k_cand_bits, k_pull_cand, k_pull_cand_long) are
 * timed, six event records per sub-batch instead of about fifty.  on = 0: off.
 * Adding 4 (on = 4, 5, 6) also counts each batch's algorithmic work
 * (mf_batch_stats.packed_total / row_degree_total): every sub-batch then
 * computes its exact 2-hop sizes, which costs device time, so a batch timed
 * for throughput should run without it.  Results are unchanged. */
int mf_profile_enable(mf_ctx* ctx, int on);
int mf_profile_reset(mf_ctx* ctx);
/* Accumulated device milliseconds, occurrences and algorithmic bytes per
 * stage (cap entries; bytes may be NULL).  Bytes are counted for the stages
 * with a device work counter (hop1, cluster_write, push_hop, pull) and are 0
 * elsewhere. */
int mf_profile_read(mf_ctx* ctx, double* ms, int64_t* calls, double* bytes, int cap);
/* Kernels launched by this library in this process so far. */
int64_t mf_kernel_launches(void);
/* Device and pinned-host allocations (cudaMalloc, cudaMallocAsync,
 * cudaMallocHost) made by this library in this process so far; a call that
 * leaves it unchanged allocated nothing.  No reference counterpart (a
 * diagnostic of this library). */
int64_t mf_allocations(void);

/* ---- trace (parity tests) ---------------------------------------------- */

/* When enabled, mf_apply_batch keeps, per sub-batch, the stage outputs the
 * tests compare with the oracle.  field: 0 header int64[10] = {p, q,
 * n_seeds, n_cands, packed (or -1 when not needed), max_after,
 * cluster_count, n_processed, n_rows, estimate}; 1 seeds (int32); 2
 * candidates (int32); 3 cluster ids after clustering (int32[n]); 4 processed
 * edges in repair order (int32 batch index); 5 membership after repair
 * (uint8[n]); 6 row lengths (int64, only when packed >= 0). */
int mf_trace_enable(mf_ctx* ctx, int on);
int mf_trace_count(mf_ctx* ctx, int64_t* count);
int mf_trace_get(mf_ctx* ctx, int64_t index, int field, void* out, int64_t cap, int64_t* len);

/* ---- serving pool (no counterpart in the reference) -------------------------
 *
 * The reference runs one graph per process.  A pool keeps many graphs on one
 * GPU and serves update batches as they arrive:
 *   - batches for one graph run in submission order, one at a time; batches
 *     of different graphs run concurrently, each graph on its own stream,
 *     driven by one of the pool's host worker threads;
 *   - admission is by HBM budget, checked before a graph runs and after each
 *     batch: idle resident graphs, least recently used first, first give up
 *     their per-batch scratch and are then evicted to pinned host memory
 *     until the resident graphs fit (a graph whose batch is running is never
 *     touched; when every resident graph is running the new one is admitted
 *     over budget and counted in over_budget);
 *   - eviction saves the graph's state exactly (base CSR, overlay with its
 *     tombstone positions and insertion order, membership, cluster ids), so
 *     every batch result equals the one a dedicated context gives. */
typedef struct mf_pool mf_pool;

typedef struct mf_pool_stats {
  int64_t graphs;               /* graphs added */
  int64_t completed;            /* batches completed */
  int64_t updates;              /* update lines in the completed batches */
  int64_t errors;               /* batches or moves that failed */
  int64_t evictions;            /* graphs moved to pinned host memory */
  int64_t restores;             /* graphs moved back to the device */
  int64_t trims;                /* idle graphs that gave up their per-batch scratch */
  int64_t over_budget;          /* admissions made while over the budget */
  int64_t resident_bytes;       /* device bytes of the resident graphs now */
  int64_t peak_resident_bytes;  /* the largest value seen */
  int64_t batched_steps;        /* mf_apply_batches steps run by the batched dispatch */
  int64_t batched_requests;     /* requests those steps carried */
  int64_t handed_to_workers;    /* small requests the dispatcher gave to idle workers */
} mf_pool_stats;

/* A pool on device `gpu` that keeps at most `hbm_budget` bytes of graph state
 * and scratch resident, with `workers` host threads (1..64). */
int mf_pool_create(int gpu, int64_t hbm_budget, int workers, mf_pool** out);
/* Waits for the running batches, then frees everything. */
int mf_pool_destroy(mf_pool* pool);
/* Adds a graph from an in-memory CSR (nindex n+1 entries; copied) with its
 * initial membership (n bytes, 0/1); *gid receives its id. */
int mf_pool_add_graph(mf_pool* pool, int32_t n, const int64_t* nindex, const int32_t* nlist, const uint8_t* mis,
                      int32_t* gid);
/* Queues one batch (arrays copied; same meaning as mf_apply_batch) and
 * returns at once; *rid identifies the request. */
int mf_pool_submit(mf_pool* pool, int32_t gid, const int32_t* u, const int32_t* v, const uint8_t* ins, int64_t m,
                   int64_t* rid);
/* Waits for request rid; returns its status and, in *latency_ms, the time
 * from submission to completion.  Each request is waited for once. */
int mf_pool_wait(mf_pool* pool, int64_t rid, double* latency_ms);
/* Waits until no batch is queued or running. */
int mf_pool_drain(mf_pool* pool);
/* Membership of graph gid after its queued batches (n bytes). */
int mf_pool_get_mis(mf_pool* pool, int32_t gid, uint8_t* out, int64_t n);
int mf_pool_stats_get(mf_pool* pool, mf_pool_stats* out);
/* Changes the budget; it applies from the next admission on. */
int mf_pool_set_budget(mf_pool* pool, int64_t hbm_budget);

/* ---- batched form: one batch for each of many graphs in one step ---------
 * No reference counterpart (the reference runs one graph per process; this
 * is the batched multi-graph form, with per-graph results equal to
 * mf_apply_batch's on each context).  Batches small enough for one CTA run
 * together in ONE persistent kernel: each CTA takes the next graph batch
 * from a device work queue (largest first) and runs that graph's whole path
 * -- overlay apply, split rule, neighbourhoods, clustering, assignment,
 * repair, clear -- with no host round trip.  The step (batch upload, queue
 * reset, the kernel, the read-back of the per-graph results) is captured
 * and launched as one CUDA graph.  Larger batches, graphs above the vertex
 * limit and contexts in exact-MIS mode take the multi-launch path
 * (mf_apply_batch, from up to 8 host threads, each graph on its own stream)
 * while the persistent kernel runs. */
typedef struct mf_batched_opts {
  int block;                  /* threads per persistent CTA: 64..1024, a multiple of 32 (default 512) */
  int ctas_per_sm;            /* persistent CTAs per SM (default 2) */
  int64_t max_cta_updates;    /* batches of at most this many lines take the kernel (default 8192) */
  int32_t max_cta_vertices;   /* ... on graphs of at most this many vertices (default 2^20) */
  int use_graph;              /* 1: capture the step as a CUDA graph (default), 0: plain launches */
  int path_threads;           /* host threads driving the batches above the kernel's limits, each
                                 graph on its own stream (1..64, default 8) */
  int pool_idle_first;        /* pools only (mf_pool_set_batching): 1 (default) hands a ready group
                                 of small requests to the workers when the idle workers can take
                                 all of it, one request each; 0 always batches it */
} mf_batched_opts;

typedef struct mf_batched_stats {
  int64_t kernel_items;       /* batches run by the persistent kernel */
  int64_t path_items;         /* batches run through the multi-launch path */
  int64_t updates;            /* lines over all batches */
  double kernel_ms;           /* device time of the persistent-kernel step (CUDA events) */
  double wall_ms;             /* host time of the whole call */
} mf_batched_stats;

int mf_batched_default_opts(mf_batched_opts* out);
/* Applies batch i (u[i], v[i], ins[i]: m[i] host lines, same meaning as
 * mf_apply_batch) to ctxs[i] for i < count, all in one step.  The contexts
 * must be distinct, on one GPU, with no asynchronous batch pending.  Every
 * batch is checked (ids in range, no self-loop) before anything runs, so a
 * bad batch changes no graph.  opts may be NULL (defaults); stats may be
 * NULL.  Each context's mf_last_batch_stats describes its batch afterwards. */
int mf_apply_batches(mf_ctx* const* ctxs, const int32_t* const* u, const int32_t* const* v,
                     const uint8_t* const* ins, const int64_t* m, int64_t count, const mf_batched_opts* opts,
                     mf_batched_stats* stats);
/* Batched dispatch for a pool (continuous batching): with opts non-NULL,
 * every request of a resident graph whose batch mf_apply_batches would give
 * to its persistent kernel (size and vertex limits of opts, compat mode),
 * on a graph whose current mean degree, added entries included, keeps
 * lines * (1 + degree)^2 within max_cta_updates * 33^2, goes to one
 * dispatcher thread instead of the workers.  The dispatcher
 * takes every such request that is ready -- one per graph -- and applies
 * them in one mf_apply_batches step; requests that arrive meanwhile form the
 * next step.  With opts->pool_idle_first set, a ready group no larger than
 * the number of idle workers goes to those workers instead (one step of the
 * batched kernel costs more than a worker's plain batch when it would hold
 * only a few requests).  Larger requests, and the requests of graphs evicted to host
 * memory (restored by the workers), stay with the workers.  opts NULL turns
 * it off.  Results per graph are unchanged. */
int mf_pool_set_batching(mf_pool* pool, const mf_batched_opts* opts);

#ifdef __cplusplus
}
#endif

#endif
