/*
 * misfit_oracle.h -- C interface of the CPU oracle for MISFIT's dynamic
 * MIS-maintenance path.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is the checker that the GPU library
 * (libmisfit_gb) is compared against; only tests, the smoke check and the
 * CPU-baseline leg of the benchmark load it.  No product code path links or
 * calls it.
 *
 * It restates, single-threaded except for the OpenMP neighbourhood stage, the
 * reference engine's host path and its six CUDA kernels under one pinned,
 * deterministic schedule:
 *   - seed order  = first appearance of an endpoint in the sub-batch
 *                   (the reference iterates a std::unordered_set,
 *                    src/misfit/misfit.cu:495,523);
 *   - candidate order = ascending vertex id (the reference merges per-thread
 *                   std::unordered_maps, src/misfit/misfit.cu:550-558);
 *   - clustering  = bulk-synchronous: every row reads the pre-kernel cluster
 *                   ids, new ids are numbered by ascending row index and the
 *                   highest row index is the last writer of every element
 *                   (src/misfit/misfit.cu:219-259 is racy);
 *   - assignment  = edges arrive in ascending sub-batch index, so each
 *                   cluster list is walked in descending index
 *                   (src/misfit/misfit.cu:261-275);
 *   - processing  = clusters run one after another in ascending id
 *                   (src/misfit/misfit.cu:277-349 is racy across clusters).
 * Every other step (overlay semantics, parse-time flags, the sub-batch split
 * and its MAX_CSR_ELEMENTS growth, 2-hop BFS order, stale cluster ids, the
 * 2*MAX_BATCH_SIZE row cap) follows the reference exactly.
 */
#ifndef MISFIT_ORACLE_H
#define MISFIT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_graph or_graph;

/* Build from an in-memory CSR (copied).  nindex has n+1 entries. */
or_graph* or_create(int32_t n, const int64_t* nindex, const int32_t* nlist);
/* Read a .egr file (int32 or int64-sentinel layout).  NULL on error. */
or_graph* or_open_egr(const char* path);
void or_destroy(or_graph* g);

int32_t or_num_nodes(const or_graph* g);
int64_t or_base_entries(const or_graph* g);
int64_t or_max_csr(const or_graph* g);
void or_set_max_csr(or_graph* g, int64_t v);
/* Exact-MIS mode (no reference counterpart): after each batch's repair, a
 * member with a smaller-id member neighbour leaves, then the uncovered
 * vertices are completed greedily in ascending id. */
void or_set_exact(or_graph* g, int on);
/* Schedule switch for vertex_clustering_csr_kernel: 0 (default) the
 * bulk-synchronous schedule above; 1 the serial one, rows one after another
 * in ascending index, each seeing the writes of the rows before it.  Both are
 * legal runs of the racy kernel; the serial one is what a launch of the
 * reference's kernel with one thread at a time gives. */
void or_set_serial_clustering(or_graph* g, int on);

void or_set_mis(or_graph* g, const uint8_t* mis);
void or_get_mis(const or_graph* g, uint8_t* out);
void or_get_cluster_ids(const or_graph* g, int32_t* out);

/* is_insertion = !isAdjacent(u, v) against the current base+overlay state
 * (core/cli_setup.h:66-82 evaluates it before any batch is applied). */
void or_flag_updates(const or_graph* g, const int32_t* u, const int32_t* v,
                     int64_t m, uint8_t* ins_out);
int or_is_adjacent(const or_graph* g, int32_t u, int32_t v);

/* One batch through the whole path: overlay apply, split, neighbourhoods,
 * clustering, assignment, repair, clear.  Returns the number of sub-batches. */
int64_t or_apply_batch(or_graph* g, const int32_t* u, const int32_t* v,
                       const uint8_t* ins, int64_t m);

/* Overlay row of x (base minus tombstones, then added in insertion order).
 * Returns the row length; writes at most cap entries. */
int64_t or_row(const or_graph* g, int32_t x, int32_t* out, int64_t cap);
int32_t or_degree(const or_graph* g, int32_t x);
/* Exact 2-hop list of s in BFS order (seed first).  Returns its length. */
int64_t or_two_hop(const or_graph* g, int32_t s, int32_t* out, int64_t cap);

/* Per-sub-batch trace of the last or_apply_batch call (when enabled). */
void or_trace_enable(or_graph* g, int on);
int64_t or_trace_count(const or_graph* g);
/* field: 0 header int64[10] = {p, q, n_seeds, n_cands, packed, max_after,
 *                              cluster_count, n_processed, n_rows, est}
 *        1 seeds (int32), 2 candidates (int32),
 *        3 cluster ids after clustering (int32[n]),
 *        4 processed edges in order (int32 batch index),
 *        5 membership after repair (uint8[n]),
 *        6 row lengths in packing order (int64) */
int64_t or_trace_get(const or_graph* g, int64_t i, int field, void* out, int64_t cap);

/* End-of-run compaction into an int64-sentinel .egr (core/flash_compactor.h). */
int or_compact(const or_graph* g, const char* out_path);

/* Greedy MIS in vertex order (tools/compute_initial_mis.py:32-43). */
void or_greedy_mis(int32_t n, const int64_t* nindex, const int32_t* nlist, uint8_t* out);

/* CPU baseline of a from-scratch recompute: the batch applied to the overlay
 * only (no repair), then the greedy MIS of tools/compute_initial_mis.py over
 * the whole current graph (written as the membership). */
void or_apply_overlay(or_graph* g, const int32_t* u, const int32_t* v, const uint8_t* ins, int64_t m);
void or_greedy_current(or_graph* g);

/* Counters of the last batch: independence violations and vertices that are
 * neither in the MIS nor adjacent to one, on the current overlay graph. */
void or_check_mis(const or_graph* g, int64_t* violations, int64_t* non_maximal);

#ifdef __cplusplus
}
#endif

#endif
