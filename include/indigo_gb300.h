/*
 * indigo_gb300.h -- C ABI of the GB300 (sm_103a) graph-analytics library.
 *
 * The library replaces the CUDA hot path of the Indigo2 suite
 * (yiqianl/Parallelization-Artifact-SC23): BFS, SSSP, connected components,
 * maximal independent set, PageRank and triangle counting over the ECLgraph
 * CSR format.  Every drop-in entry point below keeps the argument meaning
 * and the pointer residency (host or device) of the reference entry
 * function it replaces; the reference file:line is given beside each one.
 *
 * Conventions
 *   - Every call returns an ig_status; nothing calls exit().  The text of the
 *     last error on the calling thread is returned by ig_last_error().
 *   - Vertex and edge indices are int32, as in struct ECLgraph.
 *   - "d_" pointers are device pointers, "h_" pointers are host pointers.
 *   - Drop-in calls are synchronous and run on a library-owned stream of the
 *     current device; the seconds they report cover the device work of the
 *     algorithm (including any per-call preprocessing it needs), measured
 *     with CUDA events, and exclude the copy of the result back to the host,
 *     as the reference drivers' timers do.
 *   - Device-API calls (ig_graph_*) are asynchronous on the graph's stream.
 *   - Device kernels never wait without a bound: a grid barrier that does not
 *     complete within the configured timeout makes the call return
 *     IG_ERR_TIMEOUT and leaves the context usable.
 */
#ifndef INDIGO_GB300_H
#define INDIGO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IG_VERSION 1

typedef enum ig_status {
  IG_OK = 0,
  IG_ERR_INVALID_ARG = 1,  /* null pointer, negative size, source out of range */
  IG_ERR_CUDA = 2,         /* a CUDA runtime call failed */
  IG_ERR_NOMEM = 3,        /* device or host allocation failed */
  IG_ERR_TIMEOUT = 4,      /* a bounded device-side wait ran out */
  IG_ERR_UNSORTED = 5,     /* TC precondition: adjacency not strictly sorted */
  IG_ERR_NO_DEVICE = 6,    /* no CUDA device visible */
  IG_ERR_OVERFLOW = 7,     /* a device work queue or a count overflowed */
  IG_ERR_IO = 8,           /* .egr file could not be opened / read / written */
  IG_ERR_FORMAT = 9,       /* .egr contents inconsistent */
  IG_ERR_BUSY = 10,        /* serving queue full / admission refused */
  IG_ERR_CANCELLED = 11    /* serving request cancelled */
} ig_status;

/* Layout-compatible with struct ECLgraph (include/ECLgraph.h:44-50). */
typedef struct ig_csr {
  int nodes;
  int edges;
  int* nindex;   /* nodes + 1 */
  int* nlist;    /* edges */
  int* eweight;  /* edges, or NULL */
} ig_csr;

const char* ig_status_string(int status);
const char* ig_last_error(void);
int ig_version(void);

/* ---------------------------------------------------------------------------
 * Host graph utilities (no GPU needed)
 * ------------------------------------------------------------------------ */

/* Reads a binary .egr file; same format and checks as readECLgraph
 * (include/ECLgraph.h:52-80): int nodes, int edges, nindex[nodes+1],
 * nlist[edges], optional eweight[edges] (eweight = NULL when absent).
 * Arrays are malloc'ed; release with ig_csr_free_host. */
int ig_egr_read(const char* path, ig_csr* out);
/* Writes a .egr file (include/ECLgraph.h:82-96). */
int ig_egr_write(const char* path, const ig_csr* g);
/* Frees host arrays (include/ECLgraph.h:98-106). */
void ig_csr_free_host(ig_csr* g);

/* Deterministic synthetic generators.  All produce a symmetric, sorted,
 * duplicate- and self-loop-free CSR with symmetric int32 weights uniform in
 * [1, maxw] (maxw <= 0: no weights).  Arrays are malloc'ed. */
int ig_gen_grid2d(int nx, int ny, int maxw, uint64_t seed, ig_csr* out);
int ig_gen_rmat(int scale, int edge_factor, double a, double b, double c,
                uint64_t seed, int maxw, int permute, ig_csr* out);
/* nx x ny 4-neighbour grid with a fraction of grid edges deleted and
 * shortcut_frac * (grid edges) random long-range undirected shortcuts. */
int ig_gen_road(int nx, int ny, double delete_frac, double shortcut_frac,
                uint64_t seed, int maxw, ig_csr* out);
int ig_gen_er(int n, double avg_degree, uint64_t seed, int maxw, ig_csr* out);
/* Relabels vertices by ascending (degree, id); adjacency re-sorted. */
int ig_degree_order(const ig_csr* in, ig_csr* out);
/* k distinct vertices with degree > 0, drawn from seed. */
int ig_pick_sources(const ig_csr* g, int k, uint64_t seed, int* out);
/* IG_OK if every adjacency list is strictly increasing (sorted, no duplicate,
 * no self loop test is separate); IG_ERR_UNSORTED otherwise.  Mirrors the
 * check in include/tc_vertex_cuda.h:157-165. */
int ig_csr_check_sorted(const ig_csr* g);
/* FNV-1a 64 digest of (nodes, edges, nindex, nlist, eweight). */
uint64_t ig_csr_digest(const ig_csr* g);

/* ---------------------------------------------------------------------------
 * Device memory plumbing (for callers without their own CUDA runtime)
 * ------------------------------------------------------------------------ */
int ig_device_count(int* n);
int ig_set_device(int device);
int ig_device_name(char* buf, int len);
/* Free and total device memory of the current device, in bytes
 * (cudaMemGetInfo). */
int ig_device_memory(unsigned long long* free_bytes, unsigned long long* total_bytes);
int ig_dev_alloc(void** ptr, size_t bytes);
int ig_dev_free(void* ptr);
int ig_host_alloc_pinned(void** ptr, size_t bytes);
int ig_host_free_pinned(void* ptr);
/* kind: 1 = host->device, 2 = device->host, 3 = device->device */
int ig_memcpy(void* dst, const void* src, size_t bytes, int kind);
int ig_memcpy_async(void* dst, const void* src, size_t bytes, int kind, void* stream);
int ig_memset(void* dst, int value, size_t bytes);
int ig_device_synchronize(void);
/* Copies a host CSR to new device arrays (d->nodes/edges set, eweight may be NULL). */
int ig_csr_upload(const ig_csr* h, ig_csr* d);
int ig_csr_free_device(ig_csr* d);
/* Device-side preparation of a graph already on the device (no counterpart
 * in the reference, which prepares its inputs offline): self loops dropped,
 * duplicate edges merged (the smallest weight kept), every adjacency list
 * sorted -- the input contract of the drivers (include/ECLgraph.h) and the
 * triangle-counting precondition (include/tc_vertex_cuda.h:157-165).  Flags:
 * IG_PREP_SYMMETRIZE adds the reverse of every edge (same weight);
 * IG_PREP_DEGREE_ORDER relabels the vertices in ascending (degree, id) order
 * as ig_degree_order does on the host.  *d_out receives new device arrays
 * (free them with ig_csr_free_device); the input is not changed.  Synchronous;
 * temporary device memory of about 26 bytes per (symmetrised) edge. */
enum { IG_PREP_SYMMETRIZE = 1, IG_PREP_DEGREE_ORDER = 2 };
int ig_csr_prepare(const ig_csr* d_in, int flags, ig_csr* d_out);
/* CUDA events and streams as opaque handles. */
int ig_stream_create(void** stream);
/* A stream that is not ordered with the legacy default stream (host code must
 * order its work with events or synchronize calls): for copies that should
 * overlap the synchronous drop-in calls. */
int ig_stream_create_nonblocking(void** stream);
int ig_stream_destroy(void* stream);
int ig_stream_synchronize(void* stream);
int ig_event_create(void** ev);
int ig_event_destroy(void* ev);
int ig_event_record(void* ev, void* stream);
int ig_event_elapsed_ms(void* start, void* stop, float* ms);
/* Bound (milliseconds) on every device-side wait; default 5000. */
int ig_set_wait_timeout_ms(int ms);
/* Kernel tuning knobs (process-wide): blocks_per_sm, bfs_alpha (0: top-down
 * only), bfs_beta, bfs_bitmap, bfs_bu_claim, bfs_hub_degree, hub_degree,
 * sssp_delta, sssp_delta_scale, sssp_heavy_split, sssp_item_edges,
 * sssp_warp_degree, sssp_window_scale, sssp_window_degree, sssp_merge_below,
 * sssp_spin_ns, sssp_pair_slices, sssp_stage_flags, sssp_chunk,
 * sssp_item_group, sssp_static_pct, sssp_tail_split, sssp_claim_ahead,
 * sssp_expanded_check, mis_static_pct, pr_hub_degree, pr_chunk,
 * pr_blocks_per_sm, pr_prefetch, pr_subwarp, pr_static_pct, pr_two_pass,
 * tc_block_chunk, tc_grab, tc_warp_list, tc_runs, cc_bfs_seed,
 * cc_bfs_levels, cc_rounds.  Every setting gives the same results (PageRank:
 * within its tolerance; the gather forms differ in summation order); they
 * trade speed. */
int ig_set_option(const char* name, long long value);
int ig_get_option(const char* name, long long* value);
/* Number of kernels this library has launched in the process. */
int ig_kernel_launches(long long* n);

/* ---------------------------------------------------------------------------
 * Drop-in entry points (same arguments and pointer residency as the
 * reference entry functions; the shims in shim/ forward to these).
 * ------------------------------------------------------------------------ */

/* Replaces  static double GPUbfs_vertex(const int src, const ECLgraph& g,
 * basic_t* const dist)   include/bfs_vertex_cuda.h:61.
 * d_g: device nindex/nlist; h_dist: host int[nodes], INT_MAX = unreachable. */
int ig_bfs_vertex(int src, const ig_csr* d_g, int* h_dist, double* seconds);

/* Replaces  static double GPUsssp_vertex(const int src, const ECLgraph& g,
 * basic_t* const dist)   include/sssp_vertex_cuda.h:60.
 * d_g: device nindex/nlist/eweight (weights >= 0); h_dist host int[nodes]. */
int ig_sssp_vertex(int src, const ig_csr* d_g, int* h_dist, double* seconds);

/* Replaces  static double GPUcc_vertex(const ECLgraph& g, basic_t* const
 * label)   include/cc_vertex_cuda.h:57.  h_label[v] = minimum vertex id of
 * v's component (the fixed point of the reference's min-label propagation). */
int ig_cc_vertex(const ig_csr* d_g, int* h_label, double* seconds);

/* Replaces  static double GPUmis_vertex(const ECLgraph& g, data_type* const
 * priority, int* const status)   include/mis_vertex_cuda.h:54.
 * h_status[v] = 1 (in the set) or 2 (excluded).  Priorities are the
 * reference hash of v + 712313887 compared as unsigned int with the vertex id
 * as tie-break, as in codes/cpp/mis-cpp/MIS_CPP_V_Topo_Push_IntType_Atomic_
 * CopyDeterm_Block.cpp:61-73.  h_priority (may be NULL) receives the hash. */
int ig_mis_vertex(const ig_csr* d_g, unsigned int* h_priority, int* h_status,
                  double* seconds);

/* Replaces  void PR_GPU(const ECLgraph g, score_type* scores, int* degree)
 * include/pr_cuda.h:48.  h_g: HOST CSR (uploaded by the call, as PR_GPU
 * does); h_scores: in/out float[nodes]; h_degree: host int[nodes].
 * Stops when the FP64 sum of |new - old| < epsilon or after max_iter
 * iterations (reference: EPSILON 1e-4, MAX_ITER 100, include/pr_cuda.h:42-46).
 * Each iteration is a Jacobi step score[v] = (1-d)/V + d * sum score[u]/deg[u]
 * with d = 0.85. */
int ig_pr(const ig_csr* h_g, float* h_scores, const int* h_degree,
          float epsilon, int max_iter, int* iterations, double* seconds);

/* Replaces  static double GPUtc_vertex(basic_t& count, const int nodes,
 * const int* const nindex, const int* const nlist)
 * include/tc_vertex_cuda.h:42.  d_nindex/d_nlist: device; count is 64-bit
 * (the reference's int can overflow).  Requires sorted, self-loop-free
 * adjacency, else IG_ERR_UNSORTED. */
int ig_tc_vertex(long long* count, int nodes, const int* d_nindex,
                 const int* d_nlist, double* seconds);

/* Edge-centric forms (include/<algo>_edge_cuda.h).  sp is the COO source array
 * the reference drivers build (sp[e] = source vertex of edge e); residency as
 * in the reference: host for BFS/SSSP/CC (e.g. include/sssp_edge_cuda.h:60,
 * 149-155), device for MIS (include/mis_edge_cuda.h:154-161) and TC
 * (include/tc_edge_cuda.h:42).  Results are identical to the vertex forms. */
int ig_bfs_edge(int src, const ig_csr* d_g, int* h_dist, const int* h_sp, double* seconds);
int ig_sssp_edge(int src, const ig_csr* d_g, int* h_dist, const int* h_sp, double* seconds);
int ig_cc_edge(const ig_csr* d_g, int* h_label, const int* h_sp, double* seconds);
int ig_mis_edge(const ig_csr* d_g, const int* d_sp, unsigned int* h_priority,
                int* h_status, double* seconds);
int ig_tc_edge(long long* count, int edges, const int* d_nindex, const int* d_nlist,
               const int* d_sp, double* seconds);

/* No counterpart in the reference.  BFS for callers that cannot allocate
 * device memory (a host framework owns the memory budget, or the call sits
 * where the allocator must not be touched): the caller passes the device
 * graph (d_g, device nindex/nlist) and the device output d_dist[nodes]; the
 * kernel's scratch is a fixed array inside the library's device image
 * (12 MiB per GPU, held until exit), so graphs are limited to 1,048,576
 * vertices (IG_ERR_INVALID_ARG beyond).  Runs on `stream` (NULL: legacy
 * default), reads back a status word and synchronizes `stream` before it
 * returns, so it must never be called on a stream that is being captured.
 * No cudaMalloc or cudaFree is made.  The first call on a device resolves
 * the array's address with cudaGetSymbolAddress.  That address is kept for
 * the process's life, so after
 * cudaDeviceReset the entry point must not be called on that device again.
 * Calls share the array, so calls whose GPU work overlaps race; order them.
 * Errors are reported as by ig_bfs_vertex, whose results it reproduces. */
int ig_bfs_vertex_noalloc(int src, const ig_csr* d_g, int* d_dist, void* stream);

/* ---------------------------------------------------------------------------
 * Device-resident API: a graph already in HBM, results written to device
 * buffers, asynchronous on the graph's stream.  Scratch is allocated once
 * per graph handle and reused by every call.
 * ------------------------------------------------------------------------ */
typedef struct ig_graph ig_graph;

typedef struct ig_run_info {
  int status;         /* ig_status of the last run on this graph */
  int iterations;     /* BFS levels, SSSP near iterations, MIS rounds, PR iterations */
  long long work;     /* SSSP: distance improvements */
  double residual;    /* PR: last L1 residual */
  long long aux[4];   /* SSSP: far-pile splits, frontier vertices, edges expanded, - */
} ig_run_info;

/* Binds caller-owned device CSR arrays (not copied, not freed). */
int ig_graph_create(const ig_csr* d_g, ig_graph** out);
int ig_graph_destroy(ig_graph* g);
int ig_graph_stream(ig_graph* g, void** stream);
/* Runs the graph's later calls on `stream` (NULL: its own stream), so that
 * several graph handles can share one stream and one event timeline. */
int ig_graph_set_stream(ig_graph* g, void* stream);
/* Synchronises the graph's stream and reports the last run. */
int ig_graph_last_run(ig_graph* g, ig_run_info* info);

int ig_bfs(ig_graph* g, int src, int* d_dist);
int ig_sssp(ig_graph* g, int src, int* d_dist);
int ig_cc(ig_graph* g, int* d_label);
int ig_mis(ig_graph* g, int* d_status);
/* d_scores: in/out; d_degree may be NULL (derived from nindex). */
int ig_pagerank(ig_graph* g, float* d_scores, float epsilon, int max_iter);
/* d_count: device unsigned long long, overwritten. */
int ig_tc(ig_graph* g, unsigned long long* d_count);

/* ---------------------------------------------------------------------------
 * Batched form: many graphs packed as one disjoint union (no counterpart in
 * the reference, which runs one program per graph).  d_union: device CSR of
 * the union with global vertex ids; d_graph_vptr: device int[graphs+1], the
 * first global vertex of each graph (d_graph_vptr[graphs] = d_union->nodes).
 * Each algorithm is one launch sequence, captured into a CUDA graph on its
 * second call and replayed afterwards; calls are asynchronous on the batch's
 * stream.  Results equal the per-graph drop-in calls.
 * ------------------------------------------------------------------------ */
typedef struct ig_batch ig_batch;
int ig_batch_create(const ig_csr* d_union, const int* d_graph_vptr, int graphs, ig_batch** out);
int ig_batch_destroy(ig_batch* b);
int ig_batch_stream(ig_batch* b, void** stream);
/* 0: plain launches instead of CUDA-graph replay (for comparison). */
int ig_batch_use_graphs(ig_batch* b, int enable);
int ig_batch_last_run(ig_batch* b, ig_run_info* info);
/* BFS levels of every graph from d_sources[g] (global ids; NULL: local
 * vertex 0 of each graph); d_dist[v] indexed by global vertex. */
int ig_batch_bfs(ig_batch* b, const int* d_sources, int* d_dist);
/* Per-graph min-id component labels, as LOCAL ids, indexed by global vertex. */
int ig_batch_cc(ig_batch* b, int* d_label);
/* Triangles per graph: d_counts[g] (device unsigned long long[graphs]). */
int ig_batch_tc(ig_batch* b, unsigned long long* d_counts);
/* PageRank of every graph with its own (1-d)/V_g and its own stop rule;
 * d_scores in/out by global vertex; d_iters[g] receives the iterations. */
int ig_batch_pagerank(ig_batch* b, float* d_scores, float epsilon, int max_iter, int* d_iters);
/* Autotuning of the batched form (no reference counterpart): for each
 * algorithm in algo_mask (bit 0 BFS, 1 CC, 2 TC, 3 PageRank) times a small set
 * of variants on this batch -- blocks per SM, grid-expansion thresholds
 * (thread / warp / grid granularity), BFS push-pull against push-only levels
 * and bitmap against distance tests in its pull levels, CC linking in one
 * pass or in rounds, PageRank medium lists by warps or 8-lane sub-warps;
 * never a change of results -- best of `reps` runs each, and keeps the
 * fastest for the batch's later calls.  best_ms[4] (may be NULL) receives the chosen
 * variant's time per algorithm (-1 where not tuned).  Synchronous. */
int ig_batch_autotune(ig_batch* b, int algo_mask, int reps, float* best_ms);
/* The option value the batch uses for `algo` (0..3): the tuned one, else the
 * process-wide value (names as in ig_get_option). */
int ig_batch_get_option(ig_batch* b, int algo, const char* name, long long* value);
/* Sets one option for this batch's calls of algorithm `algo` (0 BFS, 1 CC,
 * 2 TC, 3 PageRank; names as ig_set_option); a captured call is captured
 * again.  Used to apply a stored tuning without timing. */
int ig_batch_set_option(ig_batch* b, int algo, const char* name, long long value);
/* Host generator of a batch: `graphs` graphs with vertex counts log-uniform
 * in [vmin, vmax]; even indices Erdos-Renyi (average degree er_degree), odd
 * ones RMAT (a, b, c; rmat_edge_factor pairs per vertex, ids taken modulo the
 * vertex count), each symmetric, sorted, simple, weights in [1, maxw];
 * returned packed as a union CSR (malloc'ed) and out_vptr[graphs+1]. */
int ig_gen_batch(int graphs, int vmin, int vmax, double er_degree, int rmat_edge_factor, double a, double b,
                 double c, uint64_t seed, int maxw, ig_csr* out_union, int* out_vptr);

/* ---------------------------------------------------------------------------
 * Served form: BFS / SSSP queries against a resident graph (no counterpart
 * in the reference).  A worker thread answers them with 64-lane multi-source
 * traversals; queries join free lanes at every step and leave when done
 * (continuous batching).  A query returns summary results, not the full
 * distance vector: vertices reached, the largest finite distance, the sum of
 * the finite distances and the distances to up to 16 requested targets.
 * ------------------------------------------------------------------------ */
typedef struct ig_server ig_server;
typedef struct ig_query_result {
  int status;              /* IG_OK or the failure of the serving worker */
  int kind;                /* 0 BFS, 1 SSSP */
  int source;
  int levels;              /* BFS: max_dist + 1; SSSP: rounds the engine ran */
  long long reached;       /* vertices reached, the source included */
  long long max_dist;      /* largest finite distance */
  long long sum_dist;      /* sum of the finite distances */
  int ntargets;
  int targets[16];
  int target_dist[16];     /* INT_MAX: unreachable */
  double submit_time;      /* seconds, steady clock */
  double admit_time;
  double done_time;
} ig_query_result;
/* d_g: device graph (eweight needed for SSSP queries); the graph stays
 * resident and caller-owned.  max_pending bounds the admission queue.
 * Queries are admitted by device memory: an engine's lane state (BFS: 44
 * bytes per vertex; SSSP: about 300) is allocated when a query of its kind
 * is pending and free device memory (less an eighth in reserve) and the
 * budget below cover it; otherwise the query stays pending (deferred) until
 * memory frees up -- an idle engine of the other kind is released to make
 * room.  A query whose engine can never fit completes with status
 * IG_ERR_NOMEM.  Fails with IG_ERR_NOMEM when even the BFS engine does not
 * fit in free device memory at creation. */
int ig_server_create(const ig_csr* d_g, int max_pending, ig_server** out);
/* kind 0 BFS, 1 SSSP; IG_ERR_BUSY when max_pending queries are waiting. */
int ig_server_submit(ig_server* s, int kind, int source, const int* targets, int ntargets, long long* ticket);
int ig_server_wait(ig_server* s, long long ticket, int timeout_ms, ig_query_result* out);
int ig_server_stats(ig_server* s, long long* completed, long long* steps);
/* Caps the bytes the engines may hold together (-1: no cap beyond free device
 * memory); takes effect at the next admission. */
int ig_server_set_memory_budget(ig_server* s, long long bytes);
/* Bytes the engines hold now, admissions deferred for lack of memory so far,
 * engines created so far (a release and a new creation count again). */
int ig_server_memory(ig_server* s, long long* held_bytes, long long* deferrals, long long* engines_created);
int ig_server_destroy(ig_server* s);

/* ---------------------------------------------------------------------------
 * Self-test (no counterpart in the reference, whose waits are host-side)
 * ------------------------------------------------------------------------ */
/* Calibration (no reference counterpart): rate of random 4-byte reads of a
 * table of table_elems floats (< 2^32), `gathers` reads per run, best of
 * `reps` runs, in reads per second.  A table the size of a per-vertex array
 * stays in L2, one larger than L2 is read from HBM.  It is the ceiling of the
 * graph kernels' data-dependent reads (each moves a 32-byte sector). */
int ig_probe_random_gather(long long table_elems, long long gathers, int reps, double* gathers_per_s);
/* Launches a persistent kernel in which one block never reaches the grid
 * barrier and reports, in *observed_status, the status the others' bounded
 * wait produced (IG_ERR_TIMEOUT when the bound works). */
int ig_selftest_wait_timeout(int timeout_ms, int* observed_status);

#ifdef __cplusplus
}
#endif

#endif /* INDIGO_GB300_H */
