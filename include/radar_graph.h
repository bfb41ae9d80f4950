/*
 * radar_graph.h -- C ABI of the GB300 frontier engine (librg.so).
 *
 * The library replaces the data-parallel hot path of RADAR-Graph: the
 * Ligra-style edgeMap/vertexMap engine (sparse push, dense push, pull) and the
 * PageRank, BFS, BC and Radii apps that drive it, in their push, push-pull,
 * DegreeSorting, HUBDUP and RADAR variants.  Paths below are relative to the
 * reference project root (RADAR variant unless another is named).
 *
 * Conventions
 *  - Every call returns rg_status; RG_OK is 0.  Nothing aborts the process
 *    (the reference abort()s / exit()s, e.g. ligra.h:285-288, IO.h:95-115).
 *    rg_last_error() gives a one-line message for the calling thread.
 *  - Vertex ids and edge offsets are uint32_t (Ligra's uintE/uintT without
 *    -DLONG/-DEDGELONG, parallel.h:100-123); graphs with >= 2^32 directed
 *    edges are refused with RG_EUNSUPPORTED.
 *  - Pointers named h_* are host memory, d_* device memory.  `stream` is a
 *    cudaStream_t passed as void* (NULL = the library's own stream).
 *  - Ids passed to and returned from the app entry points are ORIGINAL ids:
 *    when the graph was degree-sorted the library maps inputs (roots, sources)
 *    and outputs through new_ids exactly as the reference apps do
 *    (BFS.C:126-129, Radii.C:163-165, writeOutputToFile in every app), except
 *    BFS parent VALUES, which stay in the graph's internal id space as in the
 *    reference.
 */
#ifndef RADAR_GRAPH_H
#define RADAR_GRAPH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum rg_status {
  RG_OK = 0,
  RG_EINVAL = 1,        /* bad argument: null pointer, id out of range, size mismatch */
  RG_ENOMEM = 2,        /* device or host allocation failed */
  RG_ECUDA = 3,         /* a CUDA call failed */
  RG_EIO = 4,           /* a file could not be opened or read */
  RG_EFORMAT = 5,       /* malformed input ("Bad input file", IO.h:235-248) */
  RG_EUNSUPPORTED = 6,  /* option or size the engine does not implement */
  RG_ETIMEOUT = 7,      /* a bounded wait ran out (rg_server_wait_for) */
  RG_ENODEV = 8,        /* no usable CUDA device */
  RG_ECANCELED = 9      /* the query was cancelled (rg_server_cancel) */
} rg_status;

/* The five reference variants (src/<variant>/). */
typedef enum rg_variant {
  RG_PUSH = 0,       /* push-new-orig: every app pushes (dense_forward) */
  RG_PUSH_PULL = 1,  /* push-pull: dense iterations pull (edgeMapDense) */
  RG_DEGSORT = 2,    /* degree-sorting: push on a degree-sorted graph */
  RG_HUBDUP = 3,     /* hubdup: push, hub accumulators privatised (bitmap + index map) */
  RG_RADAR = 4       /* RADAR: degree sort + hubs privatised, hub <=> id < numHubs */
} rg_variant;

typedef struct rg_graph rg_graph;       /* device-resident CSR image (+ permutation) */
typedef struct rg_frontier rg_frontier; /* device frontier: id queue + bitmap */

/* Work of the calling thread goes to `stream` (a cudaStream_t; NULL = the
 * thread's own non-blocking stream, the default).  Each thread has its own
 * scratch, so threads working on one resident graph run concurrently. */
rg_status rg_set_stream(void* stream);

const char* rg_last_error(void);
const char* rg_status_str(rg_status s);
/* Library version string, e.g. "radar-graph-gb300 0.1 sm_103a". */
const char* rg_version(void);

/* ------------------------------------------------------------------------
 * Input formats and graph construction (host side; IO.h:207-632)
 * ------------------------------------------------------------------------ */

/* Seeded R-MAT (uniform=0: a=0.57 b=0.19 c=0.19) or Erdos-Renyi (uniform=1)
 * edge list of 2^scale vertices and edge_factor * 2^scale edges, following
 * the GAP generator (GAP/src/generator.h:52-114): 2^18-edge blocks, block b
 * draws from mt19937 seeded with seed+b, then ids are permuted with an
 * mt19937(seed) shuffle.  h_src/h_dst hold edge_factor<<scale entries. */
rg_status rg_generate_edges(int scale, int edge_factor, uint64_t seed, int uniform,
                            uint32_t* h_src, uint32_t* h_dst);

/* Symmetric CSR from an edge list: both directions of every edge, then per
 * vertex sort + unique + self-loop removal exactly like the symmetric text
 * loader (IO.h:429-474).  *h_off_out (n+1) and *h_adj_out are malloc'ed by
 * the library; release them with rg_host_free. */
rg_status rg_csr_from_edges(int64_t n, int64_t num_edges, const uint32_t* h_src,
                            const uint32_t* h_dst, uint32_t** h_off_out,
                            uint32_t** h_adj_out, int64_t* m_out);

/* Ligra AdjacencyGraph text: "AdjacencyGraph\n n\n m\n offsets[n]\n edges[m]"
 * (IO.h:231-268).  write: h_off has n+1 entries. */
rg_status rg_write_adjacency(const char* path, int64_t n, int64_t m, const uint32_t* h_off,
                             const uint32_t* h_adj);
/* Reads a Ligra text graph (binary=0) or the binary .config/.adj/.idx triple
 * (binary=1, IO.h:477-626) and applies the reference loader's per-list
 * clean-up (sort, unique, drop self loops): IO.h:429-474 for symmetric = 1,
 * the out-lists of a directed graph for symmetric = 0 (IO.h:287-345; pass them
 * to rg_graph_create_directed).  Text only: the binary reader does no clean-up
 * in the reference either.  Result arrays as in rg_csr_from_edges. */
rg_status rg_read_graph(const char* path, int symmetric, int binary, int64_t* n_out,
                        int64_t* m_out, uint32_t** h_off_out, uint32_t** h_adj_out);
/* Reads a GAP serialized graph (.sg, GAP/src/reader.h:251-304): bool
 * directed, int64 directed-entry count, int64 n, int64 offsets[n+1], int32
 * neighbours (a directed graph may follow with its in-lists).  GAP's builder
 * already cleaned it, so the out-lists are returned as is (bounds-checked).
 * *directed_out tells which graph it is (pass the lists to
 * rg_graph_create_directed for a directed one); with directed_out NULL a
 * directed file gives RG_EUNSUPPORTED.  Result arrays as in
 * rg_csr_from_edges. */
rg_status rg_read_sg(const char* path, int64_t* n_out, int64_t* m_out, uint32_t** h_off_out,
                     uint32_t** h_adj_out, int* directed_out);
/* Reads a GAP text edge list, the format chosen by the suffix as GAP's
 * Reader::ReadFile does (GAP/src/reader.h:50-248): .el "u v"; .wel "u v w";
 * .gr DIMACS "a u v w" lines; .graph METIS (1-based lists, fmt 0/1/100);
 * .mtx MatrixMarket coordinate (1-based; symmetric adds both directions).
 * Weights are skipped.  n = largest id + 1 (builder.h:74-83).  The edges
 * come back as read -- repeats, self loops and one direction only -- for
 * rg_csr_from_edges / rg_graph_create_from_edges (symmetric, GAP's -s) or
 * rg_graph_create_directed_from_edges to clean up.  *h_src_out and
 * *h_dst_out are released with rg_host_free. */
rg_status rg_read_edges(const char* path, int64_t* n_out, int64_t* num_edges_out, uint32_t** h_src_out,
                        uint32_t** h_dst_out);
void rg_host_free(void* p);

/* ------------------------------------------------------------------------
 * Device graph (graph.h:57-87 / vertex.h:188-274)
 * ------------------------------------------------------------------------ */

/* Uploads a symmetric CSR (h_off: n+1, h_adj: m) to the current device. */
rg_status rg_graph_create(int64_t n, int64_t m, const uint32_t* h_off, const uint32_t* h_adj,
                          rg_graph** out);
/* Builds the symmetric CSR on the device from an edge list (src/dst:
 * num_edges ids < n, on the device when on_device != 0, else host arrays):
 * both directions of every edge, neighbour lists sorted, repeats and self
 * loops dropped -- the symmetric loader's clean-up (IO.h:429-474), the same
 * result as rg_csr_from_edges + rg_graph_create, computed by device radix
 * sorts instead of on the host. */
rg_status rg_graph_create_from_edges(int64_t n, int64_t num_edges, const uint32_t* src,
                                     const uint32_t* dst, int on_device, rg_graph** out);
/* A DIRECTED graph from its cleaned out-lists (h_off: n+1, h_adj: m, e.g.
 * from rg_read_graph with symmetric = 0); the in-lists (the reference's CSC,
 * IO.h:287-345) are built on the device.  Pushes follow out-edges, pulls read
 * in-edges, and BC transposes per source as BC-manyiter-v2.C:334 does.
 * Triangle counting takes undirected graphs only. */
rg_status rg_graph_create_directed(int64_t n, int64_t m, const uint32_t* h_off, const uint32_t* h_adj,
                                   rg_graph** out);
/* A DIRECTED graph built on the device from an edge list (src -> dst, ids
 * < n; device arrays when on_device != 0): out-lists sorted, repeats and self
 * loops dropped (the directed loader's per-list clean-up, IO.h:287-345), then
 * the in-lists as in rg_graph_create_directed. */
rg_status rg_graph_create_directed_from_edges(int64_t n, int64_t num_edges, const uint32_t* src,
                                              const uint32_t* dst, int on_device, rg_graph** out);
rg_status rg_graph_is_directed(const rg_graph* g, int* directed);
/* rg_graph_create + rg_graph_degree_sort in one call (symmetric graphs),
 * the same graph and permutation: only the offsets are uploaded, and the
 * relabel reads h_adj straight from host memory when the device can (memory
 * from rg_pinned_alloc / cudaHostAlloc, 16-byte aligned), so the unsorted
 * neighbour array never lands in HBM; otherwise it is copied first.  Offsets
 * are checked (monotone, ending at m) and neighbour ids must be < n
 * (RG_EINVAL otherwise). */
rg_status rg_graph_create_sorted(int64_t n, int64_t m, const uint32_t* h_off, const uint32_t* h_adj,
                                 rg_graph** out, uint32_t* h_new_ids);
/* Uploads from arrays already on the device (copied; caller keeps ownership). */
rg_status rg_graph_create_device(int64_t n, int64_t m, const uint32_t* d_off,
                                 const uint32_t* d_adj, rg_graph** out);
/* Degree sort on the device (preprocessGraph, IO.h:843-895): rank vertices by
 * (degree desc, id desc), relabel every neighbour list (order kept).  The new
 * graph remembers new_ids; h_new_ids (n entries, may be NULL) receives it. */
rg_status rg_graph_degree_sort(const rg_graph* g, rg_graph** out, uint32_t* h_new_ids);
/* The same with the key chosen: out-degree (by_out_degree = 1, -preprocess 0)
 * or, for a directed graph, in-degree (0, -preprocess 1, what
 * rg_graph_degree_sort does; IO.h:739-750). */
rg_status rg_graph_degree_sort_by(const rg_graph* g, int by_out_degree, rg_graph** out, uint32_t* h_new_ids);
rg_status rg_graph_info(const rg_graph* g, int64_t* n, int64_t* m, int* degree_sorted);
/* Copies the device CSR back (h_off: n+1, h_adj: m) -- for checking. */
rg_status rg_graph_download(const rg_graph* g, uint32_t* h_off, uint32_t* h_adj,
                            uint32_t* h_new_ids);
rg_status rg_graph_free(rg_graph* g);

/* ------------------------------------------------------------------------
 * Apps: Compute(graph, P) of each reference app.  Outputs are indexed by
 * ORIGINAL vertex id (arr[new_ids[v]] as writeOutputToFile does).
 * ------------------------------------------------------------------------ */

/* PageRank (PageRank.C:120-189): damping 0.85, stop at L1 < 1e-7 or
 * max_iters.  h_ranks: n doubles. */
rg_status rg_pagerank(rg_graph* g, rg_variant variant, int64_t max_iters, double* h_ranks,
                      int64_t* iters_out, double* l1_out);

/* PageRankDelta (PageRankDelta.C:98-155): only vertices whose delta is
 * still above 1% of their rank propagate (vertexFilter); stops at
 * max_iters or when sum |Delta| < 1e-7.  h_ranks: n doubles (original ids),
 * may be NULL; iters_out: the reference's printed round count; l1_out: the
 * last sum |Delta|. */
rg_status rg_pagerank_delta(rg_graph* g, rg_variant variant, int64_t max_iters, double* h_ranks,
                            int64_t* iters_out, double* l1_out);

/* Triangle counting (GAP tc_local, src/<variant>/GAP/src/tc_local.cc): *total_out =
 * number of triangles; h_counts (n, may be NULL) = triangles containing each
 * vertex, by ORIGINAL id (they sum to 3 * total).  Needs a cleaned symmetric
 * graph (the loaders' output).  Works on any graph handle: the degree order
 * with sorted neighbour lists is built internally. */
rg_status rg_triangle_count(rg_graph* g, uint64_t* h_counts, uint64_t* total_out);

/* BFS (BFS.C:122-188) from ORIGINAL id `root` (-r).  h_parents (n, may be
 * NULL): parent in internal id space, UINT32_MAX if unreached.  h_depth (n,
 * may be NULL): BFS depth, -1 if unreached (bit-exact across variants). */
rg_status rg_bfs(rg_graph* g, rg_variant variant, uint32_t root, uint32_t* h_parents,
                 int32_t* h_depth, int64_t* rounds_out, int64_t* reached_out);

/* BC (BC-manyiter-v2.C:205-367): max_iters sources drawn like the reference
 * (mt19937(27491095), uniform over [0,n-1], redrawn on degree 0).  h_deps:
 * n doubles, chained across sources as the reference does (NaN where a
 * source left a vertex unreached). */
rg_status rg_bc(rg_graph* g, rg_variant variant, int max_iters, double* h_deps,
                int64_t* levels_out);
/* Same with an explicit source list (ORIGINAL ids). */
rg_status rg_bc_sources(rg_graph* g, rg_variant variant, const uint32_t* h_sources, int nsrc,
                        double* h_deps, int64_t* levels_out);
/* The sources rg_bc would use (ORIGINAL ids). */
rg_status rg_bc_pick_sources(const rg_graph* g, int k, uint32_t* h_sources);
/* k search roots (ORIGINAL ids) drawn like GAP's SourcePicker
 * (GAP/src/benchmark.h:47-64): mt19937(27491095) with
 * uniform_int_distribution<int32_t> over [0, n-1], redrawn while the vertex
 * has out-degree 0, the k picks continuing one generator. */
rg_status rg_pick_roots(const rg_graph* g, int k, uint32_t* h_roots);

/* Radii (Radii.C:140-218): min(n,64) seeds hashInt(i) % n.  h_radii: n int32
 * (-1 unreached, 0 seed, else last round the vertex's mask grew). */
rg_status rg_radii(rg_graph* g, rg_variant variant, int32_t* h_radii, int64_t* rounds_out);
/* Radii with explicit seeds (ORIGINAL ids, bit i for seeds[i], k <= 64). */
rg_status rg_radii_seeds(rg_graph* g, rg_variant variant, const uint32_t* h_seeds, int k,
                         int32_t* h_radii, int64_t* rounds_out);

/* ------------------------------------------------------------------------
 * Batched execution (no single counterpart in the reference: it runs many
 * BFS sources, or many graphs, per launch; each result equals the reference
 * app's result for that source / graph).
 * ------------------------------------------------------------------------ */

/* BFS from k <= 64 sources (ORIGINAL ids) in one traversal with 64-bit
 * bitmask frontiers (one bit per source, the propagation Radii.C uses).
 * h_depths: k*n int32, row q = depths from sources[q] in original-id order
 * (-1 unreached), equal to rg_bfs(root = sources[q]).  May be NULL. */
rg_status rg_bfs_multi(rg_graph* g, const uint32_t* h_sources, int k, int32_t* h_depths,
                       int64_t* rounds_out);

/* k <= 64 independent single-source BC queries (ORIGINAL ids) in one
 * traversal: the sources' levels from one 64-wide bitmask BFS, then path
 * counts (exact 64-bit integers) and dependencies for all sources per level,
 * one row of k values per vertex.  h_deps: k*n doubles, row q equal to
 * rg_bc_sources(g, variant, &sources[q], 1, row) for every variant (the
 * single-source pass of BC-manyiter-v2.C:180-232) up to summation order;
 * NaN where sources[q] does not reach the vertex.  A graph whose path counts
 * pass 2^64 is answered by one single-source pass per source. */
rg_status rg_bc_multi(rg_graph* g, const uint32_t* h_sources, int k, double* h_deps,
                      int64_t* levels_out);

/* nq <= 16 Radii queries in one traversal: query q samples
 * h_seeds[q*k .. q*k+k) (ORIGINAL ids, k <= 64) and owns word q of a
 * multi-word mask per vertex, so every gather fetches all queries' masks of
 * a neighbour.  h_radii: nq*n int32, row q equal to rg_radii_seeds(g, v,
 * &h_seeds[q*k], k, row) for every variant (Radii.C:140-218 per word). */
rg_status rg_radii_multi(rg_graph* g, const uint32_t* h_seeds, int k, int nq, int32_t* h_radii,
                         int64_t* rounds_out);

/* A set of graphs resident on the device, run by one persistent kernel. */
typedef struct rg_batch rg_batch;
/* Symmetric CSRs (h_offs[i]: ns[i]+1 entries, h_adjs[i]: ms[i]). */
rg_status rg_batch_create(int ngraphs, const int64_t* ns, const int64_t* ms,
                          const uint32_t* const* h_offs, const uint32_t* const* h_adjs,
                          rg_batch** out);
/* One launch: for every graph i, a k-source BFS from h_sources[i*k ..] (graph-local
 * ids) and a PageRank of at most pr_iters iterations.  Outputs (any may be
 * NULL): h_depths = per graph k rows of n_i depths, concatenated in graph
 * order; h_ranks = per graph n_i ranks, concatenated; h_pr_iters = per graph
 * the reference's iteration count; device_ms = the launch's device time. */
rg_status rg_batch_run(rg_batch* b, const uint32_t* h_sources, int k, int64_t pr_iters,
                       int32_t* h_depths, double* h_ranks, int32_t* h_pr_iters, double* device_ms);
rg_status rg_batch_free(rg_batch* b);

/* ------------------------------------------------------------------------
 * Serving: a request loop over resident graphs (no counterpart in the
 * reference).  Worker threads, each with its own stream, run queries as they
 * arrive; BFS queries, and BC queries, waiting for the same graph are
 * coalesced (up to max_batch <= 64) into one multi-source traversal
 * (rg_bfs_multi / rg_bc_multi) when the batch reaches the size at which that
 * beats one traversal per query (measured per graph at creation); a batch is
 * admitted when its estimated device memory fits hbm_fraction of the HBM free
 * at start beside running batches and unfetched results, or when no other
 * batch is running.  Results equal the single-query entry points (BC within 1e-9
 * relative):
 *   RG_QUERY_BFS   source = root (ORIGINAL id) -> int32[n] depths (rg_bfs)
 *   RG_QUERY_BC    source = BC source           -> double[n] (rg_bc_sources
 *                  with that one source)
 *   RG_QUERY_RADII source = seed s: samples hashInt(64*s + i) % n, i < 64
 *                  -> int32[n] radii (rg_radii_seeds with those samples)
 * ------------------------------------------------------------------------ */
typedef struct rg_server rg_server;
typedef enum rg_query_kind { RG_QUERY_BFS = 0, RG_QUERY_BC = 1, RG_QUERY_RADII = 2 } rg_query_kind;
typedef struct rg_server_stats {
  int64_t completed;  /* queries finished since the last reset */
  int64_t launches;   /* traversals run (a coalesced batch is one) */
  int64_t batched;    /* queries answered by a shared multi-source traversal */
  double p50_ms;      /* submit-to-result latency percentiles */
  double p99_ms;
  double qps;         /* completed / (last completion - first submission) */
  int64_t admission_waits; /* batches that waited for HBM budget before running */
  int64_t cancelled;  /* rg_server_cancel calls that took effect */
  int32_t peak_running; /* most batches on the device at once */
} rg_server_stats;
rg_status rg_server_create(rg_graph* const* graphs, int ngraphs, int nworkers, int max_batch,
                           double hbm_fraction, rg_server** out);
rg_status rg_server_submit(rg_server* s, int graph, rg_query_kind kind, uint32_t source,
                           uint64_t* ticket);
/* Blocks until the query is done and copies its result (bytes >= result)
 * from device memory straight into h_result (fastest when h_result comes
 * from rg_pinned_alloc); the result's device memory is then released.
 * RG_ECANCELED if the query was cancelled. */
rg_status rg_server_wait(rg_server* s, uint64_t ticket, void* h_result, size_t bytes,
                         double* latency_ms);
/* rg_server_wait with a limit: RG_ETIMEOUT when the query is not done within
 * timeout_ms (negative = no limit); the ticket stays valid, to be waited on
 * again or cancelled.  The reference has no serving layer; this is the
 * bounded wait its error model lacks (it blocks or aborts). */
rg_status rg_server_wait_for(rg_server* s, uint64_t ticket, void* h_result, size_t bytes,
                             double* latency_ms, double timeout_ms);
/* Cancels a query: a query still waiting never runs; a running one has its
 * result dropped when its batch ends; a finished, unfetched one releases its
 * result now.  A later wait on the ticket returns RG_ECANCELED. */
rg_status rg_server_cancel(rg_server* s, uint64_t ticket);
/* paused != 0: workers take no new queries (running batches finish);
 * 0 resumes.  Queries submitted meanwhile wait in arrival order. */
rg_status rg_server_pause(rg_server* s, int paused);
/* Page-locked host memory for result buffers (cudaHostAlloc). */
rg_status rg_pinned_alloc(size_t bytes, void** h_ptr);
rg_status rg_pinned_free(void* h_ptr);
rg_status rg_server_get_stats(rg_server* s, rg_server_stats* out);
rg_status rg_server_reset_stats(rg_server* s);
/* Finishes the queued queries, stops the workers, frees the server (the
 * graphs stay the caller's). */
rg_status rg_server_free(rg_server* s);

/* ------------------------------------------------------------------------
 * Engine (ligra.h:277-354 edgeMap, 461-493 vertexMap).  The functor of the
 * reference (update/updateAtomic/cond/mergeDuplicates, utils.h:62-79) cannot
 * cross a C ABI, so the operator is a closed enum of device functors that
 * act on caller-owned device arrays.
 * ------------------------------------------------------------------------ */

typedef enum rg_op {
  RG_OP_PAGERANK = 0,  /* p_next[d] += p_curr[s]/deg(s)          (PR_F)        */
  RG_OP_BFS = 1,       /* parents[d] CAS UINT32_MAX -> s           (BFS_F)       */
  RG_OP_BC_FWD = 2,    /* num_paths[d] += num_paths[s] if !visited (BC_F)        */
  RG_OP_BC_BWD = 3,    /* deps[d] += deps[s] if !visited           (BC_Back_F)   */
  RG_OP_RADII = 4      /* next_visited[d] |= visited[s] ...        (Radii_F)     */
} rg_op;

typedef enum rg_vop {
  RG_VOP_PR_DAMP = 0,       /* p_next[i] = 0.85*p_next[i] + 0.15/n  (PR_Vertex_F)      */
  RG_VOP_BC_VISIT = 1,      /* visited[i] = 1                       (BC_Vertex_F)      */
  RG_VOP_BC_BACK = 2,       /* visited[i] = 1; deps[i] += inv[i]    (BC_Back_Vertex_F) */
  RG_VOP_RADII_SYNC = 3     /* visited[i] = next_visited[i]          (Radii_Vertex_F)   */
} rg_vop;

/* Device arrays an operator reads and writes (unused ones may be NULL). */
typedef struct rg_op_args {
  double* p_curr;           /* PR: n */
  double* p_next;           /* PR: n */
  uint32_t* parents;        /* BFS: n */
  double* num_paths;        /* BC forward: n (inverse path counts for RG_VOP_BC_BACK) */
  double* deps;             /* BC backward: n */
  uint32_t* visited_bits;   /* BC: (n+31)/32 words, bit i = visited */
  int64_t* visited;         /* Radii: n masks */
  int64_t* next_visited;    /* Radii: n masks */
  int32_t* radii;           /* Radii: n */
  int32_t round;            /* Radii: current round */
} rg_op_args;

/* edgeMap flags (ligra.h:51-57). */
#define RG_NO_OUTPUT 1u
#define RG_DENSE_FORWARD 8u

rg_status rg_frontier_create(const rg_graph* g, rg_frontier** out);
rg_status rg_frontier_free(rg_frontier* f);
/* Sets the frontier to the given INTERNAL ids (host array, duplicates kept
 * like vertexSubset(n, m, indices)). */
rg_status rg_frontier_set(rg_frontier* f, const uint32_t* h_ids, int64_t k);
rg_status rg_frontier_set_all(rg_frontier* f);
rg_status rg_frontier_count(const rg_frontier* f, int64_t* count);
/* Copies the frontier as a byte map (n bytes, 1 = member). */
rg_status rg_frontier_get(const rg_frontier* f, uint8_t* h_member);

/* One edgeMap over `in`.  out == NULL or flags & RG_NO_OUTPUT: no output.
 * threshold -1 = m/20 (ligra.h:283).  Dense iterations push when flags has
 * RG_DENSE_FORWARD and pull otherwise, as in ligra.h:302-307. */
rg_status rg_edgemap(rg_graph* g, rg_frontier* in, rg_op op, const rg_op_args* args,
                     rg_frontier* out, uint32_t flags, int64_t threshold, void* stream);
rg_status rg_vertexmap(rg_graph* g, rg_frontier* f, rg_vop op, const rg_op_args* args,
                       void* stream);

/* Device buffers for rg_op_args (cudaMalloc'ed, zero-filled). */
rg_status rg_device_alloc(size_t bytes, void** d_ptr);
rg_status rg_device_free(void* d_ptr);
rg_status rg_copy_to_device(void* d_dst, const void* h_src, size_t bytes);
rg_status rg_copy_to_host(void* h_dst, const void* d_src, size_t bytes);
/* Waits for all of the device's work, including result copies left in flight
 * by RG_OPT_ASYNC_RESULTS. */
rg_status rg_synchronize(void);
/* The current device: its name (NUL-terminated, at most name_len bytes), SM
 * count and nominal HBM bandwidth in GB/s (memory clock x bus width x 2). */
rg_status rg_device_info(char* name, int name_len, int32_t* sms, double* nominal_hbm_gbs);

/* ------------------------------------------------------------------------
 * Allocation-free BFS.  No counterpart in the reference: it exists for
 * callers that must not allocate device memory -- code running inside
 * another framework's memory pool, whose allocator owns the device memory,
 * and latency-critical serving loops, where cudaMalloc/cudaFree synchronize
 * the device.  The caller passes a symmetric CSR (d_off: n+1 entries, d_adj:
 * m) and the output d_depth (n int32: BFS depth from `root`, -1 unreached)
 * as device pointers; the function allocates nothing.  Its working memory
 * (two frontier queues, a visited bitmap, a counter) is one fixed 16.25 MiB
 * __device__ array that every GPU loading the library holds until exit, so
 * n is limited to RG_NOALLOC_MAX_VERTICES (larger n -> RG_EINVAL).
 * Preconditions the function cannot check without reading device memory:
 * d_off must be a valid CSR (non-decreasing, d_off[0] = 0, d_off[n] = m);
 * a neighbour id >= n in d_adj is skipped by the kernel (never written
 * through).  Each call looks up the array's device address for the current
 * device (cudaGetSymbolAddress); the first call on a device may also load
 * the library's device code there, so make it before any stream capture.
 * All calls share the array: calls whose work overlaps on the GPU (other
 * streams, other threads) race and must be serialized by the caller.
 * Results equal rg_bfs's depths on the same CSR.
 * ------------------------------------------------------------------------ */
#define RG_NOALLOC_MAX_VERTICES 2097152
rg_status rg_bfs_depth_noalloc(const uint32_t* d_off, const uint32_t* d_adj, int64_t n, int64_t m,
                               uint32_t root, int32_t* d_depth, void* stream, int64_t* rounds_out);

/* ------------------------------------------------------------------------
 * Engine options (per calling thread; a graph tuned by rg_autotune uses its
 * own choice per app instead).  None of them changes any result, only how
 * the work is scheduled.
 * ------------------------------------------------------------------------ */
typedef enum rg_option {
  /* 0 (default): each variant's own direction, as in the reference: push
   * variants push in dense iterations (dense_forward), push-pull pulls.
   * 1: dense iterations pull in every variant (no atomics; BFS exits at the
   * first frontier neighbour; Radii and multi-source BFS OR every neighbour's
   * mask).  Results are identical either way. */
  RG_OPT_DIRECTION = 0,
  /* hub copies per CTA for HUBDUP/RADAR; 0 = as many as the budget allows */
  RG_OPT_HUB_SLOTS = 1,
  /* shared-memory budget for hub copies per CTA of the frontier push, in KiB
   * (default 48; PageRank's full sweeps use one CTA per SM and all of it);
   * 0 = no hub copies (HUBDUP/RADAR then update hubs with global atomics) */
  RG_OPT_HUB_SMEM_KB = 2,
  /* dense iteration when |F| + outdeg(F) > m / value (default 20, ligra.h:283) */
  RG_OPT_DENSE_DIV = 3,
  /* shape of the full-graph PageRank pull sweep: 10 * (edges per lane, 4, 8
   * or 16) + cache mode (0 plain loads; 1 streamed edge array; 2 streamed
   * edge array and gathers kept in L1/L2).  Default 161.  Never changes a
   * result. */
  RG_OPT_SWEEP_SHAPE = 4,
  /* BC's forward (path counting) pushes use hub copies too: 1 (default) or
   * 0 (only the backward pushes do).  The backward phase pushes into the
   * levels that hold the hubs, where the reductions pile up; the forward
   * reaches the hubs in its first levels.  Never changes a result. */
  RG_OPT_BC_FWD_HUBS = 5,
  /* 1: rg_pagerank, rg_bfs, rg_bc, rg_bc_sources, rg_radii and
   * rg_radii_seeds return once their results are staged on the device; the
   * copies into the caller's host buffers run on the thread's copy stream,
   * overlapping the next call, and are complete when rg_synchronize returns
   * (host buffers from rg_pinned_alloc or otherwise page-locked let them
   * overlap; pageable ones are copied before the call returns).  The host
   * buffers must not be read or freed before then.  Scalar outputs (rounds,
   * iterations, L1) are valid at return.  0 (default): every result is in
   * the host buffers when the call returns.  Never changes a result; kept
   * per thread, not per graph (an autotuned schedule does not change it). */
  RG_OPT_ASYNC_RESULTS = 6
} rg_option;
rg_status rg_set_option(rg_option opt, int64_t value);
rg_status rg_get_option(rg_option opt, int64_t* value);

/* Autotuner: times candidate schedules of PageRank (5 iterations), BFS, BC
 * (one source) and Radii on g for `variant` -- direction, dense threshold,
 * hub copies and their shared-memory budget -- and keeps the fastest per app
 * in g; later calls on g use it (instead of the thread's options).
 * best_ms[4] (may be NULL) receives the winners' times.  It and the two
 * setters below change g: no other thread may use g while they run. */
rg_status rg_autotune(rg_graph* g, rg_variant variant, double* best_ms);
/* The tuned value of `opt` for app 0 PageRank, 1 BFS, 2 BC, 3 Radii (-1 if
 * the app is not tuned); rg_graph_clear_tuning forgets every choice. */
rg_status rg_graph_tuned_option(const rg_graph* g, int app, rg_option opt, int64_t* value);
/* Sets one tuned option of app on g (e.g. to reuse a tuning on a copy). */
rg_status rg_graph_set_tuned_option(rg_graph* g, int app, rg_option opt, int64_t value);
rg_status rg_graph_clear_tuning(rg_graph* g);

/* ------------------------------------------------------------------------
 * Timing of the last app call (CUDA events on the launching stream).
 * ------------------------------------------------------------------------ */
typedef struct rg_timing {
  double total_ms;          /* whole app call on the device */
  double edge_ms;           /* time inside edge kernels */
  int64_t edges_traversed;  /* GTEPS numerator: edges examined by the edge maps */
  int64_t algorithmic_bytes;/* compulsory bytes of the app's byte model */
  int64_t edge_launches;    /* launches of the dominant edge kernel */
  int64_t kernel_launches;  /* all kernel launches of the call */
} rg_timing;
rg_status rg_last_timing(rg_timing* t);
/* on != 0: every edge-kernel launch of the following app calls is bracketed
 * by CUDA events on its stream and rg_timing.edge_ms reports their sum. */
rg_status rg_set_kernel_timing(int on);

/* Per-level trace of the calling thread's edgeMaps: the GPU form of Ligra's
 * frontierStats (ligra.h:357-370), which prints PUSH or PULL and the
 * frontier's size per iteration.  While tracing is on (rg_set_trace(1)) each
 * edgeMap of the apps and of rg_edgemap appends one record; rg_trace_take
 * copies up to cap records (oldest first) and clears the list.  Each edgeMap
 * is also an NVTX range ("edgeMap sparse-push", "edgeMap dense-push",
 * "edgeMap pull") for a profiler that records NVTX. */
typedef struct rg_level_trace {
  int32_t mode;       /* 0 sparse push, 1 dense push, 2 pull */
  int32_t hub_mode;   /* push hub copies: 0 none, 1 ids < H (RADAR), 2 hub map (HUBDUP) */
  int64_t frontier;   /* vertices in the input frontier */
  int64_t degsum;     /* their out-degree sum (edges the map examines) */
  int64_t threshold;  /* dense when frontier + degsum > threshold (ligra.h:283) */
} rg_level_trace;
rg_status rg_set_trace(int on);
rg_status rg_trace_take(rg_level_trace* h_out, int64_t cap, int64_t* count);

#ifdef __cplusplus
}
#endif
#endif /* RADAR_GRAPH_H */
