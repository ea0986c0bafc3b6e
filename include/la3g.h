/*
 * la3g.h — C ABI of the GB300-native LA3 vertex-program engine.
 *
 * One GPU, one process.  The library owns all device memory; callers own the
 * host buffers they pass in.  Every call returns an la3g_status; no C++
 * exception crosses this boundary.  la3g_last_error_string() describes the
 * last failure of the calling thread.
 *
 * Vertex ids are the ids of the input file.  A graph loaded with n vertices
 * has nslots = n + 1 slots (ids 0..n; the reference sizes its single tile
 * n + 1 wide, matrix/matrix2d.hpp:6-9); every per-vertex output array has
 * nslots entries indexed by vertex id.  For a bipartite graph
 * n = ndocs + nterms and term t (1-based in the file) is vertex ndocs + t.
 *
 * Threading: a graph handle is not re-entrant; calls on one handle must not
 * overlap.  Different handles may be used from different threads.  The
 * server API (la3g_server_*) is thread-safe for submit/poll.
 *
 * Every entry point below names the reference interface it stands in for.
 * The reference has no C ABI of its own: it is a C++ template library whose
 * plugin API is the VertexProgram<W, M, A, S> class
 * (src/vprogram/vertex_program.h:21-383) driven by the apps' run() functions.
 */
#ifndef LA3G_H
#define LA3G_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum la3g_status
{
  LA3G_OK = 0,
  LA3G_EINVAL = 1,    /* bad argument (null handle, id out of range, wrong graph kind) */
  LA3G_EIO = 2,       /* file cannot be opened or read                                 */
  LA3G_EFORMAT = 3,   /* file is not a whole number of records, or bad header          */
  LA3G_ENOMEM = 4,    /* host or device allocation failed                              */
  LA3G_EBUDGET = 5,   /* server admission: request does not fit the HBM budget         */
  LA3G_ETIMEOUT = 6,  /* a bounded device-side wait ran out                             */
  LA3G_ECUDA = 7,     /* a CUDA runtime call failed                                     */
  LA3G_EBUSY = 8,     /* server queue full / no result ready yet                        */
} la3g_status;

/* Load flags (Graph::load_directed / load_undirected / load_bipartite,
 * src/matrix/graph.h:38-47).  No DIRECTED bit = undirected (each record is
 * stored in both directions, graph.hpp:187-191). */
enum la3g_load_flags
{
  LA3G_DIRECTED = 1u << 0,   /* transpose: messages flow along out-edges (graph.hpp:171-172)   */
  LA3G_REVERSE = 1u << 1,    /* reverse_edges: no transpose                                     */
  LA3G_ACYCLIC = 1u << 2,    /* remove_cycles: orient every edge by original id (:174-179)     */
  LA3G_BIPARTITE = 1u << 3,  /* left = docs 1..n, right = terms shifted by n (:162-163)        */
  LA3G_WEIGHTED = 1u << 4,   /* records are {u32 src, u32 dst, u32 weight} triples              */
};

typedef struct la3g_graph la3g_graph;

typedef struct la3g_graph_info
{
  uint32_t nslots;      /* n + 1                                                  */
  uint32_t nvertices;   /* n                                                      */
  uint32_t nleft;       /* bipartite: ndocs                                       */
  uint32_t flags;
  uint64_t nrecords;    /* records read                                           */
  uint64_t nentries;    /* stored entries after self-loop removal and dedup       */
  uint32_t nregular, nsink, nsource, nisolated;  /* processed_matrix2d.hpp:203-228 */
  uint64_t device_bytes; /* HBM held by the graph                                  */
} la3g_graph_info;

typedef struct la3g_stats
{
  double device_ms;      /* device time of the call's compute (CUDA events)              */
  double host_ms;        /* wall time of the whole call, copies included                 */
  uint32_t iterations;   /* BSP iterations run                                            */
  uint32_t pull_iterations; /* of which ran bottom-up / pull                             */
  uint64_t teps_edges;   /* numerator of the app's GTEPS definition                       */
  uint64_t edges_examined; /* edges the kernels read (algorithmic-byte accounting)        */
  uint64_t algo_bytes;   /* algorithmic bytes of the call's kernels                       */
  uint32_t kernel_launches; /* kernels launched by the call                               */
  uint32_t reserved;
} la3g_stats;

/* Edge lists produced by the generators (host memory, owned by the library
 * until la3g_edges_free). */
typedef struct la3g_edges
{
  uint32_t* src;
  uint32_t* dst;
  uint32_t* w;        /* NULL when unweighted */
  uint64_t m;
  uint32_t n;         /* vertices (bipartite: ndocs) */
  uint32_t nright;    /* bipartite: nterms, else 0   */
  int weighted;
  int reserved;
} la3g_edges;

/* ---- errors ------------------------------------------------------------ */

const char* la3g_last_error_string(void);
const char* la3g_status_string(int status);

/* ---- graphs: replaces Graph<W>::load_binary and its wrappers
 *      (src/matrix/graph.hpp:37-214, 224-258) -------------------------- */

/* Loads an LA3 binary edge list and builds the device matrix.  n = number of
 * vertices as on the app command line (0: read the 16-byte header);
 * nright = nterms for LA3G_BIPARTITE, else ignored. */
int la3g_graph_load(const char* path, uint32_t n, uint32_t nright, uint32_t flags, la3g_graph** out);

/* Same, from LA3 records already in host memory (8-byte pairs or 12-byte
 * triples, as on disk, no header). */
int la3g_graph_from_records(const void* records, uint64_t nrecords, uint32_t n, uint32_t nright,
                            uint32_t flags, la3g_graph** out);

/* Same, from a generator's edge list (n = 0: use e->n / e->nright). */
int la3g_graph_from_edges(const la3g_edges* e, uint32_t n, uint32_t nright, uint32_t flags,
                          la3g_graph** out);

void la3g_graph_free(la3g_graph* g);
int la3g_graph_info_get(const la3g_graph* g, la3g_graph_info* out);

/* Runs the graph's subsequent calls on the caller's CUDA stream (a
 * cudaStream_t passed as void*; NULL = back to the graph's own stream).
 * The reference has no streams; this exists so that a caller can bracket
 * calls with its own CUDA events. */
int la3g_graph_set_stream(la3g_graph* g, void* cuda_stream);

/* Reverse-engine view: vertex id -> internal position (Locator order
 * regular, sink, source, isolated; src/utils/locator.h:84-120).  Either
 * array may be NULL. */
int la3g_graph_positions(const la3g_graph* g, uint32_t* pos_of_id, uint32_t* id_of_pos);

/* Device view of a loaded graph, for vertex programs compiled against the
 * template engine in la3g_vp.cuh (the reference's VertexProgram runs on its
 * own Graph's tiles, src/vprogram/vertex_program.h:99-180).  All pointers
 * are device pointers owned by the graph; positions follow
 * la3g_graph_positions.  row_ptr / col / weight: in-edges of every position
 * (rows = regular then sink positions), each row's columns in the order the
 * reference's SpMV visits them (source columns first, then regular, each
 * ascending).  weight is NULL for unweighted graphs. */
typedef struct la3g_device_graph
{
  const uint32_t* row_ptr;      /* [nslots + 1] */
  const uint32_t* col;          /* [nentries] column positions */
  const uint32_t* weight;       /* [nentries] or NULL */
  const uint32_t* hash_of_pos;  /* [nslots] hashed id passed as Edge src / dst */
  const uint32_t* id_of_pos;    /* [nslots] original vertex id */
  const uint32_t* pos_of_id;    /* [nslots] */
  uint32_t nslots, nregular, nsink, nsource;
  uint32_t flags;
  uint32_t reserved;
  uint64_t nentries;
  void* stream;                 /* cudaStream_t the graph's calls run on */
} la3g_device_graph;

int la3g_graph_device_view(la3g_graph* g, la3g_device_graph* out);

/* The push (out-edge) CSR over column positions, for engines that expand a
 * frontier of active columns: out_ptr[nslots + 1], out_row[nentries] (row
 * positions, ascending per column).  Built on the device on first use for
 * directed graphs; an undirected graph's CSR is symmetric and is returned
 * as is.  No counterpart in the reference, whose SpMV walks its per-tile
 * CSC by active column (src/vprogram/vertex_program_execute.hpp:564-603). */
int la3g_graph_push_view(la3g_graph* g, const uint32_t** out_ptr, const uint32_t** out_row);

/* ---- apps (replace the apps' run() functions) ---------------------------- */

/* PageRank, FP64, un-normalised, alpha = 0.15: the reference pr app
 * (src/apps/graph_analytics/pr.cpp:11-55, pr.h:12-46) on a graph loaded with
 * LA3G_DIRECTED.  iters = 0 runs until no rank moves by more than 1e-5.
 * Sums follow the reference's order, so ranks are bit-identical to it. */
int la3g_pr(la3g_graph* g, uint32_t iters, double* rank_out, uint32_t* degree_out, la3g_stats* st);

/* PageRank with FP32 SpMV and FP32 accumulation (precision study); the
 * residual (L1 of the rank change) and the dangling mass stay FP64.  Stops
 * after iters iterations or when the L1 residual drops below tol (tol <= 0:
 * fixed iterations).  residual_out: last L1 residual. */
int la3g_pr_f32(la3g_graph* g, uint32_t iters, double tol, double* rank_out, double* residual_out,
                la3g_stats* st);

/* The same FP32 study over a tiled copy of the matrix: the regular rows in
 * tiles of 2048 rows, each tile doubly compressed by column as the
 * reference's per-tile DCSC (src/utils/csc.h:60-130, tiles of
 * src/matrix/matrix2d.hpp:6-25): non-empty columns with offsets and a 16-bit
 * row per entry (hypersparse tiles also keep each entry's column and are
 * walked by entry); the tile's row accumulators live in shared memory; rows
 * with more than 1024 in-edges are summed from the flat CSR, a block each.  Built on the device
 * on the first call (about 14 B per entry).  Results agree with
 * la3g_pr_f32 to FP32 rounding (addition order inside a row differs). */
int la3g_pr_f32_tiled(la3g_graph* g, uint32_t iters, double tol, double* rank_out, double* residual_out,
                      la3g_stats* st);

/* BFS (src/apps/graph_analytics/bfs.cpp:11-37, bfs.h:11-49) on an undirected
 * graph: hops (uint8, 255 = unreached) and parent (the hashed id of the
 * frontier neighbour that the reference writes last, i.e. the largest).
 * Either output may be NULL (results stay on the device). */
int la3g_bfs(la3g_graph* g, uint32_t root, uint8_t* hops_out, uint32_t* parent_out, la3g_stats* st);

/* SSSP (src/apps/graph_analytics/sssp.cpp:11-37, sssp.h:11-46) on a graph
 * loaded with LA3G_DIRECTED | LA3G_WEIGHTED: uint32 distances,
 * 2147483647 = unreached. */
int la3g_sssp(la3g_graph* g, uint32_t root, uint32_t* dist_out, la3g_stats* st);

/* Connected components (src/apps/graph_analytics/cc.cpp:11-31, cc.h:11-38)
 * on an undirected graph: labels as the reference computes them (the least
 * vertex id of each component when vertex 0 has no edges). */
int la3g_cc(la3g_graph* g, uint32_t* label_out, la3g_stats* st);

/* Triangle counting (src/apps/graph_analytics/tc.cpp:11-52, tc.h:47-99) on
 * a graph loaded with LA3G_DIRECTED | LA3G_ACYCLIC: total and, per vertex,
 * the triangles in which it is the middle vertex by id (uint32, wrapping as
 * the reference's accumulator does).  per_vertex_out may be NULL. */
int la3g_tc(la3g_graph* g, uint64_t* total_out, uint32_t* per_vertex_out, la3g_stats* st);

/* Degrees (src/apps/graph_analytics/degree.cpp:16-46, degree.h:17-35): on a
 * graph loaded with LA3G_DIRECTED, the in-degree of every vertex (its number
 * of distinct in-neighbours); loaded with LA3G_DIRECTED | LA3G_REVERSE, the
 * out-degree (the reference's -o).  degree_out: nslots uint32 by id
 * (nullable).  The k (<= 64) largest, degree desc, id asc, go to topk_ids /
 * topk_degrees (nullable; *ntopk = min(k, nslots)). */
int la3g_degree(la3g_graph* g, uint32_t* degree_out, uint32_t k, uint32_t* topk_ids, uint32_t* topk_degrees,
                uint32_t* ntopk, la3g_stats* st);

/* Top-k on the device over n uint32 values (a host array, index = id):
 * the k (<= 64) largest, value desc, index asc (vertex_program.hpp:607-680,
 * with the tie order fixed). */
int la3g_topk_u32(const uint32_t* values, uint32_t n, uint32_t k, uint32_t* ids_out, uint32_t* values_out,
                  uint32_t* nout);

/* BM25 (src/apps/information_retrieval/bm25.cpp:8-114, bm25.h:11-92) on a
 * graph loaded with LA3G_BIPARTITE (undirected).  prepare runs the IDF and
 * the two doc-length passes; length_out (nslots, nullable) receives the
 * state each vertex holds afterwards (idf for terms, K(d) for docs). */
int la3g_bm25_prepare(la3g_graph* g, uint64_t* collection_ntokens_out, float* avg_doc_length_out,
                      float* length_out);

/* One query: term_vids are term VERTEX ids (ndocs + term index) in query
 * order, as prepare_queries produces them (helpers.hpp:76-123); the
 * reference's pairing of values with terms for non-ascending lists is kept.
 * Writes the first min(k, touched) docs in the order score desc, id asc.
 * all_scores_out (nslots floats) and active_out (nslots bytes) are optional
 * full dumps of the scored docs. */
int la3g_bm25_query(la3g_graph* g, const uint32_t* term_vids, uint32_t nterms, uint32_t k,
                    uint32_t* ids_out, float* scores_out, uint32_t* nout, float* all_scores_out,
                    uint8_t* active_out, la3g_stats* st);

/* LM, query likelihood with Dirichlet smoothing (mu = 2000)
 * (src/apps/information_retrieval/lm.cpp:8-144, lm.h:16-75), on a graph
 * loaded with LA3G_BIPARTITE (undirected).  prepare runs the DL and TL
 * passes; length_out (nslots, nullable) receives length(d) for docs and
 * length(t) for terms.  The score's per-vertex factor log10f(mu / (length +
 * mu)) is evaluated here with the platform's log10f, the function the
 * reference calls (lm.h:74). */
int la3g_lm_prepare(la3g_graph* g, uint64_t* collection_ntokens_out, float* length_out);

/* One LM query, same conventions as la3g_bm25_query.  As in the reference,
 * the first query after prepare also ranks the term vertices the TL pass
 * left active (score 0), since the LM program takes no mirrors. */
int la3g_lm_query(la3g_graph* g, const uint32_t* term_vids, uint32_t nterms, uint32_t k,
                  uint32_t* ids_out, float* scores_out, uint32_t* nout, float* all_scores_out,
                  uint8_t* active_out, la3g_stats* st);

/* ---- batched multi-source forms (no reference counterpart; the reference
 *      runs one root per VertexProgram, bfs.cpp:11-37 / sssp.cpp:11-37) ---- */

/* hops_out: nroots x nslots bytes, row r = la3g_bfs(roots[r]) hops. */
int la3g_bfs_batch(la3g_graph* g, const uint32_t* roots, uint32_t nroots, uint8_t* hops_out,
                   la3g_stats* st);
/* dist_out: nroots x nslots uint32, row r = la3g_sssp(roots[r]) distances. */
int la3g_sssp_batch(la3g_graph* g, const uint32_t* roots, uint32_t nroots, uint32_t* dist_out,
                    la3g_stats* st);

/* Tunes the batched BFS for this graph (level mode: per-level CUDA graph or
 * persistent kernel; block size; push/pull threshold) by timing each
 * combination on the given roots (best of two runs); the best is kept on the
 * graph handle for batches of the same number of 64-root words (batches of
 * other sizes use the nearest tuned size).  report (nullable) receives a
 * JSON list of the timings. */
int la3g_batch_autotune(la3g_graph* g, const uint32_t* roots, uint32_t nroots, char* report, size_t cap);

/* Sets the batched-BFS configuration by hand (dropping tuned ones): mode 0 =
 * per-level CUDA graph, 1 = persistent kernel; block 128 / 256 / 512;
 * push_frac in [0, 1]. */
int la3g_batch_config(la3g_graph* g, int mode, int block, double push_frac);

/* The persistent batched-BFS kernel's grid barriers wait at most `polls`
 * polls per block (default 2^26, restored by polls < 0); a block that runs
 * out sets an error word, every block leaves its kernel, and the call returns
 * LA3G_ETIMEOUT with the device left usable.  No counterpart in the
 * reference (it has no device waits); polls = 0 makes any wait give up at
 * once, which exercises that error path. */
int la3g_batch_set_wait_limit(la3g_graph* g, long long polls);

/* The batched SSSP's distance window: an iteration relaxes only the roots
 * whose distance is at most (smallest distance in the frontier) + delta and
 * keeps the others active for a later iteration (delta-stepping's buckets,
 * one window over all roots of a 256-root chunk).  delta = 0 picks the width
 * from the graph's largest weight; 0xFFFFFFFF relaxes every active root each
 * iteration.  The distances are the same for every delta. */
int la3g_batch_sssp_window(la3g_graph* g, uint32_t delta);

/* ---- serving loop (no reference counterpart; the reference answers one
 *      query per VertexProgram run, bfs.cpp:11-37, sssp.cpp:11-37,
 *      bm25.cpp:8-114) ------------------------------------------------------ */

typedef struct la3g_server la3g_server;

enum
{
  LA3G_QUERY_BFS = 1,   /* hops from root (la3g_bfs) */
  LA3G_QUERY_SSSP = 2,  /* distances from root (la3g_sssp) */
  LA3G_QUERY_BM25 = 3,  /* top-k documents (la3g_bm25_query) */
  LA3G_QUERY_LM = 4     /* top-k documents by query likelihood (la3g_lm_query) */
};

typedef struct la3g_query
{
  uint32_t kind;          /* LA3G_QUERY_* */
  uint32_t graph;         /* id returned by la3g_server_add_graph */
  uint32_t root;          /* BFS / SSSP root vertex id */
  uint32_t k;             /* BM25 / LM: documents wanted */
  const uint32_t* terms;  /* BM25 / LM: term vertex ids (copied at submit) */
  uint32_t nterms;
  void* out;              /* BFS: uint8 hops[nslots]; SSSP: uint32 dist[nslots]; BM25 / LM: uint32 ids[k]; may be NULL */
  float* scores_out;      /* BM25 / LM: scores[k]; may be NULL */
} la3g_query;

typedef struct la3g_query_result
{
  int status;             /* LA3G_OK or the query's error */
  uint32_t kind;
  double queue_ms;        /* submit -> admitted into a lane / started */
  double latency_ms;      /* submit -> result written */
  uint32_t in_flight;     /* queries on the graph's engine when it was admitted */
  uint32_t nout;          /* BM25: documents written */
} la3g_query_result;

typedef struct la3g_server_stats
{
  uint64_t budget_bytes, used_bytes;
  uint64_t completed, queued, pending;
  uint32_t ngraphs, reserved;
} la3g_server_stats;

/* A server with an HBM budget (bytes).  bfs_lanes / sssp_lanes: queries one
 * BFS / SSSP engine holds at once (multiples of 64; 0 = 256 / 256).  A BFS
 * engine admits queries 64 at a time into free 64-lane words (queries that
 * are queued when a word frees up start together); an SSSP engine admits
 * them into any free lane. */
int la3g_server_create(uint64_t budget_bytes, uint32_t bfs_lanes, uint32_t sssp_lanes, la3g_server** out);
/* Makes a loaded graph resident in the server: undirected graphs serve BFS,
 * DIRECTED|WEIGHTED graphs SSSP, BIPARTITE graphs BM25 and LM (both
 * prepared here if needed; LM's first-query leftover activity is taken here,
 * so every served LM query sees the reference's steady state).  The graph's device bytes plus its engine's lane state must fit
 * in the budget left (the lane count is halved down to 64 first), else
 * LA3G_EBUDGET.  The caller keeps ownership but must not use the graph while
 * it is served; la3g_server_free releases it. */
int la3g_server_add_graph(la3g_server* s, la3g_graph* g, uint32_t* graph_id);
/* Queues a query and returns its ticket at once; thread-safe.  The query's
 * output buffers must stay valid until the ticket is polled done. */
int la3g_server_submit(la3g_server* s, const la3g_query* q, uint64_t* ticket);
/* Waits up to timeout_ms (0 = do not wait, < 0 = forever) for the ticket:
 * LA3G_OK with res filled (the ticket is then released), or LA3G_EBUSY while
 * it is still pending.  Thread-safe. */
int la3g_server_poll(la3g_server* s, uint64_t ticket, int timeout_ms, la3g_query_result* res);
int la3g_server_info(la3g_server* s, la3g_server_stats* out);
/* Adaptive batching: an engine with no lanes in flight answers queries one at
 * a time through the single-root entry point while at most this many wait
 * (defaults 16 for BFS, 4 for SSSP); deeper queues use lanes.  0 = always
 * lanes.  Results are the same either way. */
int la3g_server_set_solo(la3g_server* s, uint32_t bfs_depth, uint32_t sssp_depth);
/* Lanes the engine of graph_id was given (after budget halving). */
int la3g_server_lanes(la3g_server* s, uint32_t graph_id, uint32_t* lanes);
/* Stops the workers (queries still queued are dropped) and frees the
 * server's device state; the graphs stay with the caller. */
void la3g_server_free(la3g_server* s);

/* ---- caller-allocated form -------------------------------------------- */

/* BFS that allocates nothing.  It has no counterpart in the reference: it is
 * for callers that cannot allocate device memory at call time — code running
 * under a memory manager that owns every device byte, a serving loop that
 * must not take cudaMalloc/cudaFree's implicit device synchronisation on its
 * latency path, or a host that pre-reserves all memory at start-up.  The
 * caller passes an undirected graph already in device memory as a CSR over
 * vertices 0..nvertices-1 (row_ptr: nvertices + 1 offsets; col: neighbour
 * ids, each row sorted by ascending key; key: one uint32 per vertex) and the
 * device output arrays hops and parent (nvertices each).  Results follow
 * la3g_bfs: hops 255 = unreached; parent = the key of the frontier neighbour
 * with the largest key (with key = the hashed id of the reference's bucket
 * hasher, hops and parent equal la3g_bfs's).  The library's temporaries sit in
 * one fixed device array of about 12.8 MB, so nvertices is limited to
 * 1048576 (2^20); larger graphs are rejected with LA3G_EINVAL.  Each call
 * looks up the array's address on the current device (no allocation).  The
 * call waits for its stream at every BFS level, since it reads the frontier
 * size back to the host, and again before it returns, also after an error.
 * Calls share the array, so calls that overlap on the GPU race; run them one
 * at a time.  row_ptr must be non-decreasing with row_ptr[nvertices] = the
 * entry count; that is not checked, while neighbour ids >= nvertices are
 * skipped.  cuda_stream: a cudaStream_t as void* (NULL = the default
 * stream).  st may be NULL. */
int la3g_bfs_noalloc(const uint32_t* row_ptr, const uint32_t* col, const uint32_t* key, uint32_t nvertices,
                     uint32_t root, uint8_t* hops, uint32_t* parent, void* cuda_stream, la3g_stats* st);

/* ---- synthetic inputs -------------------------------------------------- */

int la3g_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                  int weighted, uint64_t wseed, la3g_edges* out);
int la3g_gen_er(uint32_t n, uint64_t m, uint64_t seed, int weighted, uint64_t wseed, la3g_edges* out);
int la3g_gen_bipartite(uint32_t ndocs, uint32_t nterms, uint32_t terms_per_doc, double zipf_s,
                       double df_cap, uint64_t seed, la3g_edges* out);
/* Writes LA3 binary records (the layout tools/mtx2bin.cpp:77-111 writes),
 * with the 16-byte header when header != 0. */
int la3g_edges_write(const la3g_edges* e, const char* path, int header);
void la3g_edges_free(la3g_edges* e);

/* ---- measurement ------------------------------------------------------- */

/* When on, every kernel launch of the library is bracketed by CUDA events on
 * its stream and its time is accumulated per kernel name. */
void la3g_profile_enable(int on);
void la3g_profile_reset(void);
/* JSON object {"kernel": {"launches": L, "ms": T, "bytes": B}, ...}; returns
 * the length needed (excluding the terminating NUL). */
size_t la3g_profile_report(char* buf, size_t cap);

#ifdef __cplusplus
}
#endif

#endif
