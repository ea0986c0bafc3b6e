/*
 * la3_oracle — CPU restatement of the LA3 vertex-program path (np = 1).
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this code, and only as
 * the checker.  The product path (libla3g) never links or calls it.
 *
 * It restates, in plain C, the reference's ingest (Graph::load_binary,
 * SimpleBucketHasher, vertex classification, locators, per-tile dedup + CSC),
 * its BSP execution engine (VertexProgram::execute and its optimizable /
 * non-optimizable / single-iteration paths) and the apps (pr, bfs, sssp,
 * cc, tc, bm25, lm, graph simulation).  Every result is indexed by
 * ORIGINAL vertex id 0..nslots-1.
 * Function comments cite the reference file:line each one follows.
 *
 * Parity is pinned against the reference itself: the same sources are built
 * with a single-rank MPI stand-in (oracle/refshim) and the committed golden
 * vectors under tests/golden were produced by that build.
 */
#ifndef LA3_ORACLE_H
#define LA3_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum og_flags
{
  OG_DIRECTED = 1u << 0,   /* Graph::load_directed (transposed: y = A^T x)      */
  OG_REVERSE = 1u << 1,    /* reverse_edges (no transpose)                      */
  OG_ACYCLIC = 1u << 2,    /* remove_cycles (orient by original id)             */
  OG_BIPARTITE = 1u << 3,  /* load_bipartite (col += nrows, NullHasher)         */
  OG_WEIGHTED = 1u << 4,   /* records are (u32, u32, u32) triples               */
};

enum og_status
{
  OG_OK = 0,
  OG_EIO = 1,      /* cannot open / read the file                              */
  OG_EFORMAT = 2,  /* file size not a whole number of records, bad header      */
  OG_EINVAL = 3,   /* vertex id outside [0, nslots)                            */
  OG_ENOMEM = 4,
};

typedef struct og_graph og_graph;

/* Ingest an LA3 binary edge list (graph.hpp:37-214).  n = number of vertices
 * as given on the app command line (0 = read the 16-byte header); for
 * bipartite graphs n = ndocs (left side) and nright = nterms. */
int og_load(const char* path, uint32_t n, uint32_t nright, uint32_t flags, og_graph** out);
void og_free(og_graph* g);

uint32_t og_nslots(const og_graph* g);
uint64_t og_nedges(const og_graph* g);  /* stored (deduplicated) entries */
void og_classes(const og_graph* g, uint32_t* nregular, uint32_t* nsink, uint32_t* nsource);
/* Internal position of each original id, and back. */
void og_positions(const og_graph* g, uint32_t* pos_of_orig, uint32_t* orig_of_pos);
uint32_t og_hash(const og_graph* g, uint32_t v);

/* Apps.  Output arrays have og_nslots() entries, indexed by original id. */
int og_pagerank(const og_graph* g, uint32_t iters, double* rank, uint32_t* degree);
int og_bfs(const og_graph* g, uint32_t root, uint8_t* hops, uint32_t* parent, uint32_t* niters);
int og_sssp(const og_graph* g, uint32_t root, uint32_t* dist, uint32_t* niters);
int og_cc(const og_graph* g, uint32_t* label, uint32_t* niters);
/* g_acyclic: load_directed(..., reverse=0, remove_cycles=1); the reversed
 * acyclic graph is derived internally. */
int og_tc(const og_graph* g_acyclic, uint32_t* ntriangles, uint64_t* total);

/* BM25 (bm25.cpp:8-114).  g: load_bipartite(..., directed=false). */
typedef struct og_bm25 og_bm25;
int og_bm25_prepare(const og_graph* g, og_bm25** out, uint64_t* collection_ntokens,
                    float* avg_doc_length, float* length /* nslots, nullable */);
/* term_vids: query term VERTEX ids (term index + ndocs) in query order, as
 * prepare_queries (helpers.hpp:76-123) produces them.  scores: nslots floats
 * (score of every active doc, 0 elsewhere), active: nslots bytes (1 = the doc
 * was touched by the query).  topk_ids/topk_scores: the first k entries in
 * the canonical order score desc, id asc. */
int og_bm25_query(og_bm25* b, const uint32_t* term_vids, uint32_t nterms, uint32_t k,
                  float* scores, uint8_t* active, uint32_t* topk_ids, float* topk_scores,
                  uint32_t* ntopk);
void og_bm25_free(og_bm25* b);

/* LM (lm.cpp:8-144), same graph and query conventions as BM25.  length:
 * length(d) for docs, length(t) for terms after the TL pass. */
typedef struct og_lm og_lm;
int og_lm_prepare(const og_graph* g, og_lm** out, uint64_t* collection_ntokens, float* length /* nullable */);
int og_lm_query(og_lm* b, const uint32_t* term_vids, uint32_t nterms, uint32_t k, float* scores,
                uint8_t* active, uint32_t* topk_ids, float* topk_scores, uint32_t* ntopk);
void og_lm_free(og_lm* b);

/* Graph simulation (graphsim.cpp:45-90).  g: load_directed(..., reverse=1).
 * vlabel: nslots label ids by vertex id (0 = the empty string, i.e. no
 * label); the query: qsize (<= 32) label ids and nqedges edges (i, j) in file
 * order.  matched: nslots bytes (is_matched), res: nslots x qsize chars. */
int og_graphsim(const og_graph* g, const uint32_t* vlabel, uint32_t qsize, const uint32_t* qlabel,
                const uint32_t* qedges, uint32_t nqedges, uint8_t* matched, char* res, uint32_t* nmatches,
                uint32_t* niters);

const char* og_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
