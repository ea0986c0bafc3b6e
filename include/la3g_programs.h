/* la3g_programs.h: C entry points of libla3g_programs.so, the reference's
 * apps written as vertex programs against la3g_vp.cuh (the plugin API) and
 * run by la3g_vp::Engine.  Outputs are by original vertex id (nslots
 * entries); each returns an la3g_status. */
#ifndef LA3G_PROGRAMS_H
#define LA3G_PROGRAMS_H

#include <stdint.h>

#include "la3g.h"

#ifdef __cplusplus
extern "C" {
#endif

/* DegVertex (degree.h:17-35), execute(1): in-degrees of the graph given. */
int la3gp_degree(la3g_graph* g, uint32_t* degree);
/* pr.cpp:11-55: g loaded LA3G_DIRECTED, gr the same file with LA3G_REVERSE. */
int la3gp_pagerank(la3g_graph* g, la3g_graph* gr, uint32_t iters, double* rank, uint32_t* degree);
int la3gp_bfs(la3g_graph* g, uint32_t root, uint8_t* hops, uint32_t* parent, uint32_t* iters);
int la3gp_sssp(la3g_graph* g, uint32_t root, uint32_t* dist, uint32_t* iters);
int la3gp_cc(la3g_graph* g, uint32_t* label, uint32_t* iters);

/* The degree app's tail (degree.cpp:34-43) through the engine's topk and
 * reduce: DegVertex execute(1) on g, then topk<vid, vid>(k) by degree,
 * largest first (ids[k], degrees[k]), and reduce(sum of degrees).  With
 * btopk set, also btopk<2>(k) over (degree, ~degree): the k largest and the
 * k smallest degrees (bids[2k], bvals[2k]).  k <= 512. */
int la3gp_degree_topk(la3g_graph* g, uint32_t k, uint32_t* ids, uint32_t* degrees, uint64_t* degree_sum,
                      uint32_t* bids, uint32_t* bvals);

/* TC (tc.cpp:11-52) through the engine: g loaded LA3G_DIRECTED |
 * LA3G_ACYCLIC, gr the same file LA3G_DIRECTED | LA3G_ACYCLIC |
 * LA3G_REVERSE.  CtVertex's neighbour lists travel as variable-size
 * messages.  total: sum of the per-vertex counts (reduce); ntri: nslots
 * counts by vertex id (nullable). */
int la3gp_tc(la3g_graph* g, la3g_graph* gr, uint64_t* total, uint32_t* ntri);

/* BFS (bfs.h) from root, then topk over the ACTIVE vertices (those apply
 * reached; not the root, which init activates without marking) by hops,
 * largest first: ids[k], hops[k]. */
int la3gp_bfs_topk(la3g_graph* g, uint32_t root, uint32_t k, uint32_t* ids, uint32_t* hops);

/* Graph simulation (src/apps/graph_simulation/graphsim.cpp:45-90,
 * graphsim.h:60-184) on the data graph loaded LA3G_DIRECTED | LA3G_REVERSE,
 * as the reference loads it.  vlabel: nslots label ids by vertex id (0 = the
 * empty string, i.e. no label; equal strings, equal ids); the query: qsize
 * (1..32) label ids and nqedges (<= 1024) edges (i, j) as pairs, in file
 * order.  matched: nslots bytes (is_matched), res: nslots x qsize chars
 * ('U', '0', '1'), both nullable. */
int la3gp_graphsim(la3g_graph* gr, const uint32_t* vlabel, uint32_t qsize, const uint32_t* qlabel,
                   const uint32_t* qedges, uint32_t nqedges, uint8_t* matched, char* res, uint32_t* nmatches,
                   uint32_t* iters);

#ifdef __cplusplus
}
#endif

#endif
