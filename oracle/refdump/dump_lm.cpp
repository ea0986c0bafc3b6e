/*
 * Reference LM dump: replays apps/information_retrieval/lm.cpp:run
 * (lm.cpp:8-144).  Writes the per-vertex DtState.length after the TL pass
 * (length(d) for docs, length(t) for terms), and for every query the score
 * of every active doc plus the reference's own top-k list.
 */
#include <cstring>
#include "utils/dist_timer.h"
#include "apps/information_retrieval/helpers.hpp"
#include "apps/information_retrieval/lm.h"
#include "dump_common.h"

int main(int argc, char** argv)
{
  Env::init();
  if (argc < 8)
  {
    std::fprintf(stderr, "usage: %s <graph> <term.labels> <ndocs> <nterms> <queries> <k> <out_prefix>\n", argv[0]);
    return 1;
  }
  std::string graph = argv[1], labels = argv[2];
  vid_t ndocs = (vid_t) atoi(argv[3]);
  vid_t nterms = (vid_t) atoi(argv[4]);
  std::string qpath = argv[5];
  uint32_t k = atoi(argv[6]);
  std::string out = argv[7];

  std::vector<std::vector<vid_t>> queries;
  prepare_queries(labels, qpath, queries, ndocs);

  Graph<ew_t> G;
  G.load_bipartite(true, graph, ndocs, nterms, false);
  DL dl(&G, true);
  dl.initialize_bipartite<false, true>();
  dl.execute(1);
  uint64_t ntokens = dl.reduce<uint64_t>([&](uint32_t, const DtState& s) -> uint64_t { return s.length; },
                                         [&](uint64_t& a, const uint64_t& b) { a += b; });
  TL tl(dl, true);
  tl.collection_ntokens = ntokens;
  tl.reset_activity();
  tl.initialize_bipartite<true, false>();
  tl.execute(1);

  size_t N = (size_t) G.get_nvertices() + 1;
  std::vector<float> length(N, 0.0f);
  tl.reduce<long>([&](uint32_t idx, const DtState& s) -> long { length[idx] = s.length; return 0; },
                  [&](long&, const long&) {});
  dump_array(out + ".length.f32", length);

  TFIDF tfidf(dl);
  FILE* fq = std::fopen((out + ".queries.bin").c_str(), "wb");
  double total = 0;
  for (size_t q = 0; q < queries.size(); q++)
  {
    double t0 = Env::now();
    tfidf.reset();
    tfidf.initialize(queries[q]);
    tfidf.query_nterms = queries[q].size();
    tfidf.execute(1);
    using iv_t = std::pair<vid_t, fp_t>;
    std::vector<iv_t> topk;
    tfidf.topk<vid_t, fp_t>(k, topk, [&](vid_t, const DtState& s) { return s.score; },
                            [&](const iv_t& a, const iv_t& b) { return a.second > b.second; }, true);
    total += Env::now() - t0;
    std::vector<iv_t> active;
    tfidf.reduce<long>([&](uint32_t idx, const DtState& s) -> long { active.push_back(iv_t(idx, s.score)); return 0; },
                       [&](long&, const long&) {}, true);
    tfidf.reset_activity();
    uint32_t na = (uint32_t) active.size(), nk = (uint32_t) topk.size();
    std::fwrite(&na, 4, 1, fq);
    for (auto& iv : active) { std::fwrite(&iv.first, 4, 1, fq); std::fwrite(&iv.second, 4, 1, fq); }
    std::fwrite(&nk, 4, 1, fq);
    for (auto& iv : topk) { std::fwrite(&iv.first, 4, 1, fq); std::fwrite(&iv.second, 4, 1, fq); }
  }
  std::fclose(fq);
  std::printf("{\"app\": \"lm\", \"collection_ntokens\": %lu, \"nqueries\": %zu, \"query_s_total\": %.9f, "
              "\"nslots\": %zu}\n",
              (unsigned long) ntokens, queries.size(), total, N);
  Env::finalize();
  return 0;
}
