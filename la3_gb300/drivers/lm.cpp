// lm <graph_filepath> <labels_filepath> <num_docs> <num_terms> <queries_filepath> <k>
// (src/apps/information_retrieval/lm.cpp:8-176)
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "driver_common.h"

int main(int argc, char** argv)
{
  if (argc < 7)
  {
    std::printf("Usage: %s <graph_filepath> <labels_filepath> <num_docs> <num_terms> <queries_filepath> <k> \n",
                argv[0]);
    return 1;
  }
  const uint32_t ndocs = (uint32_t) std::atoi(argv[3]), nterms = (uint32_t) std::atoi(argv[4]);
  const uint32_t k = (uint32_t) std::atoi(argv[6]);
  auto queries = read_queries(argv[2], argv[5], ndocs);
  std::printf("Total queries: %zu \n", queries.size());
  la3g_graph* g = load(argv[1], ndocs, LA3G_BIPARTITE | LA3G_WEIGHTED, nterms);
  uint64_t ntokens = 0;
  check(la3g_lm_prepare(g, &ntokens, nullptr), "lm prepare");
  std::printf("Collection.Tokens= %lu \n", (unsigned long) ntokens);
  std::vector<uint32_t> ids(k);
  std::vector<float> scores(k);
  double total_ms = 0;
  for (size_t q = 0; q < queries.size(); q++)
  {
    uint32_t nout = 0;
    la3g_stats st{};
    check(la3g_lm_query(g, queries[q].data(), (uint32_t) queries[q].size(), k, ids.data(), scores.data(), &nout,
                        nullptr, nullptr, &st),
          "lm query");
    total_ms += st.host_ms;
    std::string terms;
    for (uint32_t t : queries[q]) terms += std::to_string(t - ndocs) + " ";
    std::printf("q %zu (%s): top-%u docs: \n", q, terms.c_str(), k);
    for (uint32_t i = 0; i < nout; i++) std::printf("idx %u: score %lf \n", ids[i], (double) scores[i]);
  }
  if (!queries.empty()) std::printf("LM time: %lf ms \n", total_ms / queries.size());
  la3g_graph_free(g);
  return 0;
}
