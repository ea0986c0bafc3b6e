// degree <filepath> <num_vertices: 0 if header present> [-o (out-degree)]
// (src/apps/graph_analytics/degree.cpp:16-66).  The reference's display()
// lists ids 0..30 in its hashed order; here they come in id order.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "driver_common.h"

int main(int argc, char** argv)
{
  if (argc < 3)
  {
    std::printf("Usage: %s <filepath> <num_vertices: 0 if header present> [-o (out-degree)] \n", argv[0]);
    return 1;
  }
  const uint32_t n = (uint32_t) std::atol(argv[2]);
  const bool out_degree = argc > 3 && std::string(argv[3]) == "-o";
  la3g_graph* g = load(argv[1], n, LA3G_DIRECTED | (out_degree ? LA3G_REVERSE : 0));
  const uint32_t N = nslots(g);
  std::vector<uint32_t> deg(N), ids(3), top(3);
  uint32_t nk = 0;
  la3g_stats st{};
  check(la3g_degree(g, deg.data(), 3, ids.data(), top.data(), &nk, &st), "degree");
  std::printf(out_degree ? "Out-Degrees: \n" : "In-Degrees: \n");
  for (uint32_t v = 0; v < N && v <= 30; v++) std::printf("%u: {degree: %u}\n", v, deg[v]);
  std::printf("Top-%d: \n", 3);
  for (uint32_t i = 0; i < nk; i++) std::printf("idx %u: degree %u \n", ids[i], top[i]);
  report("Degree Execution", st);
  la3g_graph_free(g);
  return 0;
}
