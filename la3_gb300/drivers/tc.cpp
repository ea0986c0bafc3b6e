// tc <filepath> <num_vertices: 0 if header present>
// (src/apps/graph_analytics/tc.cpp:11-70)
#include <cstdio>
#include <cstdlib>

#include "driver_common.h"

int main(int argc, char** argv)
{
  if (argc < 3)
  {
    std::printf("Usage: %s <filepath> <num_vertices: 0 if header present> \n", argv[0]);
    return 1;
  }
  la3g_graph* g = load(argv[1], (uint32_t) std::atol(argv[2]), LA3G_DIRECTED | LA3G_ACYCLIC);
  uint64_t total = 0;
  la3g_stats st{};
  check(la3g_tc(g, &total, nullptr, &st), "tc");
  report("Triangle Counting", st);
  std::printf("Triangles = %lu \n", (unsigned long) total);
  la3g_graph_free(g);
  return 0;
}
