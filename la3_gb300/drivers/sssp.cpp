// sssp <filepath (weighted)> <num_vertices: 0 if header present> <root>
// (src/apps/graph_analytics/sssp.cpp:11-60)
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "driver_common.h"

int main(int argc, char** argv)
{
  if (argc < 4)
  {
    std::printf("Usage: %s <filepath> <num_vertices: 0 if header present> <root> \n", argv[0]);
    return 1;
  }
  la3g_graph* g = load(argv[1], (uint32_t) std::atol(argv[2]), LA3G_DIRECTED | LA3G_WEIGHTED);
  const uint32_t root = (uint32_t) std::atol(argv[3]);
  const uint32_t N = nslots(g);
  std::vector<uint32_t> dist(N);
  la3g_stats st{};
  check(la3g_sssp(g, root, dist.data(), &st), "sssp");
  report("SSSP Execution", st);
  long reach = 0, sum = 0;
  for (uint32_t v = 0; v < N; v++)
  {
    reach += dist[v] != 0x7FFFFFFFu;
    sum += (long) dist[v];
  }
  std::printf("Reachable Vertices = %lu \n", (unsigned long) reach);
  std::printf("Checksum = %lu \n", (unsigned long) sum);
  la3g_graph_free(g);
  return 0;
}
