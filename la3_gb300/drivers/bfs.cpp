// bfs <filepath> <num_vertices: 0 if header present> <root>
// (src/apps/graph_analytics/bfs.cpp:11-60)
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
  la3g_graph* g = load(argv[1], (uint32_t) std::atol(argv[2]), 0);
  const uint32_t root = (uint32_t) std::atol(argv[3]);
  const uint32_t N = nslots(g);
  std::vector<uint8_t> hops(N);
  std::vector<uint32_t> parent(N);
  la3g_stats st{};
  check(la3g_bfs(g, root, hops.data(), parent.data(), &st), "bfs");
  report("BFS Execution", st);
  long reach = 0, sum = 0;
  for (uint32_t v = 0; v < N; v++)
  {
    reach += hops[v] != 255;
    sum += (long) hops[v] * (long) parent[v];
  }
  std::printf("Reachable Vertices = %lu \n", (unsigned long) reach);
  std::printf("Checksum = %lu \n", (unsigned long) sum);
  la3g_graph_free(g);
  return 0;
}
