// cc <filepath> <num_vertices: 0 if header present>
// (src/apps/graph_analytics/cc.cpp:11-50)
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "driver_common.h"

int main(int argc, char** argv)
{
  if (argc < 3)
  {
    std::printf("Usage: %s <filepath> <num_vertices: 0 if header present> \n", argv[0]);
    return 1;
  }
  la3g_graph* g = load(argv[1], (uint32_t) std::atol(argv[2]), 0);
  const uint32_t N = nslots(g);
  std::vector<uint32_t> label(N);
  la3g_stats st{};
  check(la3g_cc(g, label.data(), &st), "cc");
  report("CC Execution", st);
  long sum = 0;
  for (uint32_t v = 0; v < N; v++) sum += (long) label[v];
  std::printf("Checksum = %lu \n", (unsigned long) sum);
  la3g_graph_free(g);
  return 0;
}
