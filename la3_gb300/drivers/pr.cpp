// pr <filepath> <num_vertices: 0 if header present> [iterations]
// (src/apps/graph_analytics/pr.cpp:11-76)
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "driver_common.h"

int main(int argc, char** argv)
{
  if (argc < 3)
  {
    std::printf("Usage: %s <filepath> <num_vertices: 0 if header present> [<num_iterations>] \n", argv[0]);
    return 1;
  }
  const uint32_t n = (uint32_t) std::atol(argv[2]);
  const uint32_t iters = argc > 3 ? (uint32_t) std::atol(argv[3]) : 0;  // 0: until convergence
  la3g_graph* g = load(argv[1], n, LA3G_DIRECTED);
  const uint32_t N = nslots(g);
  std::vector<double> rank(N);
  std::vector<uint32_t> deg(N);
  la3g_stats st{};
  check(la3g_pr(g, iters, rank.data(), deg.data(), &st), "pagerank");
  report("Pagerank Execution", st);
  long deg_sum = 0;
  double pr_sum = 0.0;
  for (uint32_t v = 0; v < N; v++)
  {
    deg_sum += deg[v];
    pr_sum += rank[v];
  }
  std::printf("Iterations = %u \n", st.iterations);
  std::printf("Degree Checksum = %lu \n", (unsigned long) deg_sum);
  std::printf("Pagerank Checksum = %lf \n", pr_sum);
  la3g_graph_free(g);
  return 0;
}
