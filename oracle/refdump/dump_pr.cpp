/* Reference PageRank dump: replays apps/graph_analytics/pr.cpp:run (pr.cpp:11-55). */
#include "apps/graph_analytics/pr.h"
#include "dump_common.h"

int main(int argc, char* argv[])
{
  Env::init();
  if (argc < 5) { std::fprintf(stderr, "usage: %s <file> <n> <iters> <out_prefix>\n", argv[0]); return 1; }
  std::string path = argv[1];
  vid_t n = (vid_t) std::atol(argv[2]);
  uint32_t iters = (uint32_t) std::atoi(argv[3]);
  std::string out = argv[4];

  Graph<ew_t> GR;
  GR.load_directed(true, path, n, true);
  DegVertex<ew_t> vp_degree(&GR, true);
  double t0 = Env::now();
  vp_degree.execute(1);
  double t_deg = Env::now() - t0;
  GR.free();

  Graph<ew_t> G;
  G.load_directed(true, path, n);
  PrVertex vp(&G, true);
  vp.initialize(vp_degree);
  vp_degree.free();
  t0 = Env::now();
  vp.execute(iters);
  double t_pr = Env::now() - t0;

  size_t N = (size_t) G.get_nvertices() + 1;
  std::vector<double> rank(N, 0.0);
  std::vector<uint32_t> deg(N, 0);
  vp.reduce<long>([&](uint32_t idx, const PrState& s) -> long { rank[idx] = s.rank; deg[idx] = s.degree; return 0; },
                  [&](long&, const long&) {});
  long deg_checksum = vp.reduce<long>([&](uint32_t, const PrState& s) -> long { return s.degree; },
                                      [&](long& a, const long& b) { a += b; });
  double pr_checksum = vp.reduce<double>([&](uint32_t, const PrState& s) -> double { return s.rank; },
                                         [&](double& a, const double& b) { a += b; });
  dump_array(out + ".rank.f64", rank);
  dump_array(out + ".degree.u32", deg);
  std::printf("{\"app\": \"pr\", \"exec_s\": %.9f, \"degree_exec_s\": %.9f, \"degree_checksum\": %ld, "
              "\"pr_checksum\": %.17g, \"nslots\": %zu}\n", t_pr, t_deg, deg_checksum, pr_checksum, N);
  Env::finalize();
  return 0;
}
