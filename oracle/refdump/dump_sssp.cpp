/* Reference SSSP dump: replays apps/graph_analytics/sssp.cpp:run (sssp.cpp:11-37). */
#include "apps/graph_analytics/sssp.h"
#include "dump_common.h"

int main(int argc, char* argv[])
{
  Env::init();
  if (argc < 5) { std::fprintf(stderr, "usage: %s <file.w> <n> <root> <out_prefix>\n", argv[0]); return 1; }
  std::string path = argv[1];
  vid_t n = (vid_t) std::atol(argv[2]);
  vid_t root = (vid_t) std::atol(argv[3]);
  std::string out = argv[4];

  Graph<ew_t> G;
  G.load_directed(true, path, n);
  SpVertex vp(&G);
  vp.root = root;
  vp.initialize();
  double t0 = Env::now();
  vp.execute();
  double t = Env::now() - t0;

  size_t N = (size_t) G.get_nvertices() + 1;
  std::vector<uint32_t> dist(N, 0);
  vp.reduce<long>([&](uint32_t idx, const SpState& s) -> long { dist[idx] = s.distance.value; return 0; },
                  [&](long&, const long&) {});
  long nreach = vp.reduce<long>([&](uint32_t, const SpState& s) -> long { return s.distance != INF; },
                                [&](long& a, const long& b) { a += b; });
  long checksum = vp.reduce<long>([&](uint32_t, const SpState& s) -> long { return s.distance.value; },
                                  [&](long& a, const long& b) { a += b; });
  dump_array(out + ".dist.u32", dist);
  std::printf("{\"app\": \"sssp\", \"exec_s\": %.9f, \"reachable\": %ld, \"checksum\": %ld, \"nslots\": %zu}\n",
              t, nreach, checksum, N);
  Env::finalize();
  return 0;
}
