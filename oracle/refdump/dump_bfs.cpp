/* Reference BFS dump: replays apps/graph_analytics/bfs.cpp:run (bfs.cpp:11-37). */
#include "apps/graph_analytics/bfs.h"
#include "dump_common.h"

int main(int argc, char* argv[])
{
  Env::init();
  if (argc < 5) { std::fprintf(stderr, "usage: %s <file> <n> <root> <out_prefix>\n", argv[0]); return 1; }
  std::string path = argv[1];
  vid_t n = (vid_t) std::atol(argv[2]);
  vid_t root = (vid_t) std::atol(argv[3]);
  std::string out = argv[4];

  Graph<ew_t> G;
  G.load_undirected(true, path, n);
  BfsVertex vp(&G);
  vp.root = root;
  vp.initialize();
  double t0 = Env::now();
  vp.execute();
  double t = Env::now() - t0;

  size_t N = (size_t) G.get_nvertices() + 1;
  std::vector<uint8_t> hops(N, 0);
  std::vector<uint32_t> parent(N, 0);
  vp.reduce<long>([&](uint32_t idx, const BfsState& s) -> long { hops[idx] = s.hops; parent[idx] = s.parent; return 0; },
                  [&](long&, const long&) {});
  long nreach = vp.reduce<long>([&](uint32_t, const BfsState& s) -> long { return s.hops != INF; },
                                [&](long& a, const long& b) { a += b; });
  long checksum = vp.reduce<long>([&](uint32_t, const BfsState& s) -> long { return s.hops * s.parent; },
                                  [&](long& a, const long& b) { a += b; });
  dump_array(out + ".hops.u8", hops);
  dump_array(out + ".parent.u32", parent);
  std::printf("{\"app\": \"bfs\", \"exec_s\": %.9f, \"reachable\": %ld, \"checksum\": %ld, \"nslots\": %zu}\n",
              t, nreach, checksum, N);
  Env::finalize();
  return 0;
}
