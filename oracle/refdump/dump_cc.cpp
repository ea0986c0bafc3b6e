/* Reference CC dump: replays apps/graph_analytics/cc.cpp:run (cc.cpp:11-31). */
#include "apps/graph_analytics/cc.h"
#include "dump_common.h"

int main(int argc, char* argv[])
{
  Env::init();
  if (argc < 4) { std::fprintf(stderr, "usage: %s <file> <n> <out_prefix>\n", argv[0]); return 1; }
  std::string path = argv[1];
  vid_t n = (vid_t) std::atol(argv[2]);
  std::string out = argv[3];

  Graph<ew_t> G;
  G.load_undirected(true, path, n);
  CcVertex vp(&G);
  vp.initialize();
  double t0 = Env::now();
  vp.execute();
  double t = Env::now() - t0;

  size_t N = (size_t) G.get_nvertices() + 1;
  std::vector<uint32_t> label(N, 0);
  vp.reduce<long>([&](uint32_t idx, const CcState& s) -> long { label[idx] = s.label; return 0; },
                  [&](long&, const long&) {});
  long checksum = vp.reduce<long>([&](uint32_t, const CcState& s) -> long { return s.label; },
                                  [&](long& a, const long& b) { a += b; });
  dump_array(out + ".label.u32", label);
  std::printf("{\"app\": \"cc\", \"exec_s\": %.9f, \"checksum\": %ld, \"nslots\": %zu}\n", t, checksum, N);
  Env::finalize();
  return 0;
}
