/* Reference TC dump: replays apps/graph_analytics/tc.cpp:run (tc.cpp:11-52). */
#include "apps/graph_analytics/tc.h"
#include "dump_common.h"

int main(int argc, char* argv[])
{
  Env::init();
  if (argc < 4) { std::fprintf(stderr, "usage: %s <file> <n> <out_prefix>\n", argv[0]); return 1; }
  std::string path = argv[1];
  vid_t n = (vid_t) std::atol(argv[2]);
  std::string out = argv[3];

  Graph<ew_t>* G = new Graph<ew_t>();
  G->load_directed(true, path, n, false, true);
  Graph<ew_t> GR;
  GR.load_directed(true, path, n, true, true);
  GnVertex* vp_gn = new GnVertex(G, true);
  vp_gn->initialize();
  double t0 = Env::now();
  vp_gn->execute(1);
  double t1 = Env::now();
  delete G;
  CtVertex vp_ct(&GR, true);
  vp_ct.initialize(*vp_gn);
  delete vp_gn;
  double t2 = Env::now();
  vp_ct.execute(1);
  double t3 = Env::now();

  size_t N = (size_t) GR.get_nvertices() + 1;
  std::vector<uint32_t> ntri(N, 0);
  vp_ct.reduce<long>([&](uint32_t idx, const CtState& s) -> long { ntri[idx] = s.ntriangles; return 0; },
                     [&](long&, const long&) {});
  long total = vp_ct.reduce<long>([&](uint32_t, const CtState& s) -> long { return s.ntriangles; },
                                  [&](long& a, const long& b) { a += b; });
  dump_array(out + ".ntri.u32", ntri);
  std::printf("{\"app\": \"tc\", \"exec_s\": %.9f, \"p1_s\": %.9f, \"p2_s\": %.9f, \"triangles\": %ld, \"nslots\": %zu}\n",
              (t1 - t0) + (t3 - t2), t1 - t0, t3 - t2, total, N);
  Env::finalize();
  return 0;
}
