/*
 * Reference graph simulation dump: replays
 * apps/graph_simulation/graphsim.cpp:run (graphsim.cpp:45-90) through the
 * reference's InitVertex / GsVertex / Query and writes, per vertex id
 * 0..nvertices, its result string res[0..qsize) and is_matched().  The data
 * labels file is read by the rules of graphsim.cpp:14-40 (first line "[",
 * then one {"key":"label"} line per vertex, a first line "null," for a
 * vertex 0 without a label).
 */
#include <cstring>
#include <fstream>
#include "utils/dist_timer.h"
#include "apps/graph_simulation/graphsim.h"
#include "dump_common.h"

static void read_data_labels(const std::string& path, std::vector<std::string>& labels)
{
  std::ifstream f(path);
  char buf[2048];
  f.getline(buf, sizeof buf);  // "["
  for (size_t i = 0; i < labels.size(); i++)
  {
    f.getline(buf, sizeof buf);
    if (i == 0 && std::strcmp(buf, "null,") == 0) continue;
    char* t = std::strtok(buf, ":");
    t = t ? std::strtok(nullptr, ":") : nullptr;
    t = t ? std::strtok(t + 1, "\"") : nullptr;
    if (t) labels[i] = std::string(t);
  }
}

int main(int argc, char** argv)
{
  Env::init();
  if (argc < 7)
  {
    std::fprintf(stderr, "usage: %s <data.labels> <data.bin> <nvertices> <query.labels> <query.mtx> <out_prefix>\n",
                 argv[0]);
    return 1;
  }
  std::string dgl = argv[1], dgm = argv[2], qgl = argv[4], qgm = argv[5], out = argv[6];
  vid_t n = (vid_t) atoi(argv[3]);
  Graph<ew_t> GR;
  GR.load_directed(true, dgm, n, true);
  GsVertex vp(&GR);
  InitVertex vp_init(vp, true);
  std::vector<std::string> labels(n);
  read_data_labels(dgl, labels);
  vp_init.labels = &labels;
  vp_init.execute(1);
  Query query(qgl, qgm);
  vp.q = &query;
  double t0 = Env::now();
  vp.execute();
  double t1 = Env::now();
  const size_t N = (size_t) GR.get_nvertices() + 1;
  const size_t Q = (size_t) query.size;
  std::vector<char> res(N * Q, '?');
  std::vector<uint8_t> matched(N, 0);
  vid_t nm = vp.reduce<vid_t>([&](uint32_t idx, const GsState& s) -> vid_t {
                                for (size_t i = 0; i < Q && i < s.res.size(); i++) res[idx * Q + i] = s.res[i];
                                matched[idx] = s.is_matched() ? 1 : 0;
                                return s.is_matched() ? 1 : 0; },
                              [&](vid_t& a, const vid_t& b) { a += b; });
  dump_array(out + ".res.u8", res);
  dump_array(out + ".matched.u8", matched);
  std::printf("{\"app\": \"graphsim\", \"nmatches\": %u, \"qsize\": %zu, \"exec_s\": %.9f, \"nslots\": %zu}\n", nm, Q,
              t1 - t0, N);
  Env::finalize();
  return 0;
}
