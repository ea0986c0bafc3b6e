/*
 * Reference CPU benchmark driver (test / baseline infrastructure).
 *
 * Times the reference's own implementation of the plain apps on one
 * workload: each graph is ingested once (Graph::load_*, untimed), then each
 * step runs BFS and SSSP from the step's root, CC and TC, replaying the apps'
 * run() sequences (bfs.cpp:11-37, sssp.cpp:11-37, cc.cpp:11-31,
 * tc.cpp:11-52).  Only the execute() windows are timed, as the apps' own
 * DistTimer windows are.  The TEPS numerators are computed from the results
 * and from the input files (not timed):
 *   BFS  = undirected edges with both endpoints reached
 *   SSSP = directed edges whose source is reachable
 *   CC   = stored symmetric entries
 *   TC   = undirected edges
 *
 *   bench_ref <pairs> <triples> <n> <tc_pairs> <n_tc> <steps> <root0> [root1 ...]
 * One JSON line per step, then a summary line.
 */
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "apps/graph_analytics/bfs.h"
#undef INF
#define BFS_INF_ 255
#include "dump_common.h"

namespace sssp_ns {
#include "apps/graph_analytics/sssp.h"
}
namespace cc_ns {
#include "apps/graph_analytics/cc.h"
}
namespace tc_ns {
#include "apps/graph_analytics/tc.h"
}

static std::vector<uint32_t> read_u32(const char* path)
{
  FILE* f = std::fopen(path, "rb");
  if (!f) { std::perror(path); std::exit(2); }
  std::fseek(f, 0, SEEK_END);
  long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  std::vector<uint32_t> v(sz / 4);
  if (!v.empty() && std::fread(v.data(), 4, v.size(), f) != v.size()) { std::perror(path); std::exit(2); }
  std::fclose(f);
  return v;
}

// unique neighbour counts (self-loops dropped) over records with the given stride
static std::vector<uint32_t> degrees(const std::vector<uint32_t>& rec, int stride, uint32_t N, bool undirected,
                                     uint64_t* nuniq)
{
  std::vector<uint64_t> keys;
  keys.reserve(rec.size() / stride * (undirected ? 2 : 1));
  for (size_t i = 0; i + stride <= rec.size(); i += stride)
  {
    uint32_t s = rec[i], d = rec[i + 1];
    if (s == d) continue;
    keys.push_back((uint64_t) s << 32 | d);
    if (undirected) keys.push_back((uint64_t) d << 32 | s);
  }
  std::sort(keys.begin(), keys.end());
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  std::vector<uint32_t> deg(N, 0);
  for (uint64_t k : keys) deg[k >> 32]++;
  *nuniq = keys.size();
  return deg;
}

int main(int argc, char** argv)
{
  Env::init();
  if (argc < 8)
  {
    std::fprintf(stderr, "usage: %s <pairs> <triples> <n> <tc_pairs> <n_tc> <steps> <root>...\n", argv[0]);
    return 1;
  }
  const char* pairs = argv[1];
  const char* triples = argv[2];
  uint32_t n = (uint32_t) std::atol(argv[3]);
  const char* tcpairs = argv[4];
  uint32_t ntc = (uint32_t) std::atol(argv[5]);
  int steps = std::atoi(argv[6]);
  std::vector<uint32_t> roots;
  for (int i = 7; i < argc; i++) roots.push_back((uint32_t) std::atol(argv[i]));

  uint64_t m_sym = 0, m_dir = 0, m_tc = 0;
  std::vector<uint32_t> deg_u = degrees(read_u32(pairs), 2, n + 1, true, &m_sym);
  std::vector<uint32_t> deg_o = degrees(read_u32(triples), 3, n + 1, false, &m_dir);
  degrees(read_u32(tcpairs), 2, ntc + 1, true, &m_tc);
  m_tc /= 2;

  double t_ing = Env::now();
  Graph<Empty> GU;
  GU.load_undirected(true, pairs, n);
  Graph<uint32_t> GW;
  GW.load_directed(true, triples, n);
  double t_ing_end = Env::now();

  double tot_t[4] = {0, 0, 0, 0};
  uint64_t tot_e[4] = {0, 0, 0, 0};
  for (int s = 0; s < steps; s++)
  {
    uint32_t root = roots[s % roots.size()];
    double t[4];
    uint64_t e[4];
    {  // BFS
      BfsVertex vp(&GU);
      vp.root = root;
      vp.initialize();
      double t0 = Env::now();
      vp.execute();
      t[0] = Env::now() - t0;
      long reached_deg = vp.reduce<long>(
          [&](uint32_t idx, const BfsState& st) -> long { return st.hops != BFS_INF_ ? (long) deg_u[idx] : 0L; },
          [&](long& a, const long& b) { a += b; });
      e[0] = (uint64_t) reached_deg / 2;
    }
    {  // SSSP
      sssp_ns::SpVertex vp(&GW);
      vp.root = root;
      vp.initialize();
      double t0 = Env::now();
      vp.execute();
      t[1] = Env::now() - t0;
      long reached = vp.reduce<long>(
          [&](uint32_t idx, const sssp_ns::SpState& st) -> long {
            return st.distance != sssp_ns::INF ? (long) deg_o[idx] : 0L;
          },
          [&](long& a, const long& b) { a += b; });
      e[1] = (uint64_t) reached;
    }
    {  // CC
      cc_ns::CcVertex vp(&GU);
      vp.initialize();
      double t0 = Env::now();
      vp.execute();
      t[2] = Env::now() - t0;
      e[2] = m_sym;
    }
    {  // TC (its two graphs are loaded per run, as tc.cpp does; ingest is not timed)
      auto* G = new Graph<Empty>();
      G->load_directed(true, tcpairs, ntc, false, true);
      Graph<Empty> GR;
      GR.load_directed(true, tcpairs, ntc, true, true);
      auto* vp_gn = new tc_ns::GnVertex(G, true);
      vp_gn->initialize();
      double t0 = Env::now();
      vp_gn->execute(1);
      double t1 = Env::now();
      delete G;
      tc_ns::CtVertex vp_ct(&GR, true);
      vp_ct.initialize(*vp_gn);
      delete vp_gn;
      double t2 = Env::now();
      vp_ct.execute(1);
      double t3 = Env::now();
      t[3] = (t1 - t0) + (t3 - t2);
      e[3] = m_tc;
    }
    for (int a = 0; a < 4; a++) { tot_t[a] += t[a]; tot_e[a] += e[a]; }
    std::printf("{\"step\": %d, \"root\": %u, \"bfs_s\": %.9f, \"sssp_s\": %.9f, \"cc_s\": %.9f, \"tc_s\": %.9f, "
                "\"bfs_e\": %llu, \"sssp_e\": %llu, \"cc_e\": %llu, \"tc_e\": %llu}\n",
                s, root, t[0], t[1], t[2], t[3], (unsigned long long) e[0], (unsigned long long) e[1],
                (unsigned long long) e[2], (unsigned long long) e[3]);
    std::fflush(stdout);
  }
  std::printf("{\"summary\": true, \"steps\": %d, \"ingest_s\": %.3f, \"bfs_s\": %.9f, \"sssp_s\": %.9f, "
              "\"cc_s\": %.9f, \"tc_s\": %.9f, \"bfs_e\": %llu, \"sssp_e\": %llu, \"cc_e\": %llu, \"tc_e\": %llu}\n",
              steps, t_ing_end - t_ing, tot_t[0], tot_t[1], tot_t[2], tot_t[3], (unsigned long long) tot_e[0],
              (unsigned long long) tot_e[1], (unsigned long long) tot_e[2], (unsigned long long) tot_e[3]);
  Env::finalize();
  return 0;
}
