/*
 * Reference CPU benchmark driver (test / baseline infrastructure).
 *
 * Times the reference's own implementation of the plain apps on one
 * workload: every graph is ingested once (Graph::load_*, untimed), then the
 * apps run through the sequences of their run() functions (bfs.cpp:11-37,
 * sssp.cpp:11-37, cc.cpp:11-31, tc.cpp:11-52), and only the execute()
 * windows are timed, as the apps' own DistTimer windows are (TC: pass 1 and
 * pass 2).  The TEPS numerators come from the results and from the input
 * files (not timed):
 *   BFS  = undirected edges with both endpoints reached
 *   SSSP = directed edges whose source is reachable
 *   CC   = stored symmetric entries
 *   TC   = undirected edges
 *
 *   bench_ref <pairs> <triples> <n> <tc_pairs> <n_tc> <warmup> <steps> <cc_runs> <tc_runs>
 *             <bfs_root0> <sssp_root0> [<bfs_root1> <sssp_root1> ...]
 *
 * Plan: `warmup` untimed BFS runs, then `cc_runs` CC runs and `tc_runs` TC
 * runs, then `steps` steps that alternate BFS and SSSP: step k runs BFS
 * (k even) or SSSP (k odd) from root pair k / 2 (modulo the pair count).
 * One JSON line per run, then a summary line with the per-app sums.
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

static void line(const char* app, uint32_t root, double s, uint64_t e, bool warm)
{
  std::printf("{\"app\": \"%s\", \"root\": %u, \"s\": %.9f, \"e\": %llu, \"warmup\": %s}\n", app, root, s,
              (unsigned long long) e, warm ? "true" : "false");
  std::fflush(stdout);
}

int main(int argc, char** argv)
{
  Env::init();
  if (argc < 11)
  {
    std::fprintf(stderr,
                 "usage: %s <pairs> <triples> <n> <tc_pairs> <n_tc> <warmup> <steps> <cc_runs> <tc_runs> <root>...\n",
                 argv[0]);
    return 1;
  }
  const char* pairs = argv[1];
  const char* triples = argv[2];
  uint32_t n = (uint32_t) std::atol(argv[3]);
  const char* tcpairs = argv[4];
  uint32_t ntc = (uint32_t) std::atol(argv[5]);
  const int warmup = std::atoi(argv[6]), steps = std::atoi(argv[7]), cc_runs = std::atoi(argv[8]),
            tc_runs = std::atoi(argv[9]);
  std::vector<uint32_t> broots, sroots;
  for (int i = 10; i + 1 < argc; i += 2)
  {
    broots.push_back((uint32_t) std::atol(argv[i]));
    sroots.push_back((uint32_t) std::atol(argv[i + 1]));
  }
  if (broots.empty())
  {
    std::fprintf(stderr, "bench_ref: no root pair given\n");
    return 1;
  }

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
  // TC's two graphs (tc.cpp:14-20), loaded once and kept for every run
  Graph<Empty> GT;
  GT.load_directed(true, tcpairs, ntc, false, true);
  Graph<Empty> GR;
  GR.load_directed(true, tcpairs, ntc, true, true);
  double t_ing_end = Env::now();

  auto run_bfs = [&](uint32_t root, uint64_t* e) {
    BfsVertex vp(&GU);
    vp.root = root;
    vp.initialize();
    double t0 = Env::now();
    vp.execute();
    double t = Env::now() - t0;
    long reached_deg = vp.reduce<long>(
        [&](uint32_t idx, const BfsState& st) -> long { return st.hops != BFS_INF_ ? (long) deg_u[idx] : 0L; },
        [&](long& a, const long& b) { a += b; });
    *e = (uint64_t) reached_deg / 2;
    return t;
  };
  auto run_sssp = [&](uint32_t root, uint64_t* e) {
    sssp_ns::SpVertex vp(&GW);
    vp.root = root;
    vp.initialize();
    double t0 = Env::now();
    vp.execute();
    double t = Env::now() - t0;
    long reached = vp.reduce<long>(
        [&](uint32_t idx, const sssp_ns::SpState& st) -> long {
          return st.distance != sssp_ns::INF ? (long) deg_o[idx] : 0L;
        },
        [&](long& a, const long& b) { a += b; });
    *e = (uint64_t) reached;
    return t;
  };

  double tot_t[4] = {0, 0, 0, 0};
  uint64_t tot_e[4] = {0, 0, 0, 0};
  int runs[4] = {0, 0, 0, 0};
  for (int w = 0; w < warmup; w++)
  {
    uint64_t e = 0;
    uint32_t root = broots[w % broots.size()];
    const double t = run_bfs(root, &e);
    line("bfs", root, t, e, true);
  }
  for (int r = 0; r < cc_runs; r++)
  {
    cc_ns::CcVertex vp(&GU);
    vp.initialize();
    double t0 = Env::now();
    vp.execute();
    double t = Env::now() - t0;
    tot_t[2] += t;
    tot_e[2] += m_sym;
    runs[2]++;
    line("cc", 0, t, m_sym, false);
  }
  for (int r = 0; r < tc_runs; r++)
  {
    auto* vp_gn = new tc_ns::GnVertex(&GT, true);
    vp_gn->initialize();
    double t0 = Env::now();
    vp_gn->execute(1);
    double t1 = Env::now();
    tc_ns::CtVertex vp_ct(&GR, true);
    vp_ct.initialize(*vp_gn);
    delete vp_gn;
    double t2 = Env::now();
    vp_ct.execute(1);
    double t3 = Env::now();
    double t = (t1 - t0) + (t3 - t2);
    tot_t[3] += t;
    tot_e[3] += m_tc;
    runs[3]++;
    line("tc", 0, t, m_tc, false);
  }
  for (int k = 0; k < steps; k++)
  {
    const size_t j = (size_t) (k / 2) % broots.size();
    uint64_t e = 0;
    if (k % 2 == 0)
    {
      double t = run_bfs(broots[j], &e);
      tot_t[0] += t;
      tot_e[0] += e;
      runs[0]++;
      line("bfs", broots[j], t, e, false);
    }
    else
    {
      double t = run_sssp(sroots[j], &e);
      tot_t[1] += t;
      tot_e[1] += e;
      runs[1]++;
      line("sssp", sroots[j], t, e, false);
    }
  }
  std::printf("{\"summary\": true, \"ingest_s\": %.3f, \"runs\": {\"bfs\": %d, \"sssp\": %d, \"cc\": %d, \"tc\": %d}, "
              "\"bfs_s\": %.9f, \"sssp_s\": %.9f, \"cc_s\": %.9f, \"tc_s\": %.9f, \"bfs_e\": %llu, \"sssp_e\": %llu, "
              "\"cc_e\": %llu, \"tc_e\": %llu}\n",
              t_ing_end - t_ing, runs[0], runs[1], runs[2], runs[3], tot_t[0], tot_t[1], tot_t[2], tot_t[3],
              (unsigned long long) tot_e[0], (unsigned long long) tot_e[1], (unsigned long long) tot_e[2],
              (unsigned long long) tot_e[3]);
  Env::finalize();
  return 0;
}
