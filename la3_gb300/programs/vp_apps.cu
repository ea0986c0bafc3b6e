// The reference's graph apps written as vertex programs against the
// device-functor API (la3g_vp.cuh), the way a user of the reference writes a
// VertexProgram subclass (src/apps/graph_analytics/*.h).  They run through
// the generic engine, not the hand-tuned kernels of libla3g, and serve as
// templates for new programs; their results equal the reference's.
//
// Exported with C linkage (libla3g_programs.so), outputs by vertex id:
//   la3gp_degree(gr, degree)           DegVertex, execute(1), on a reversed graph
//   la3gp_pagerank(g, gr, iters, rank, degree)    pr.cpp:11-55
//   la3gp_bfs(g, root, hops, parent, iters)       bfs.cpp:11-37
//   la3gp_sssp(g, root, dist, iters)              sssp.cpp:11-37
//   la3gp_cc(g, label, iters)                     cc.cpp:11-31
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "la3g.h"
#include "la3g_programs.h"
#include "la3g_vp.cuh"

using la3g_vp::Edge;

namespace {

struct Empty
{
};

// degree.h:17-35
struct DegState
{
  uint32_t degree = 0;
};

struct DegProgram
{
  using Msg = Empty;
  using Acc = uint32_t;
  using State = DegState;
  static constexpr bool stationary = true;
  static constexpr bool gather_with_state = false;
  static constexpr bool apply_with_iteration = false;
  __device__ bool init(uint32_t, State&) const { return true; }
  __device__ Msg scatter(const State&) const { return Msg{}; }
  __device__ Acc gather(const Edge&, const Msg&, const State&) const { return 1u; }
  __device__ void combine(const Acc& y1, Acc& y2) const { y2 += y1; }
  __device__ bool apply(const Acc& y, State& s, uint32_t) const
  {
    s.degree = y;
    return true;
  }
  __device__ Acc zero() const { return 0u; }
};

// pr.h:12-46 (every operation rounded as the reference's compiled code,
// without contraction)
struct PrState
{
  uint32_t degree = 0;
  double rank = 0.15;
};

struct PrProgram
{
  using Msg = double;
  using Acc = double;
  using State = PrState;
  static constexpr bool stationary = true;
  static constexpr bool gather_with_state = false;
  static constexpr bool apply_with_iteration = false;
  const uint32_t* degree_by_id;  // from the degree program (PrVertex::init(vid, other, s))
  __device__ bool init(uint32_t vid, State& s) const
  {
    s.degree = degree_by_id[vid];
    return true;
  }
  __device__ Msg scatter(const State& s) const { return __ddiv_rn(s.rank, (double) s.degree); }
  __device__ Acc gather(const Edge&, const Msg& m, const State&) const { return m; }
  __device__ void combine(const Acc& y1, Acc& y2) const { y2 = __dadd_rn(y2, y1); }
  __device__ bool apply(const Acc& y, State& s, uint32_t) const
  {
    const double tmp = s.rank;
    s.rank = __dadd_rn(0.15, __dmul_rn(1.0 - 0.15, y));
    return fabs(__dsub_rn(s.rank, tmp)) > 1e-5;
  }
  __device__ Acc zero() const { return 0.0; }
};

// bfs.h:11-49
struct BfsState
{
  uint32_t parent = 0;
  uint8_t hops = 255;
};

struct BfsProgram
{
  using Msg = Empty;
  using Acc = uint32_t;
  using State = BfsState;
  static constexpr bool stationary = false;
  static constexpr bool gather_with_state = false;
  static constexpr bool apply_with_iteration = true;
  uint32_t root;
  __device__ bool init(uint32_t vid, State& s) const
  {
    if (vid == root)
    {
      s.hops = 0;
      return true;
    }
    return false;
  }
  __device__ Msg scatter(const State&) const { return Msg{}; }
  __device__ Acc gather(const Edge& e, const Msg&, const State&) const { return e.src; }
  __device__ void combine(const Acc& y1, Acc& y2) const { y2 = y1; }
  __device__ bool apply(const Acc& y, State& s, uint32_t iter) const
  {
    if (s.hops != 255) return false;
    s.hops = (uint8_t) (iter + 1);
    s.parent = y;
    return true;
  }
  __device__ Acc zero() const { return 0u; }
};

// sssp.h:11-46 (INF = UINT32_MAX / 2, the IntegerWrapper default)
constexpr uint32_t kInf = 0x7FFFFFFFu;

struct SpState
{
  uint32_t distance = kInf;
};

struct SpProgram
{
  using Msg = uint32_t;
  using Acc = uint32_t;
  using State = SpState;
  static constexpr bool stationary = false;
  static constexpr bool gather_with_state = false;
  static constexpr bool apply_with_iteration = false;
  uint32_t root;
  __device__ bool init(uint32_t vid, State& s) const
  {
    if (vid == root)
    {
      s.distance = 0;
      return true;
    }
    return false;
  }
  __device__ Msg scatter(const State& s) const { return s.distance; }
  __device__ Acc gather(const Edge& e, const Msg& m, const State&) const { return m + e.weight; }
  __device__ void combine(const Acc& y1, Acc& y2) const { y2 = y1 < y2 ? y1 : y2; }
  __device__ bool apply(const Acc& y, State& s, uint32_t) const
  {
    const uint32_t tmp = s.distance;
    s.distance = y < s.distance ? y : s.distance;
    return tmp != s.distance;
  }
  __device__ Acc zero() const { return kInf; }
};

// cc.h:11-38 (0 acts as "no value yet" in combine)
struct CcState
{
  uint32_t label = 0;
};

struct CcProgram
{
  using Msg = uint32_t;
  using Acc = uint32_t;
  using State = CcState;
  static constexpr bool stationary = false;
  static constexpr bool gather_with_state = false;
  static constexpr bool apply_with_iteration = false;
  __device__ bool init(uint32_t vid, State& s) const
  {
    s.label = vid;
    return true;
  }
  __device__ Msg scatter(const State& s) const { return s.label; }
  __device__ Acc gather(const Edge&, const Msg& m, const State&) const { return m; }
  __device__ void combine(const Acc& y1, Acc& y2) const { y2 = y2 == 0 ? y1 : (y1 < y2 ? y1 : y2); }
  __device__ bool apply(const Acc& y, State& s, uint32_t) const
  {
    const uint32_t tmp = s.label;
    s.label = y < s.label ? y : s.label;
    return tmp != s.label;
  }
  __device__ Acc zero() const { return 0u; }
};

template <class P, class F>
int run(la3g_graph* g, const P& prog, uint32_t iters, uint32_t* iters_out, F&& take)
{
  la3g_vp::Engine<P> e(g, prog);
  int st = e.initialize();
  if (st == LA3G_OK) st = e.execute(iters, iters_out);
  if (st != LA3G_OK) return st;
  la3g_device_graph v = e.view();
  std::vector<typename P::State> out(v.nslots);
  st = e.states(out.data());
  if (st == LA3G_OK) take(out);
  return st;
}

}  // namespace

extern "C" int la3gp_degree(la3g_graph* gr, uint32_t* degree)
{
  if (!gr) return LA3G_EINVAL;
  return run(gr, DegProgram{}, 1, nullptr, [&](const std::vector<DegState>& s) {
    for (size_t i = 0; i < s.size(); i++)
      if (degree) degree[i] = s[i].degree;
  });
}

extern "C" int la3gp_pagerank(la3g_graph* g, la3g_graph* gr, uint32_t iters, double* rank, uint32_t* degree)
{
  if (!g || !gr) return LA3G_EINVAL;
  la3g_device_graph v;
  if (la3g_graph_device_view(g, &v) != LA3G_OK) return LA3G_EINVAL;
  std::vector<uint32_t> deg(v.nslots, 0);
  int st = la3gp_degree(gr, deg.data());
  if (st != LA3G_OK) return st;
  uint32_t* d = nullptr;
  if (cudaMalloc(&d, deg.size() * 4) != cudaSuccess) return LA3G_ENOMEM;
  cudaMemcpy(d, deg.data(), deg.size() * 4, cudaMemcpyHostToDevice);
  PrProgram p{d};
  st = run(g, p, iters, nullptr, [&](const std::vector<PrState>& s) {
    for (size_t i = 0; i < s.size(); i++)
    {
      if (rank) rank[i] = s[i].rank;
      if (degree) degree[i] = s[i].degree;
    }
  });
  cudaFree(d);
  return st;
}

extern "C" int la3gp_bfs(la3g_graph* g, uint32_t root, uint8_t* hops, uint32_t* parent, uint32_t* iters)
{
  if (!g) return LA3G_EINVAL;
  return run(g, BfsProgram{root}, 0, iters, [&](const std::vector<BfsState>& s) {
    for (size_t i = 0; i < s.size(); i++)
    {
      if (hops) hops[i] = s[i].hops;
      if (parent) parent[i] = s[i].parent;
    }
  });
}

extern "C" int la3gp_sssp(la3g_graph* g, uint32_t root, uint32_t* dist, uint32_t* iters)
{
  if (!g) return LA3G_EINVAL;
  return run(g, SpProgram{root}, 0, iters, [&](const std::vector<SpState>& s) {
    for (size_t i = 0; i < s.size(); i++)
      if (dist) dist[i] = s[i].distance;
  });
}

extern "C" int la3gp_cc(la3g_graph* g, uint32_t* label, uint32_t* iters)
{
  if (!g) return LA3G_EINVAL;
  return run(g, CcProgram{}, 0, iters, [&](const std::vector<CcState>& s) {
    for (size_t i = 0; i < s.size(); i++)
      if (label) label[i] = s[i].label;
  });
}
