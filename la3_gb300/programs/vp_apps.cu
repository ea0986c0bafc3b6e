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
  static constexpr bool associative = true;  // integer sum
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
  static constexpr bool associative = true;  // "keep the later value" groups freely
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
  static constexpr bool associative = true;  // min
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

namespace {

// topk / reduce functors (device callable)
struct DegreeOf
{
  __device__ uint32_t operator()(uint32_t, const DegState& s) const { return s.degree; }
};
struct DegreeSum
{
  __device__ unsigned long long operator()(uint32_t, const DegState& s) const { return s.degree; }
};
struct AddU64
{
  __device__ void operator()(unsigned long long& acc, const unsigned long long& v) const { acc += v; }
};
struct Larger
{
  __device__ bool operator()(const la3g_vp::Pair<uint32_t, uint32_t>& a, const la3g_vp::Pair<uint32_t, uint32_t>& b) const
  {
    return a.second > b.second;
  }
};
struct Two
{
  uint32_t v[2];
  __device__ uint32_t operator[](uint32_t b) const { return v[b]; }
};
struct DegreeAndComplement
{
  __device__ Two operator()(uint32_t, const DegState& s) const { return Two{{s.degree, ~s.degree}}; }
};
struct HopsOf
{
  __device__ uint32_t operator()(uint32_t, const BfsState& s) const { return s.hops; }
};

}  // namespace

extern "C" int la3gp_degree_topk(la3g_graph* g, uint32_t k, uint32_t* ids, uint32_t* degrees, uint64_t* degree_sum,
                                 uint32_t* bids, uint32_t* bvals)
{
  if (!g) return LA3G_EINVAL;
  la3g_vp::Engine<DegProgram> e(g, DegProgram{});
  int st = e.initialize();
  if (st == LA3G_OK) st = e.execute(1);
  std::vector<std::pair<uint32_t, uint32_t>> top;
  if (st == LA3G_OK) st = e.topk<uint32_t, uint32_t>(k, top, DegreeOf{}, Larger{});
  if (st != LA3G_OK) return st;
  for (uint32_t i = 0; i < k; i++)
  {
    if (ids) ids[i] = top[i].first;
    if (degrees) degrees[i] = top[i].second;
  }
  unsigned long long sum = 0;
  st = e.reduce<unsigned long long>(&sum, DegreeSum{}, AddU64{});
  if (st != LA3G_OK) return st;
  if (degree_sum) *degree_sum = sum;
  if (bids || bvals)
  {
    std::vector<std::pair<uint32_t, uint32_t>> b2[2];
    st = e.btopk<2, uint32_t, uint32_t>(k, b2, DegreeAndComplement{}, Larger{});
    if (st != LA3G_OK) return st;
    for (uint32_t b = 0; b < 2; b++)
      for (uint32_t i = 0; i < k; i++)
      {
        if (bids) bids[b * k + i] = b2[b][i].first;
        if (bvals) bvals[b * k + i] = b2[b][i].second;
      }
  }
  return LA3G_OK;
}

extern "C" int la3gp_bfs_topk(la3g_graph* g, uint32_t root, uint32_t k, uint32_t* ids, uint32_t* hops)
{
  if (!g) return LA3G_EINVAL;
  la3g_vp::Engine<BfsProgram> e(g, BfsProgram{root});
  int st = e.initialize();
  if (st == LA3G_OK) st = e.execute(0);
  std::vector<std::pair<uint32_t, uint32_t>> top;
  if (st == LA3G_OK) st = e.topk<uint32_t, uint32_t>(k, top, HopsOf{}, Larger{}, true);
  if (st != LA3G_OK) return st;
  for (uint32_t i = 0; i < k; i++)
  {
    if (ids) ids[i] = top[i].first;
    if (hops) hops[i] = top[i].second;
  }
  return LA3G_OK;
}

// ---- TC through the engine (tc.h:47-99, tc.cpp:11-52) ----------------------
//
// GnVertex on the acyclic graph G (edges from the lower to the higher id)
// leaves each vertex the sorted hashed ids of its in-neighbours; CtVertex on
// the reversed acyclic graph starts from those lists, scatters its list (a
// message whose size is the vertex's degree: the engine's variable-size
// message path) and gathers at each row the size of the intersection of the
// row's own list (its state, gather_with_state) with the message; the sum
// over a row's edges is its triangle count.
//
// The Gn pass needs a variable-size accumulator (the reference appends
// edge.src and sorts in apply).  Its result is, for every row of G, the
// hashed ids of the row's columns in ascending order; the pull CSR already
// holds those columns as two ascending runs (source columns, then regular
// columns, each by hashed id), so a merge of the two runs builds the lists.
namespace {

__global__ void k_gn_lists(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col,
                           const uint32_t* __restrict__ hash_of_pos, const uint32_t* __restrict__ id_of_pos,
                           uint32_t nrows, uint32_t src_base, uint32_t* out, uint32_t* off_by_id, uint32_t* len_by_id)
{
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x)
  {
    const uint32_t b = ptr[r], e = ptr[r + 1];
    uint32_t split = b;  // source columns come first
    while (split < e && col[split] >= src_base) split++;
    uint32_t i = b, j = split, k = b;
    while (i < split && j < e)
    {
      const uint32_t hi = hash_of_pos[col[i]], hj = hash_of_pos[col[j]];
      if (hi <= hj)
      {
        out[k++] = hi;
        i++;
      }
      else
      {
        out[k++] = hj;
        j++;
      }
    }
    while (i < split) out[k++] = hash_of_pos[col[i++]];
    while (j < e) out[k++] = hash_of_pos[col[j++]];
    const uint32_t v = id_of_pos[r];
    off_by_id[v] = b;
    len_by_id[v] = e - b;
  }
}

struct CtState
{
  const uint32_t* list;
  uint32_t len;
  uint32_t ntri;
};

struct CtProgram
{
  using Elem = uint32_t;
  using Msg = la3g_vp::MsgView<uint32_t>;
  using Acc = uint32_t;
  using State = CtState;
  static constexpr bool stationary = true;
  static constexpr bool gather_with_state = true;
  static constexpr bool apply_with_iteration = false;
  static constexpr bool associative = true;  // integer sum
  static constexpr bool var_msg = true;
  const uint32_t* gn;      // the Gn lists (device), at gn_off[id], gn_len[id] elements
  const uint32_t* gn_off;
  const uint32_t* gn_len;
  // CtVertex::init (tc.h:76-83): the vertex's Gn list; active iff not empty
  __device__ bool init(uint32_t vid, State& s) const
  {
    s.len = gn_len[vid];
    s.list = gn + gn_off[vid];
    s.ntri = 0;
    return s.len != 0;
  }
  __device__ uint32_t msg_len(const State& s) const { return s.len; }
  __device__ void scatter_into(const State& s, uint32_t* out) const
  {
    for (uint32_t i = 0; i < s.len; i++) out[i] = s.list[i];
  }
  __device__ Msg scatter(const State& s) const { return Msg{s.list, s.len}; }
  // CtVertex::gather (tc.h:86-95): |list(row) n msg| by a sorted merge
  __device__ Acc gather(const Edge&, const Msg& m, const State& s) const
  {
    uint32_t t = 0, i = 0, j = 0;
    while (i < s.len && j < m.len)
    {
      const uint32_t a = s.list[i], b = m.data[j];
      if (a == b)
      {
        t++;
        i++;
        j++;
      }
      else if (a < b) i++;
      else j++;
    }
    return t;
  }
  __device__ void combine(const Acc& y1, Acc& y2) const { y2 += y1; }
  __device__ bool apply(const Acc& y, State& s, uint32_t) const
  {
    s.ntri = y;
    return false;
  }
  __device__ Acc zero() const { return 0u; }
};

struct CtCount
{
  __device__ long long operator()(uint32_t, const CtState& s) const { return (long long) s.ntri; }
};
struct AddI64
{
  __device__ void operator()(long long& a, const long long& b) const { a += b; }
};

}  // namespace

extern "C" int la3gp_tc(la3g_graph* g, la3g_graph* gr, uint64_t* total, uint32_t* ntri)
{
  if (!g || !gr) return LA3G_EINVAL;
  la3g_device_graph v;
  if (la3g_graph_device_view(g, &v) != LA3G_OK) return LA3G_EINVAL;
  const uint32_t N = v.nslots;
  uint32_t *gn = nullptr, *off = nullptr, *len = nullptr;
  if (cudaMalloc(&gn, (size_t) v.nentries * 4 + 4) != cudaSuccess || cudaMalloc(&off, (size_t) N * 4) != cudaSuccess ||
      cudaMalloc(&len, (size_t) N * 4) != cudaSuccess)
  {
    cudaGetLastError();
    cudaFree(gn);
    cudaFree(off);
    return LA3G_ENOMEM;
  }
  cudaStream_t s = (cudaStream_t) v.stream;
  cudaMemsetAsync(off, 0, (size_t) N * 4, s);
  cudaMemsetAsync(len, 0, (size_t) N * 4, s);
  const uint32_t nrows = v.nregular + v.nsink;
  if (nrows)
    k_gn_lists<<<(nrows + 255) / 256, 256, 0, s>>>(v.row_ptr, v.col, v.hash_of_pos, v.id_of_pos, nrows,
                                                  v.nregular + v.nsink, gn, off, len);
  int st = cudaGetLastError() == cudaSuccess ? LA3G_OK : LA3G_ECUDA;
  if (st == LA3G_OK && cudaStreamSynchronize(s) != cudaSuccess) st = LA3G_ECUDA;
  if (st == LA3G_OK)
  {
    la3g_vp::Engine<CtProgram> e(gr, CtProgram{gn, off, len});
    st = e.initialize();
    if (st == LA3G_OK) st = e.execute(1);  // vp_ct.execute(1)
    long long sum = 0;
    if (st == LA3G_OK) st = e.reduce<long long>(&sum, CtCount{}, AddI64{});
    if (st == LA3G_OK && total) *total = (uint64_t) sum;
    if (st == LA3G_OK && ntri)
    {
      std::vector<CtState> out(N);
      st = e.states(out.data());
      for (uint32_t i = 0; st == LA3G_OK && i < N; i++) ntri[i] = out[i].ntri;
    }
  }
  cudaFree(gn);
  cudaFree(off);
  cudaFree(len);
  return st;
}
