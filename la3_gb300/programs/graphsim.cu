// Graph simulation (src/apps/graph_simulation/graphsim.h:60-184,
// graphsim.cpp:45-90) as a vertex program on la3g_vp::Engine.
//
// The reference's messages and accumulators are variable-size
// (SerializableVector<bool> / <int> of the query's size); here the query has
// at most 32 vertices, so a message is a 32-bit mask of the sender's
// mismatched query vertices and an accumulator 32 counters, which keeps the
// generic engine's fixed-size types.  The reference runs InitVertex first
// (label, and out-degree as the in-degree of the reversed graph) on states
// that GsVertex then shares; here GsProgram's init takes the label and the
// degree (DegVertex on the same reversed graph, la3gp_degree) by vertex id.
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "la3g.h"
#include "la3g_programs.h"
#include "la3g_vp.cuh"

using la3g_vp::Edge;

namespace {

constexpr int kQMax = 32;
constexpr uint32_t kQMaxEdges = 1024;

struct GsQuery
{
  uint32_t qsize;
  uint32_t label[kQMax];
  uint32_t cptr[kQMax + 1];  // children of query vertex i: cidx[cptr[i], cptr[i + 1]), file order
  uint32_t cidx[kQMaxEdges];
};

// GsState (graphsim.h:24-58)
struct GsState
{
  uint32_t vid, label;
  int32_t degree, deps;
  uint32_t mm;          // temp mismatches, bit i = query vertex i
  int32_t pm[kQMax];    // potential matches
  uint8_t res[kQMax];   // 'U' | '0' | '1'
};

struct GsAcc
{
  int32_t c[kQMax];  // per query vertex: in-neighbours that mismatched it
};

struct GsProgram
{
  using Msg = uint32_t;
  using Acc = GsAcc;
  using State = GsState;
  static constexpr bool stationary = false;
  static constexpr bool gather_with_state = false;
  static constexpr bool apply_with_iteration = true;
  static constexpr bool associative = true;  // counters add up in any grouping
  const GsQuery* q;          // device
  const uint32_t* vlabel;    // device, by vertex id
  const uint32_t* degree;    // device, by vertex id

  // GsVertex::init (graphsim.h:110-137), after InitVertex (:77-84)
  __device__ bool init(uint32_t vid, State& s) const
  {
    s.vid = vid;
    s.label = vlabel[vid];
    s.degree = (int32_t) degree[vid];
    s.deps = 0;
    s.mm = 0;
    const uint32_t n = q->qsize;
    for (uint32_t i = 0; i < n; i++)
    {
      s.res[i] = 'U';
      s.pm[i] = -1;
    }
    for (uint32_t i = 0; i < n; i++)
    {
      const bool same = s.label == q->label[i];
      if (same && q->cptr[i] == q->cptr[i + 1]) s.res[i] = '1';
      else if (same && s.degree > 0)
      {
        s.deps++;
        for (uint32_t e = q->cptr[i]; e < q->cptr[i + 1]; e++) s.pm[q->cidx[e]] = s.degree;
      }
      else
      {
        s.res[i] = '0';
        s.mm |= 1u << i;
      }
    }
    return s.mm != 0;
  }
  __device__ Msg scatter(const State& s) const { return s.mm; }
  __device__ Acc gather(const Edge&, const Msg& m, const State&) const
  {
    Acc a;
#pragma unroll
    for (int i = 0; i < kQMax; i++) a.c[i] = (int32_t) ((m >> i) & 1u);
    return a;
  }
  __device__ void combine(const Acc& y1, Acc& y2) const
  {
#pragma unroll
    for (int i = 0; i < kQMax; i++) y2.c[i] += y1.c[i];
  }
  // GsVertex::apply (graphsim.h:148-182): only the first undecided query
  // vertex is looked at; its children's potential matches drop by the
  // mismatch counts, and one reaching zero mismatches it.
  __device__ bool apply(const Acc& y, State& s, uint32_t) const
  {
    if (s.label == 0) return false;  // s.label.empty()
    s.mm = 0;
    const uint32_t n = q->qsize;
    for (uint32_t i = 0; i < n; i++)
    {
      if (s.res[i] != 'U') continue;
      for (uint32_t e = q->cptr[i]; e < q->cptr[i + 1]; e++)
      {
        const uint32_t j = q->cidx[e];
        if (s.pm[j] > 0)
        {
          s.pm[j] -= y.c[j];
          if (s.pm[j] == 0)
          {
            s.res[i] = '0';
            s.mm |= 1u << i;
            s.deps--;
            break;
          }
        }
      }
      break;
    }
    return s.mm != 0;
  }
  __device__ Acc zero() const
  {
    Acc a;
#pragma unroll
    for (int i = 0; i < kQMax; i++) a.c[i] = 0;
    return a;
  }
};

// is_matched (graphsim.h:50-57) and the per-query-vertex results of every
// vertex, by original id, computed where the states are (a state is ~180
// bytes; the outputs are 1 + qsize bytes per vertex).
__global__ void k_gs_results(uint32_t N, const uint32_t* __restrict__ id_of_pos, const GsState* __restrict__ S,
                             uint32_t qsize, uint8_t* matched, char* res, unsigned long long* nmatches)
{
  unsigned long long cnt = 0;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x)
  {
    const uint32_t v = id_of_pos[p];
    bool m = false;
    for (uint32_t i = 0; i < qsize; i++)
    {
      const uint8_t r = S[p].res[i];
      m |= r != '0';
      if (res) res[(size_t) v * qsize + i] = (char) r;
    }
    matched[v] = m;
    cnt += m;
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(nmatches, cnt);
}

}  // namespace

extern "C" int la3gp_graphsim(la3g_graph* gr, const uint32_t* vlabel, uint32_t qsize, const uint32_t* qlabel,
                              const uint32_t* qedges, uint32_t nqedges, uint8_t* matched, char* res,
                              uint32_t* nmatches, uint32_t* iters)
{
  if (!gr || !vlabel || !qlabel || (nqedges && !qedges)) return LA3G_EINVAL;
  if (qsize == 0 || qsize > (uint32_t) kQMax || nqedges > kQMaxEdges) return LA3G_EINVAL;
  la3g_graph_info gi;
  if (la3g_graph_info_get(gr, &gi) != LA3G_OK) return LA3G_EINVAL;
  if ((gi.flags & (LA3G_DIRECTED | LA3G_REVERSE)) != (LA3G_DIRECTED | LA3G_REVERSE)) return LA3G_EINVAL;
  GsQuery hq{};
  hq.qsize = qsize;
  for (uint32_t i = 0; i < qsize; i++) hq.label[i] = qlabel[i];
  for (uint32_t e = 0; e < nqedges; e++)
  {
    if (qedges[2 * e] >= qsize || qedges[2 * e + 1] >= qsize) return LA3G_EINVAL;
    hq.cptr[qedges[2 * e] + 1]++;
  }
  for (uint32_t i = 0; i < qsize; i++) hq.cptr[i + 1] += hq.cptr[i];
  std::vector<uint32_t> fill(qsize, 0);
  for (uint32_t e = 0; e < nqedges; e++)
  {
    const uint32_t i = qedges[2 * e];
    hq.cidx[hq.cptr[i] + fill[i]++] = qedges[2 * e + 1];
  }
  const uint32_t N = (uint32_t) gi.nslots;
  std::vector<uint32_t> deg(N, 0);
  int st = la3gp_degree(gr, deg.data());  // InitVertex's degree (DegVertex on the reversed graph)
  if (st != LA3G_OK) return st;
  GsQuery* dq = nullptr;
  uint32_t *dl = nullptr, *dd = nullptr;
  uint8_t* dm = nullptr;
  char* dr = nullptr;
  unsigned long long* dn = nullptr;
  auto release = [&]() {
    cudaFree(dq);
    cudaFree(dl);
    cudaFree(dd);
    cudaFree(dm);
    cudaFree(dr);
    cudaFree(dn);
  };
  if (cudaMalloc(&dq, sizeof(GsQuery)) != cudaSuccess || cudaMalloc(&dl, (size_t) N * 4) != cudaSuccess ||
      cudaMalloc(&dd, (size_t) N * 4) != cudaSuccess || cudaMalloc(&dm, N) != cudaSuccess ||
      cudaMalloc(&dn, 8) != cudaSuccess || (res && cudaMalloc(&dr, (size_t) N * qsize) != cudaSuccess))
  {
    cudaGetLastError();
    release();
    return LA3G_ENOMEM;
  }
  cudaMemcpy(dq, &hq, sizeof(GsQuery), cudaMemcpyHostToDevice);
  cudaMemcpy(dl, vlabel, (size_t) N * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dd, deg.data(), (size_t) N * 4, cudaMemcpyHostToDevice);
  cudaMemset(dn, 0, 8);
  unsigned long long nm = 0;
  {
    la3g_vp::Engine<GsProgram> e(gr, GsProgram{dq, dl, dd});
    st = e.initialize();
    if (st == LA3G_OK) st = e.execute(0, iters);  // until convergence (graphsim.cpp:72)
    if (st == LA3G_OK)
    {
      cudaStream_t s = (cudaStream_t) e.view().stream;
      k_gs_results<<<(N + 255) / 256, 256, 0, s>>>(N, e.view().id_of_pos, e.device_states(), qsize, dm, dr, dn);
      if (cudaGetLastError() != cudaSuccess) st = LA3G_ECUDA;
      if (st == LA3G_OK && cudaStreamSynchronize(s) != cudaSuccess) st = LA3G_ECUDA;
    }
  }
  if (st == LA3G_OK)
  {
    if (cudaMemcpy(&nm, dn, 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        (matched && cudaMemcpy(matched, dm, N, cudaMemcpyDeviceToHost) != cudaSuccess) ||
        (res && cudaMemcpy(res, dr, (size_t) N * qsize, cudaMemcpyDeviceToHost) != cudaSuccess))
      st = LA3G_ECUDA;
  }
  release();
  if (st != LA3G_OK) return st;
  if (nmatches) *nmatches = (uint32_t) nm;
  return LA3G_OK;
}
