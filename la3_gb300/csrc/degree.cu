// Degrees: the reference degree app (src/apps/graph_analytics/degree.cpp:16-46,
// degree.h:17-35) on the device, and a standalone top-k over per-vertex
// uint32 values (vertex_program.hpp:607-680).
//
// DegVertex is stationary, gathers 1 per edge and sums (execute(1) over every
// column, sources included, and the sink rows): a vertex's in-degree is the
// number of its distinct in-neighbours, which is the length of its row in
// the deduplicated pull CSR.  Loaded with LA3G_REVERSE (the reference's
// `-o`, load_directed(..., reverse = true)) the same rows give out-degrees.
// Sources and isolated vertices keep 0.
//
// Top-k: keys (value << 32 | ~id) per block, then one block over the
// candidates; the order is value desc, id asc (the reference's partial_sort
// leaves ties unspecified).
#include <algorithm>

#include "la3g_internal.h"
#include "ir.cuh"

namespace la3g {

__global__ void k_degree(const uint32_t* __restrict__ in_ptr, uint32_t nrows, uint32_t N,
                         const uint32_t* __restrict__ id_of_pos, uint32_t* deg)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x)
    deg[id_of_pos[p]] = p < nrows ? in_ptr[p + 1] - in_ptr[p] : 0u;
}

__global__ void __launch_bounds__(kTopThreads)
k_topk_u32_partial(const uint32_t* __restrict__ v, uint32_t n, int k, unsigned long long* cand)
{
  unsigned long long mine[kTopKMax];
  for (int i = 0; i < k; i++) mine[i] = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    keep_best(mine, k, ((unsigned long long) v[i] << 32) | (0xFFFFFFFFu - i));
  block_topk(mine, k, cand + (size_t) blockIdx.x * k);
}

__global__ void __launch_bounds__(kTopThreads)
k_topk_u32_final(const unsigned long long* __restrict__ cand, int ncand, int k, unsigned long long* best)
{
  unsigned long long mine[kTopKMax];
  for (int i = 0; i < k; i++) mine[i] = 0;
  for (int i = threadIdx.x; i < ncand; i += blockDim.x) keep_best(mine, k, cand[i]);
  block_topk(mine, k, best);
}

// Top k of v[0, n) (device memory) on the stream; results to host arrays.
static int topk_u32(const uint32_t* v, uint32_t n, uint32_t k, cudaStream_t s, uint32_t* ids, uint32_t* vals,
                    uint32_t* nout)
{
  const uint32_t kk = std::min(k, n);
  if (nout) *nout = kk;
  if (kk == 0) return LA3G_OK;
  DevBuf cand, best;
  LA3G_TRY(cand.alloc((size_t) kTopBlocks * kk * 8));
  LA3G_TRY(best.alloc((size_t) kk * 8));
  k_topk_u32_partial<<<kTopBlocks, kTopThreads, 0, s>>>(v, n, (int) kk, cand.as<unsigned long long>());
  LA3G_LAUNCHED();
  k_topk_u32_final<<<1, kTopThreads, 0, s>>>(cand.as<unsigned long long>(), kTopBlocks * (int) kk, (int) kk,
                                             best.as<unsigned long long>());
  LA3G_LAUNCHED();
  tls_launches += 2;
  unsigned long long h[kTopKMax];
  LA3G_CUDA(cudaMemcpyAsync(h, best.p, (size_t) kk * 8, cudaMemcpyDeviceToHost, s));
  LA3G_CUDA(cudaStreamSynchronize(s));
  for (uint32_t i = 0; i < kk; i++)
  {
    if (ids) ids[i] = 0xFFFFFFFFu - (uint32_t) h[i];
    if (vals) vals[i] = (uint32_t) (h[i] >> 32);
  }
  return LA3G_OK;
}

}  // namespace la3g

using namespace la3g;

extern "C" int la3g_degree(la3g_graph* G, uint32_t* degree_out, uint32_t k, uint32_t* topk_ids,
                           uint32_t* topk_degrees, uint32_t* ntopk, la3g_stats* st)
{
  if (!G) return set_error(LA3G_EINVAL, "null graph");
  DevGraph& g = G->g;
  if (!g.directed() || (g.flags & (LA3G_ACYCLIC | LA3G_BIPARTITE)))
    return set_error(LA3G_EINVAL, "degree needs a graph loaded with LA3G_DIRECTED (| LA3G_REVERSE for out-degrees)");
  if (k > kTopKMax) return set_error(LA3G_EINVAL, "k = %u exceeds the maximum of %d", k, kTopKMax);
  CallTimer T(G, st);
  cudaStream_t s = G->stream;
  const uint32_t N = g.nslots;
  DevBuf deg;
  LA3G_TRY(deg.alloc((size_t) N * 4));
  T.device_begin();
  {
    ProfileScope p("degree", s, 4.0 * (g.nrows() + 1) + 4.0 * N);
    k_degree<<<grid_for(N, 256), 256, 0, s>>>(g.in_ptr, g.nrows(), N, g.id_of_pos, deg.as<uint32_t>());
    LA3G_LAUNCHED();
    tls_launches++;
  }
  T.device_end();
  if (degree_out) LA3G_CUDA(cudaMemcpyAsync(degree_out, deg.p, (size_t) N * 4, cudaMemcpyDeviceToHost, s));
  LA3G_TRY(topk_u32(deg.as<uint32_t>(), N, k, s, topk_ids, topk_degrees, ntopk));
  LA3G_CUDA(cudaStreamSynchronize(s));
  LA3G_TRY(T.finish());
  if (st)
  {
    st->iterations = 1;
    st->teps_edges = g.nent;
    st->edges_examined = g.nent;
  }
  return LA3G_OK;
}

extern "C" int la3g_topk_u32(const uint32_t* values, uint32_t n, uint32_t k, uint32_t* ids_out, uint32_t* values_out,
                             uint32_t* nout)
{
  if (n && !values) return set_error(LA3G_EINVAL, "values is null");
  if (k > kTopKMax) return set_error(LA3G_EINVAL, "k = %u exceeds the maximum of %d", k, kTopKMax);
  cudaStream_t s = nullptr;
  LA3G_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  DevBuf v;
  int rc = v.alloc((size_t) std::max<uint32_t>(n, 1) * 4);
  if (!rc && n && cudaMemcpyAsync(v.p, values, (size_t) n * 4, cudaMemcpyHostToDevice, s) != cudaSuccess)
    rc = set_error(LA3G_ECUDA, "upload failed");
  if (!rc) rc = topk_u32(v.as<uint32_t>(), n, k, s, ids_out, values_out, nout);
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  return rc;
}
