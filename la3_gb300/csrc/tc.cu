// Triangle counting: the reference tc app (src/apps/graph_analytics/
// tc.cpp:11-52, tc.h:47-99) on the device.
//
// The reference orients every edge from the lower to the higher original id
// (remove_cycles, graph.hpp:174-179), collects for each vertex v the list
// N<(v) of its lower neighbours (GnVertex), and then, for every oriented
// edge (u, v) with u < v, adds |N<(u) ∩ N<(v)| to u (CtVertex gathers at
// the lower endpoint, accumulating in uint32).  Each triangle w < u < v is
// counted once, at its middle vertex u.
//
// On the device the lists are the rows of the pull CSR of the graph loaded
// with LA3G_DIRECTED | LA3G_ACYCLIC (rows = higher endpoint, entries = lower
// endpoints, all sorted by one column key), and the oriented edges are the
// rows of the push CSR (column u -> its higher neighbours v).  One warp
// handles one edge: lanes take the elements of the shorter list and binary-
// search them in the longer one; the warp's count goes to u with one
// atomicAdd (uint32, wrapping as the reference's accumulator does).
#include <algorithm>
#include <cstring>

#include "la3g_internal.h"

namespace la3g {

struct TcScratch
{
  uint32_t* ntri = nullptr;
  uint32_t* esrc = nullptr;  // lower endpoint of each oriented edge
  unsigned long long* total = nullptr;
};

static void tc_scratch_free(void* p) { delete (TcScratch*) p; }

// column key: sources first, then regular columns (the in-CSR sort order)
__device__ __forceinline__ uint32_t ckey(uint32_t c, uint32_t src_base, uint32_t nsrc)
{
  return c >= src_base ? c - src_base : c + nsrc;
}

// Lower endpoint of every push-CSR entry.
__global__ void k_tc_expand(const uint32_t* __restrict__ optr, uint32_t ncols, uint32_t* __restrict__ src)
{
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < ncols; u += gridDim.x * blockDim.x)
    for (uint32_t e = optr[u]; e < optr[u + 1]; e++) src[e] = u;
}

// One warp per oriented edge (u, v): lanes take the elements of the shorter
// of N<(u), N<(v) and binary-search them in the longer one.
__global__ void __launch_bounds__(256)
k_tc(const uint32_t* __restrict__ esrc, const uint32_t* __restrict__ orow, uint64_t m, const uint32_t* __restrict__ iptr,
     const uint32_t* __restrict__ icol, uint32_t src_base, uint32_t nsrc, uint32_t* ntri)
{
  const int lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t) gridDim.x * blockDim.x) >> 5;
  for (uint64_t e = warp; e < m; e += nwarps)
  {
    const uint32_t u = esrc[e], v = orow[e];
    const uint32_t ub = iptr[u], ue = iptr[u + 1], vb = iptr[v], ve = iptr[v + 1];
    uint32_t ab = ub, ae = ue, bb = vb, be = ve;
    if (ae - ab > be - bb) { ab = vb; ae = ve; bb = ub; be = ue; }
    if (ab == ae) continue;
    uint32_t acc = 0;
    for (uint32_t i = ab + lane; i < ae; i += 32)
    {
      const uint32_t key = ckey(icol[i], src_base, nsrc);
      uint32_t lo = bb, hi = be;
      while (lo < hi)
      {
        uint32_t mid = (lo + hi) >> 1;
        if (ckey(icol[mid], src_base, nsrc) < key) lo = mid + 1;
        else hi = mid;
      }
      if (lo < be && ckey(icol[lo], src_base, nsrc) == key) acc++;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0 && acc) atomicAdd(&ntri[u], acc);
  }
}

__global__ void k_tc_sum(uint32_t N, const uint32_t* __restrict__ ntri, unsigned long long* total)
{
  unsigned long long s = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x) s += ntri[v];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(total, s);
}

__global__ void k_tc_by_id(uint32_t N, const uint32_t* __restrict__ id_of_pos, const uint32_t* __restrict__ v,
                           uint32_t* out)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) out[id_of_pos[p]] = v[p];
}

}  // namespace la3g

using namespace la3g;

extern "C" int la3g_tc(la3g_graph* G, uint64_t* total_out, uint32_t* per_vertex_out, la3g_stats* st)
{
  if (!G) return set_error(LA3G_EINVAL, "null graph");
  DevGraph& g = G->g;
  if ((g.flags & (LA3G_DIRECTED | LA3G_ACYCLIC | LA3G_REVERSE | LA3G_BIPARTITE)) != (LA3G_DIRECTED | LA3G_ACYCLIC))
    return set_error(LA3G_EINVAL, "tc needs a graph loaded with LA3G_DIRECTED | LA3G_ACYCLIC");
  CallTimer T(G, st);
  LA3G_TRY(build_push_csr(G));
  TcScratch* ts = (TcScratch*) G->slot[kSlotTc];
  if (!ts)
  {
    ts = new (std::nothrow) TcScratch();
    if (!ts) return set_error(LA3G_ENOMEM, "out of host memory");
    G->slot[kSlotTc] = ts;
    G->slot_free[kSlotTc] = tc_scratch_free;
    LA3G_TRY(galloc(G, &ts->ntri, g.nslots));
    LA3G_TRY(galloc(G, &ts->total, 1));
    LA3G_TRY(galloc(G, &ts->esrc, g.nent + 1));
    k_tc_expand<<<grid_for(g.nslots, 256), 256, 0, G->stream>>>(g.out_ptr, g.nslots, ts->esrc);
    LA3G_LAUNCHED();
  }
  cudaStream_t s = G->stream;
  const uint32_t N = g.nslots;
  T.device_begin();
  LA3G_CUDA(cudaMemsetAsync(ts->ntri, 0, (size_t) N * 4, s));
  LA3G_CUDA(cudaMemsetAsync(ts->total, 0, 8, s));
  {
    ProfileScope p("tc_intersect", s, 8.0 * g.nent);
    k_tc<<<grid_for((uint64_t) g.nent * 32, 256, kSMs * 32), 256, 0, s>>>(ts->esrc, g.out_row, g.nent, g.in_ptr,
                                                                          g.in_col, g.src_base(), g.nsrc, ts->ntri);
    LA3G_LAUNCHED();
  }
  k_tc_sum<<<grid_for(N, 256), 256, 0, s>>>(N, ts->ntri, ts->total);
  LA3G_LAUNCHED();
  tls_launches++;
  T.device_end();
  unsigned long long total = 0;
  LA3G_CUDA(cudaMemcpyAsync(&total, ts->total, 8, cudaMemcpyDeviceToHost, s));
  if (per_vertex_out)
  {
    DevBuf tmp;
    LA3G_TRY(tmp.alloc((size_t) N * 4));
    k_tc_by_id<<<grid_for(N, 256), 256, 0, s>>>(N, g.id_of_pos, ts->ntri, tmp.as<uint32_t>());
    LA3G_LAUNCHED();
    LA3G_CUDA(cudaMemcpyAsync(per_vertex_out, tmp.p, (size_t) N * 4, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
  }
  LA3G_TRY(T.finish());
  if (total_out) *total_out = total;
  if (st)
  {
    st->iterations = 2;
    st->teps_edges = g.nent;
    st->edges_examined = g.nent;
    st->algo_bytes = (uint64_t) (8.0 * g.nent + 8.0 * N);
  }
  return LA3G_OK;
}
