// Connected components: the reference cc app (src/apps/graph_analytics/
// cc.cpp:11-31, cc.h:11-38) on the device.
//
// The reference propagates labels (initially the vertex's own id) with
// combine y2 = (y2 == 0) ? y1 : min(y1, y2) until nothing changes.  When
// vertex 0 has no edges no label is ever 0, combine is a plain min, and
// the fixed point is: every vertex with edges carries the least id of its
// component, every isolated vertex its own id.  That fixed point is computed
// here with a lock-free union-find whose roots are always the least id of
// their set (a root is only ever hooked under a root with a smaller id),
// followed by full path compression.  Edges are processed Afforest-style
// (Sutton et al.): each vertex first unites with two neighbours, the giant
// component is found by sampling, and only vertices outside it then walk
// their remaining edges.
//
// When vertex 0 does have edges, label 0 behaves as "no value yet" and the
// outcome depends on the order messages arrive in, so that case runs the
// reference's BSP iterations literally: each row folds the messages of its
// active in-neighbours in ascending column order with the reference's
// combine.
#include <algorithm>
#include <cstring>
#include <vector>

#include "la3g_internal.h"

namespace la3g {

struct CcScratch
{
  uint32_t* label = nullptr;   // by original id (union-find parents)
  uint32_t* probe = nullptr;   // roots of sampled vertices
  uint32_t* lab_pos = nullptr; // BSP path: labels by position
  uint32_t* msg = nullptr;
  uint8_t* active[2] = {nullptr, nullptr};
  int* flag = nullptr;
  unsigned long long* walked = nullptr;  // [0] rows, [1] edges k_cc_rest walked
  unsigned long long* hwalked = nullptr; // pinned mirror
  uint32_t* giant = nullptr;   // the sampled giant component's root
  int zero_has_edges = -1;     // whether vertex 0 has edges (-1: not looked up yet)
};

static void cc_scratch_free(void* p)
{
  CcScratch* s = (CcScratch*) p;
  if (s->hwalked) cudaFreeHost(s->hwalked);
  delete s;
}

__global__ void k_cc_init(uint32_t N, uint32_t* parent)
{
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x) parent[v] = v;
}

__device__ __forceinline__ uint32_t cc_find(uint32_t* parent, uint32_t v)
{
  // path halving; concurrent halving writes only ever point further up
  uint32_t p = parent[v];
  while (p != v)
  {
    uint32_t gp = parent[p];
    if (gp != p) parent[v] = gp;
    v = p;
    p = gp;
  }
  return v;
}

__device__ __forceinline__ void cc_union(uint32_t* parent, uint32_t a, uint32_t b)
{
  uint32_t ru = cc_find(parent, a), rv = cc_find(parent, b);
  while (ru != rv)
  {
    if (ru > rv) { uint32_t t = ru; ru = rv; rv = t; }
    // hook the larger root under the smaller one
    uint32_t old = atomicCAS(&parent[rv], rv, ru);
    if (old == rv) break;
    rv = cc_find(parent, old);
    ru = cc_find(parent, ru);
  }
}

// Afforest-style sampling round r: every row unites with its r-th
// neighbour (rounds are separated by a full path compression, which keeps
// the finds of the next round short).
__global__ void k_cc_sample(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col,
                            const uint32_t* __restrict__ id_of_pos, uint32_t nrows, uint32_t r, uint32_t* parent)
{
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < nrows; u += gridDim.x * blockDim.x)
  {
    const uint32_t i = ptr[u] + r;
    if (i < ptr[u + 1]) cc_union(parent, id_of_pos[u], id_of_pos[col[i]]);
  }
}

// Remaining edges (from the k-th neighbour on) of the rows whose root is not
// the sampled giant root; the graph is symmetric, so every edge that leaves
// the giant component is seen from its other endpoint.  One warp per row.
__global__ void __launch_bounds__(256)
k_cc_rest(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, const uint32_t* __restrict__ id_of_pos,
          uint32_t nrows, uint32_t k, const uint32_t* __restrict__ giant_ptr, uint32_t* parent,
          unsigned long long* walked)
{
  const uint32_t giant = *giant_ptr;
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  unsigned long long rows = 0, edges = 0;
  for (uint32_t u = warp; u < nrows; u += nwarps)
  {
    const uint32_t b = ptr[u] + k, e = ptr[u + 1];
    if (b >= e) continue;
    const uint32_t iu = id_of_pos[u];
    if (cc_find(parent, iu) == giant) continue;
    rows++;
    edges += e - b;
    for (uint32_t i = b + lane; i < e; i += 32) cc_union(parent, iu, id_of_pos[col[i]]);
  }
  if (lane == 0 && rows)
  {
    atomicAdd(&walked[0], rows);
    atomicAdd(&walked[1], edges);
  }
}

__global__ void k_cc_probe(const uint32_t* __restrict__ id_of_pos, uint32_t nrows, uint32_t nsamples, uint64_t seed,
                           uint32_t* parent, uint32_t* out)
{
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nsamples; i += gridDim.x * blockDim.x)
  {
    uint64_t x = seed + 0x9E3779B97F4A7C15ull * (i + 1);
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    out[i] = cc_find(parent, id_of_pos[(uint32_t) (x % nrows)]);
  }
}

// The most frequent root among the samples (ties: the smallest), on the
// device: one block sorts them in shared memory and counts runs.
template <uint32_t NS>
__global__ void __launch_bounds__(NS) k_cc_giant(const uint32_t* __restrict__ probe, uint32_t* giant)
{
  __shared__ uint32_t v[NS];
  __shared__ uint32_t best_len, best_val;
  const uint32_t t = threadIdx.x;
  v[t] = probe[t];
  if (t == 0)
  {
    best_len = 0;
    best_val = 0xFFFFFFFFu;
  }
  __syncthreads();
  for (uint32_t size = 2; size <= NS; size <<= 1)
    for (uint32_t stride = size >> 1; stride > 0; stride >>= 1)
    {
      const uint32_t j = t ^ stride;
      if (j > t)
      {
        const bool up = (t & size) == 0;
        const uint32_t a = v[t], b = v[j];
        if ((a > b) == up)
        {
          v[t] = b;
          v[j] = a;
        }
      }
      __syncthreads();
    }
  // run starts: thread t owns the run beginning at t
  if (t == 0 || v[t] != v[t - 1])
  {
    uint32_t e = t + 1;
    while (e < NS && v[e] == v[t]) e++;
    const uint32_t len = e - t;
    // longest run, the smallest root among equal lengths: pack (len, ~val) into one word
    atomicMax(&best_len, len);
  }
  __syncthreads();
  if ((t == 0 || v[t] != v[t - 1]))
  {
    uint32_t e = t + 1;
    while (e < NS && v[e] == v[t]) e++;
    if (e - t == best_len) atomicMin(&best_val, v[t]);
  }
  __syncthreads();
  if (t == 0) *giant = best_val;
}

__global__ void k_cc_flatten(uint32_t N, uint32_t* parent)
{
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x)
  {
    uint32_t r = v;
    while (parent[r] != r) r = parent[r];
    parent[v] = r;
  }
}

// ---- literal BSP path (vertex 0 has edges) ---------------------------------

__global__ void k_ccb_init(uint32_t N, uint32_t nrows, const uint32_t* __restrict__ id_of_pos, uint32_t* lab,
                           uint32_t* msg, uint8_t* act)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x)
  {
    lab[p] = id_of_pos[p];  // init: label = vid, returns true (cc.h:28)
    msg[p] = id_of_pos[p];
    act[p] = p < nrows;     // regular vertices scatter
  }
}

// One thread per row: fold active in-neighbours in column order.
__global__ void k_ccb_step(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, uint32_t nrows,
                           const uint8_t* __restrict__ act, uint8_t* next_act, const uint32_t* __restrict__ msg,
                           uint32_t* lab, uint32_t* next_msg, int* flag)
{
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x)
  {
    uint32_t y = 0;
    bool touched = false;
    for (uint32_t i = ptr[r]; i < ptr[r + 1]; i++)
    {
      uint32_t c = col[i];
      if (!act[c]) continue;
      uint32_t m = msg[c];
      y = (y == 0) ? m : min(m, y);
      touched = true;
    }
    bool activated = false;
    if (touched)
    {
      uint32_t f = 0;
      f = (f == 0) ? y : min(y, f);  // combine(partial, A())
      uint32_t old = lab[r];
      uint32_t nl = min(old, f);
      lab[r] = nl;
      activated = nl != old;
    }
    next_act[r] = activated;
    if (activated) { next_msg[r] = lab[r]; *flag = 1; }
  }
}

__global__ void k_ccb_by_id(uint32_t N, const uint32_t* __restrict__ id_of_pos, const uint32_t* __restrict__ lab,
                            uint32_t* out)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) out[id_of_pos[p]] = lab[p];
}

static int cc_scratch(la3g_graph* G, CcScratch** out)
{
  CcScratch* cs = (CcScratch*) G->slot[kSlotCc];
  if (cs) { *out = cs; return LA3G_OK; }
  cs = new (std::nothrow) CcScratch();
  if (!cs) return set_error(LA3G_ENOMEM, "out of host memory");
  G->slot[kSlotCc] = cs;
  G->slot_free[kSlotCc] = cc_scratch_free;
  LA3G_TRY(galloc(G, &cs->label, G->g.nslots));
  LA3G_TRY(galloc(G, &cs->flag, 1));
  LA3G_TRY(galloc(G, &cs->walked, 2));
  LA3G_CUDA(cudaHostAlloc(&cs->hwalked, 2 * sizeof(unsigned long long), cudaHostAllocDefault));
  *out = cs;
  return LA3G_OK;
}

}  // namespace la3g

using namespace la3g;

extern "C" int la3g_cc(la3g_graph* G, uint32_t* label_out, la3g_stats* st)
{
  if (!G) return set_error(LA3G_EINVAL, "null graph");
  DevGraph& g = G->g;
  if (g.directed()) return set_error(LA3G_EINVAL, "cc needs an undirected graph (load without LA3G_DIRECTED)");
  CallTimer T(G, st);
  CcScratch* cs = nullptr;
  LA3G_TRY(cc_scratch(G, &cs));
  cudaStream_t s = G->stream;
  const uint32_t N = g.nslots, nrows = g.nrows();
  if (cs->zero_has_edges < 0)
  {
    uint32_t p0 = 0;  // a property of the graph: looked up once
    LA3G_CUDA(cudaMemcpyAsync(&p0, g.pos_of_id, 4, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    cs->zero_has_edges = p0 < nrows ? 1 : 0;
  }
  const bool zero_has_edges = cs->zero_has_edges == 1;
  uint32_t iters = 0;
  bool rest_counted = false;
  T.device_begin();
  if (!zero_has_edges && nrows)
  {
    const uint32_t k = 2, nsamples = 1024;
    k_cc_init<<<grid_for(N, 256), 256, 0, s>>>(N, cs->label);
    LA3G_LAUNCHED();
    tls_launches++;
    for (uint32_t r = 0; r < k; r++)
    {
      {
        // row offsets, one index, two ids, and the two finds' parents
        ProfileScope p("cc_sample", s, 8.0 * nrows + 4.0 * nrows + 8.0 * nrows + 8.0 * nrows);
        k_cc_sample<<<grid_for(nrows, 256), 256, 0, s>>>(g.in_ptr, g.in_col, g.id_of_pos, nrows, r, cs->label);
        LA3G_LAUNCHED();
      }
      {
        ProfileScope p("cc_flatten", s, 8.0 * N);
        k_cc_flatten<<<grid_for(N, 256), 256, 0, s>>>(N, cs->label);
        LA3G_LAUNCHED();
      }
    }
    if (!cs->probe) LA3G_TRY(galloc(G, &cs->probe, nsamples));
    k_cc_probe<<<4, 256, 0, s>>>(g.id_of_pos, nrows, nsamples, 0x5A3Dull, cs->label, cs->probe);
    LA3G_LAUNCHED();
    tls_launches++;
    if (!cs->giant) LA3G_TRY(galloc(G, &cs->giant, 1));
    k_cc_giant<1024><<<1, 1024, 0, s>>>(cs->probe, cs->giant);
    LA3G_LAUNCHED();
    tls_launches++;
    LA3G_CUDA(cudaMemsetAsync(cs->walked, 0, 16, s));
    {
      // every row: its offsets, id and root (16 B); the walked rows' edges:
      // index, neighbour id and its root (12 B each), added once the walked
      // counts are back on the host
      ProfileScope p("cc_rest", s, 16.0 * nrows);
      k_cc_rest<<<grid_for((uint64_t) nrows * 32, 256, num_sms() * 32), 256, 0, s>>>(g.in_ptr, g.in_col, g.id_of_pos, nrows,
                                                                               k, cs->giant, cs->label, cs->walked);
      LA3G_LAUNCHED();
    }
    LA3G_CUDA(cudaMemcpyAsync(cs->hwalked, cs->walked, 16, cudaMemcpyDeviceToHost, s));
    rest_counted = true;
    {
      ProfileScope p("cc_flatten", s, 8.0 * N);
      k_cc_flatten<<<grid_for(N, 256), 256, 0, s>>>(N, cs->label);
      LA3G_LAUNCHED();
    }
    iters = 1;
  }
  else if (!zero_has_edges)
  {
    k_cc_init<<<grid_for(N, 256), 256, 0, s>>>(N, cs->label);
    LA3G_LAUNCHED();
    tls_launches++;
    iters = 1;
  }
  else
  {
    if (!cs->lab_pos)
    {
      LA3G_TRY(galloc(G, &cs->lab_pos, N));
      LA3G_TRY(galloc(G, &cs->msg, 2 * (size_t) N));
      LA3G_TRY(galloc(G, &cs->active[0], N));
      LA3G_TRY(galloc(G, &cs->active[1], N));
    }
    uint32_t* msg[2] = {cs->msg, cs->msg + N};
    k_ccb_init<<<grid_for(N, 256), 256, 0, s>>>(N, nrows, g.id_of_pos, cs->lab_pos, msg[0], cs->active[0]);
    LA3G_LAUNCHED();
    int cur = 0;
    for (;;)
    {
      if (iters > 10000000) return set_error(LA3G_ETIMEOUT, "cc did not converge");
      LA3G_CUDA(cudaMemsetAsync(cs->flag, 0, 4, s));
      {
        ProfileScope p("cc_bsp_step", s, 4.0 * g.nent);
        k_ccb_step<<<grid_for(nrows, 256), 256, 0, s>>>(g.in_ptr, g.in_col, nrows, cs->active[cur], cs->active[cur ^ 1],
                                                        msg[cur], cs->lab_pos, msg[cur ^ 1], cs->flag);
        LA3G_LAUNCHED();
      }
      iters++;
      int f = 0;
      LA3G_CUDA(cudaMemcpyAsync(&f, cs->flag, 4, cudaMemcpyDeviceToHost, s));
      LA3G_CUDA(cudaStreamSynchronize(s));
      cur ^= 1;
      if (!f) break;
    }
    k_ccb_by_id<<<grid_for(N, 256), 256, 0, s>>>(N, g.id_of_pos, cs->lab_pos, cs->label);
    LA3G_LAUNCHED();
  }
  T.device_end();
  if (st)
  {
    st->iterations = iters;
    st->teps_edges = g.nent;
    st->edges_examined = g.nent;
    st->algo_bytes = (uint64_t) (4.0 * g.nent + 12.0 * N);
  }
  if (label_out) LA3G_CUDA(cudaMemcpyAsync(label_out, cs->label, (size_t) N * 4, cudaMemcpyDeviceToHost, s));
  LA3G_TRY(T.finish());
  if (rest_counted)
  {
    profile_add_bytes("cc_rest", 12.0 * (double) cs->hwalked[1]);
    if (st)
    {
      // two sampled neighbours per row (28 B), three compressions (8 B per
      // vertex each), every row's root test (16 B), the walked edges (12 B)
      st->edges_examined = 2ull * nrows + cs->hwalked[1];
      st->algo_bytes = (uint64_t) (56.0 * nrows + 24.0 * N + 16.0 * nrows + 12.0 * (double) cs->hwalked[1]);
    }
  }
  return LA3G_OK;
}
