// SSSP: the reference sssp app (src/apps/graph_analytics/sssp.cpp:11-37,
// sssp.h:11-46) on the device.
//
// Reference semantics kept exactly (np = 1, the optimizable path
// execute_, vertex_program_execute.hpp:55-163):
//   * dist is uint32 with INF = 2^31 - 1; gather = msg + weight in uint32
//     arithmetic; combine = min; apply = min and activates on change;
//   * iteration i relaxes the out-edges of the vertices activated in
//     iteration i - 1 (the root in iteration 0, if it has out-edges), with
//     the message each of them scattered when it was activated, into the
//     REGULAR rows only;
//   * after convergence the sink rows are computed once from every regular
//     vertex's final distance (activated or not, INF included) and from the
//     root's message if the root is a source (:131-148).
// Push relaxation uses atomicMin on dist: the value a row holds after the
// iteration is min(old, min over messages) exactly as apply computes it,
// and a row is activated iff some relaxation lowered it.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "frontier.cuh"
#include "la3g_internal.h"

namespace la3g {

static constexpr uint32_t kInf = 0x7FFFFFFFu;
static constexpr uint32_t kPullLong = 64;     // pull rows longer than this are cut into tasks
static constexpr uint32_t kPullChunk = 512;   // in-edges per long-row task (one warp)
static constexpr uint32_t kPullLanes = 4;     // lanes per short row in a pull step

// The frontier is two lists: vertices with at most kBigDeg out-edges into
// regular rows (one warp each) and hubs (their edges shared by the grid).
struct SsspScratch
{
  uint32_t* dist = nullptr;
  uint32_t* msg = nullptr;
  uint32_t* stamp = nullptr;
  uint32_t* reg_end = nullptr;   // [nslots] end of each vertex's out-edges into regular rows
  uint32_t* raw = nullptr;       // vertices lowered in the current iteration
  uint32_t* small[2] = {nullptr, nullptr};
  uint32_t* big[2] = {nullptr, nullptr};
  uint32_t* big_task0[2] = {nullptr, nullptr};
  // [0] raw count, [1] next degree sum, [2] next small count, [3] hub slots and tasks (frontier.cuh),
  // [4] scratch
  unsigned long long* ctr = nullptr;
  unsigned long long* hctr = nullptr;
  uint32_t* fmsg = nullptr;       // pull steps: msg of the frontier vertices, INF elsewhere
  uint32_t* long_rows = nullptr;  // regular rows with more than kPullLong in-edges
  uint32_t nlong = 0;
  uint32_t* task_row = nullptr;   // pull tasks over the long rows: kPullChunk in-edges each
  uint32_t* task_begin = nullptr;
  uint32_t ntasks = 0;
  uint64_t task_edges = 0;        // in-edges of the long rows
  uint32_t* ymin = nullptr;       // [nlong] partial minima of the long rows (INF between steps)
  uint64_t reg_in = 0;            // in-edges of the regular rows
  uint32_t max_w = 0;             // largest weight: pull steps need INF + w to stay in uint32
  uint32_t* by_id = nullptr;      // [nslots] distances reordered by id before they leave the device
};

static void sssp_scratch_free(void* p)
{
  SsspScratch* s = (SsspScratch*) p;
  if (s->hctr) cudaFreeHost(s->hctr);
  delete s;
}

__global__ void k_sssp_init(uint32_t N, uint32_t* dist, uint32_t* stamp)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x)
  {
    dist[p] = kInf;
    stamp[p] = 0;
  }
}

__global__ void k_sssp_root(uint32_t rp, int push, uint32_t* dist, uint32_t* msg, uint32_t* list, uint32_t* task0)
{
  dist[rp] = 0;
  msg[rp] = 0;
  if (push) { list[0] = rp; task0[0] = 0; }
}

// End of the regular-row part of every out-edge list (rows ascend, so the
// sinks come last).
__global__ void k_sssp_reg_end(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ row, uint32_t N,
                               uint32_t nreg, uint32_t* reg_end)
{
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < N; u += gridDim.x * blockDim.x)
  {
    uint32_t lo = ptr[u], hi = ptr[u + 1];
    while (lo < hi)
    {
      uint32_t mid = (lo + hi) >> 1;
      if (row[mid] < nreg) lo = mid + 1;
      else hi = mid;
    }
    reg_end[u] = lo;
  }
}

__device__ __forceinline__ void relax(uint32_t v, uint32_t cand, bool valid, uint32_t* dist, uint32_t* stamp,
                                      uint32_t tag, uint32_t* raw, unsigned long long* ctr, int lane)
{
  bool add = false;
  if (valid && cand < dist[v])
  {
    const uint32_t old = atomicMin(&dist[v], cand);
    if (cand < old) add = atomicExch(&stamp[v], tag) != tag;
  }
  const unsigned mask = __ballot_sync(0xffffffffu, add);
  if (mask)
  {
    uint32_t base = 0;
    if (lane == 0) base = (uint32_t) atomicAdd(&ctr[0], (unsigned long long) __popc(mask));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (add) raw[base + __popc(mask & ((1u << lane) - 1))] = v;
  }
}

// Relaxation over a split frontier: hubs first (all warps share each hub's
// edges), then one warp per small vertex.  Messages are the distances the
// frontier vertices held when they were activated (msg), as the reference's
// scatter values are.
__global__ void __launch_bounds__(256)
k_sssp_push(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ reg_end, const uint32_t* __restrict__ row,
            const uint32_t* __restrict__ w, const uint32_t* __restrict__ small, uint32_t nsmall,
            const uint32_t* __restrict__ big, const uint32_t* __restrict__ big_task0, uint32_t nbig, uint32_t ntasks,
            const uint32_t* __restrict__ msg, uint32_t* dist, uint32_t* stamp, uint32_t tag, uint32_t* raw,
            unsigned long long* ctr)
{
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t t = warp; t < ntasks; t += nwarps)
  {
    const uint32_t slot = hub_of_task(big_task0, nbig, t);
    const uint32_t u = big[slot];
    const uint32_t mu = msg[u];
    const uint32_t b = ptr[u] + (t - big_task0[slot]) * kHubTask;
    const uint32_t e = min(b + kHubTask, reg_end[u]);
    for (uint32_t i0 = b; i0 < e; i0 += 32)
    {
      const uint32_t i = i0 + lane;
      const bool ok = i < e;
      relax(ok ? row[i] : 0, ok ? mu + w[i] : 0, ok, dist, stamp, tag, raw, ctr, lane);
    }
  }
  for (uint32_t f = warp; f < nsmall; f += nwarps)
  {
    const uint32_t u = small[f];
    const uint32_t mu = msg[u];
    const uint32_t b = ptr[u], e = reg_end[u];
    for (uint32_t i0 = b; i0 < e; i0 += 32)
    {
      const uint32_t i = i0 + lane;
      const bool ok = i < e;
      relax(ok ? row[i] : 0, ok ? mu + w[i] : 0, ok, dist, stamp, tag, raw, ctr, lane);
    }
  }
}

// Activated vertices scatter their new distance and form the next frontier
// (stamp = this iteration's tag: the pull step finds the frontier by it).
__global__ void k_sssp_apply(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ reg_end,
                             const uint32_t* __restrict__ raw, const uint32_t* __restrict__ dist, uint32_t* msg,
                             uint32_t* stamp, uint32_t tag, uint32_t* small, uint32_t* big, uint32_t* big_task0,
                             unsigned long long* ctr)
{
  unsigned long long deg = 0;
  const uint32_t n = (uint32_t) ctr[0];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
  {
    uint32_t v = raw[i];
    msg[v] = dist[v];
    stamp[v] = tag;
    uint32_t d = reg_end[v] - ptr[v];
    deg += d;
    if (d > kBigDeg) hub_append(v, d, big, big_task0, &ctr[3]);
    else if (d) small[atomicAdd(&ctr[2], 1ull)] = v;
  }
  for (int o = 16; o > 0; o >>= 1) deg += __shfl_xor_sync(0xffffffffu, deg, o);
  if ((threadIdx.x & 31) == 0 && deg) atomicAdd(&ctr[1], deg);
}

// Pull step (for large frontiers; the reference's own SpMV direction):
// every regular row takes the min over its in-neighbours in the frontier
// (the previous iteration's frontier lists) of msg + w, and is activated if
// that lowers it.  fmsg holds msg for the frontier and INF for every other
// vertex, so each edge is one load and one add: INF + w (w <= 2^31) stays
// above INF in uint32 and never lowers a row.  Short rows are owned by one
// lane group and long rows are cut into tasks whose minima meet in ymin,
// so dist needs no atomics; fmsg is not written while the step runs.
// Sources are frontier vertices only in the first iteration, which always
// pushes.
__device__ __forceinline__ void sssp_pull_edge(uint32_t e, const uint32_t* __restrict__ col,
                                               const uint32_t* __restrict__ w, const uint32_t* __restrict__ fmsg,
                                               uint32_t& y)
{
  y = min(y, fmsg[col[e]] + w[e]);
}

// fmsg = msg for the frontier lists' vertices (small list, then hub slots).
__global__ void k_fill_inf(uint32_t n, uint32_t* a)
{
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = kInf;
}

__global__ void k_sssp_fmsg(const uint32_t* __restrict__ small, uint32_t nsmall, const uint32_t* __restrict__ big,
                            uint32_t nbig, const uint32_t* __restrict__ msg, uint32_t* fmsg)
{
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nsmall + nbig; i += gridDim.x * blockDim.x)
  {
    const uint32_t v = i < nsmall ? small[i] : big[i - nsmall];
    fmsg[v] = msg[v];
  }
}

__global__ void __launch_bounds__(256)
k_sssp_pull(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, const uint32_t* __restrict__ w,
            uint32_t nreg, const uint32_t* __restrict__ task_row, const uint32_t* __restrict__ task_begin,
            uint32_t ntasks, uint32_t task_warps, uint32_t* ymin, const uint32_t* __restrict__ fmsg,
            const uint32_t* __restrict__ msg, uint32_t* dist, uint32_t* raw, unsigned long long* ctr)
{
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp < task_warps)
  {
    // long rows: each task's minimum goes to the row's partial slot
    for (uint32_t t = warp; t < ntasks; t += task_warps)
    {
      const uint32_t k = task_row[t];  // index into the long-row list
      const uint32_t b = task_begin[t], e = task_begin[ntasks + t];  // [begins | ends]
      uint32_t y = kInf;
      for (uint32_t i = b + lane; i < e; i += 32) sssp_pull_edge(i, col, w, fmsg, y);
      for (int o = 16; o > 0; o >>= 1) y = min(y, __shfl_xor_sync(0xffffffffu, y, o));
      if (lane == 0 && y < kInf) atomicMin(&ymin[k], y);
    }
    return;
  }
  // short rows: a group of kPullLanes lanes per row; each lane keeps four
  // independent loads in flight per step (indices, then frontier words,
  // then messages), since the step is bound by memory latency
  constexpr uint32_t G = kPullLanes;
  const uint32_t sub = lane & (G - 1);
  const uint32_t group = (((blockIdx.x * blockDim.x + threadIdx.x) >> 5) - task_warps) * (32 / G) + lane / G;
  const uint32_t ngroups = (((gridDim.x * blockDim.x) >> 5) - task_warps) * (32 / G);
  const uint32_t rounds = (nreg + ngroups - 1) / ngroups;
  for (uint32_t k = 0; k < rounds; k++)
  {
    const uint32_t v = group + k * ngroups;
    uint32_t y = kInf;
    bool mine = false;
    if (v < nreg)
    {
      const uint32_t b = ptr[v], e = ptr[v + 1];
      mine = e - b <= kPullLong;
      if (mine)
        for (uint32_t i = b + sub; i < e; i += 4 * G)
        {
          uint32_t c[4], ww[4], m[4];
#pragma unroll
          for (int u = 0; u < 4; u++)
          {
            const bool ok = i + u * G < e;
            c[u] = ok ? col[i + u * G] : 0u;
            ww[u] = ok ? w[i + u * G] : kInf;
          }
#pragma unroll
          for (int u = 0; u < 4; u++) m[u] = fmsg[c[u]];
#pragma unroll
          for (int u = 0; u < 4; u++) y = min(y, m[u] + ww[u]);
        }
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) y = min(y, __shfl_xor_sync(0xffffffffu, y, o));
    const bool low = mine && sub == 0 && y < dist[v];
    if (low) dist[v] = y;
    const unsigned m = __ballot_sync(0xffffffffu, low);
    if (m)
    {
      uint32_t base = 0;
      if (lane == 0) base = (uint32_t) atomicAdd(&ctr[0], (unsigned long long) __popc(m));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (low) raw[base + __popc(m & ((1u << lane) - 1))] = v;
    }
  }
}

// Long rows after a pull step: apply the partial minimum, reset it.
__global__ void k_sssp_pull_long(const uint32_t* __restrict__ long_rows, uint32_t nlong, uint32_t* ymin, uint32_t* dist,
                                 uint32_t* raw, unsigned long long* ctr)
{
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nlong; k += gridDim.x * blockDim.x)
  {
    const uint32_t y = ymin[k];
    if (y == kInf) continue;
    ymin[k] = kInf;
    const uint32_t v = long_rows[k];
    if (y < dist[v])
    {
      dist[v] = y;
      raw[atomicAdd(&ctr[0], 1ull)] = v;
    }
  }
}

__global__ void k_sssp_long_rows(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ w, uint32_t nreg,
                                 uint32_t* list, unsigned long long* n, unsigned long long* edges, unsigned int* maxw)
{
  unsigned long long s = 0;
  unsigned int mw = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nreg; v += gridDim.x * blockDim.x)
  {
    const uint32_t d = ptr[v + 1] - ptr[v];
    s += d;
    for (uint32_t i = ptr[v]; i < ptr[v + 1]; i++) mw = max(mw, w[i]);
    if (d > kPullLong) list[atomicAdd(n, 1ull)] = v;
  }
  for (int o = 16; o > 0; o >>= 1)
  {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    mw = max(mw, __shfl_xor_sync(0xffffffffu, mw, o));
  }
  if ((threadIdx.x & 31) == 0)
  {
    if (s) atomicAdd(edges, s);
    if (mw) atomicMax(maxw, mw);
  }
}

// A step pulls when its frontier's out-degree sum exceeds the regular rows'
// in-edges / kPullDivisor (measured on R-MAT s22: 2 and 4 are best).
static constexpr double kPullDivisor = 4.0;

// Sink pass: y = min over in-neighbours (regular: final dist; the root if it
// is a source: its message 0) of msg + w; dist = min(dist, y).
__global__ void k_sssp_sinks(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col,
                             const uint32_t* __restrict__ w, uint32_t nreg, uint32_t nsink, uint32_t src_root,
                             uint32_t* dist)
{
  for (uint32_t v = nreg + blockIdx.x * blockDim.x + threadIdx.x; v < nreg + nsink; v += gridDim.x * blockDim.x)
  {
    uint32_t y = kInf;
    for (uint32_t i = ptr[v]; i < ptr[v + 1]; i++)
    {
      const uint32_t c = col[i];
      uint32_t cand;
      if (c < nreg) cand = dist[c] + w[i];
      else if (c == src_root) cand = 0u + w[i];
      else continue;
      y = min(y, cand);
    }
    dist[v] = min(dist[v], y);
  }
}

__global__ void k_reached_outdeg(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ dist, uint32_t N,
                                 unsigned long long* out)
{
  unsigned long long s = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x)
    if (dist[v] != kInf) s += ptr[v + 1] - ptr[v];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, s);
}

__global__ void k_u32_by_id(uint32_t N, const uint32_t* __restrict__ id_of_pos, const uint32_t* __restrict__ val,
                            uint32_t* __restrict__ out)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) out[id_of_pos[p]] = val[p];
}

static int sssp_scratch(la3g_graph* G, SsspScratch** out)
{
  SsspScratch* ss = (SsspScratch*) G->slot[kSlotSssp];
  if (ss) { *out = ss; return LA3G_OK; }
  ss = new (std::nothrow) SsspScratch();
  if (!ss) return set_error(LA3G_ENOMEM, "out of host memory");
  G->slot[kSlotSssp] = ss;
  G->slot_free[kSlotSssp] = sssp_scratch_free;
  const uint32_t N = G->g.nslots;
  LA3G_TRY(galloc(G, &ss->dist, N));
  LA3G_TRY(galloc(G, &ss->msg, N));
  LA3G_TRY(galloc(G, &ss->stamp, N));
  LA3G_TRY(galloc(G, &ss->reg_end, N));
  LA3G_TRY(galloc(G, &ss->raw, N));
  LA3G_TRY(galloc(G, &ss->small[0], N));
  LA3G_TRY(galloc(G, &ss->small[1], N));
  LA3G_TRY(galloc(G, &ss->big[0], N));
  LA3G_TRY(galloc(G, &ss->big[1], N));
  LA3G_TRY(galloc(G, &ss->big_task0[0], N));
  LA3G_TRY(galloc(G, &ss->big_task0[1], N));
  LA3G_TRY(galloc(G, &ss->ctr, 8));
  LA3G_TRY(galloc(G, &ss->by_id, N));
  LA3G_CUDA(cudaHostAlloc(&ss->hctr, 8 * sizeof(unsigned long long), cudaHostAllocDefault));
  k_sssp_reg_end<<<grid_for(N, 256), 256, 0, G->stream>>>(G->g.out_ptr, G->g.out_row, N, G->g.nreg, ss->reg_end);
  LA3G_LAUNCHED();
  LA3G_TRY(galloc(G, &ss->long_rows, std::max<uint32_t>(G->g.nreg, 1)));
  LA3G_TRY(galloc(G, &ss->fmsg, N));
  LA3G_CUDA(cudaMemsetAsync(ss->ctr, 0, 8 * sizeof(unsigned long long), G->stream));
  k_sssp_long_rows<<<grid_for(G->g.nreg, 256), 256, 0, G->stream>>>(G->g.in_ptr, G->g.in_w, G->g.nreg, ss->long_rows,
                                                                     ss->ctr, ss->ctr + 1, (unsigned int*) (ss->ctr + 2));
  LA3G_LAUNCHED();
  LA3G_CUDA(cudaMemcpyAsync(ss->hctr, ss->ctr, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, G->stream));
  LA3G_CUDA(cudaStreamSynchronize(G->stream));
  ss->nlong = (uint32_t) ss->hctr[0];
  ss->reg_in = ss->hctr[1];
  ss->max_w = (uint32_t) ss->hctr[2];
  if (ss->nlong)
  {
    // cut the long rows into tasks of kPullChunk in-edges (host side: few rows)
    std::vector<uint32_t> rows(ss->nlong), b(ss->nlong), e(ss->nlong), ptr((size_t) G->g.nreg + 1);
    LA3G_CUDA(cudaMemcpy(rows.data(), ss->long_rows, ss->nlong * 4, cudaMemcpyDeviceToHost));
    LA3G_CUDA(cudaMemcpy(ptr.data(), G->g.in_ptr, ptr.size() * 4, cudaMemcpyDeviceToHost));
    for (uint32_t k = 0; k < ss->nlong; k++)
    {
      b[k] = ptr[rows[k]];
      e[k] = ptr[rows[k] + 1];
    }
    std::vector<uint32_t> trow, tbeg;
    for (uint32_t k = 0; k < ss->nlong; k++)
    {
      ss->task_edges += e[k] - b[k];
      for (uint32_t x = b[k]; x < e[k]; x += kPullChunk)
      {
        trow.push_back(k);
        tbeg.push_back(x);
      }
    }
    ss->ntasks = (uint32_t) trow.size();
    LA3G_TRY(galloc(G, &ss->task_row, trow.size()));
    LA3G_TRY(galloc(G, &ss->task_begin, 2 * trow.size()));  // [begins | ends]
    LA3G_TRY(galloc(G, &ss->ymin, ss->nlong));
    std::vector<uint32_t> be(2 * trow.size());
    for (size_t t = 0; t < trow.size(); t++)
    {
      be[t] = tbeg[t];
      be[trow.size() + t] = std::min<uint32_t>(tbeg[t] + kPullChunk, e[trow[t]]);
    }
    LA3G_CUDA(cudaMemcpy(ss->task_row, trow.data(), trow.size() * 4, cudaMemcpyHostToDevice));
    LA3G_CUDA(cudaMemcpy(ss->task_begin, be.data(), be.size() * 4, cudaMemcpyHostToDevice));
    std::vector<uint32_t> inf(ss->nlong, kInf);
    LA3G_CUDA(cudaMemcpy(ss->ymin, inf.data(), ss->nlong * 4, cudaMemcpyHostToDevice));
  }
  *out = ss;
  return LA3G_OK;
}

static int sssp_run(la3g_graph* G, SsspScratch* ss, uint32_t root, la3g_stats* st)
{
  DevGraph& g = G->g;
  cudaStream_t s = G->stream;
  const uint32_t N = g.nslots;
  k_sssp_init<<<grid_for(N, 256), 256, 0, s>>>(N, ss->dist, ss->stamp);
  LA3G_LAUNCHED();
  tls_launches++;
  uint32_t rp = 0xFFFFFFFFu, src_root = 0xFFFFFFFFu;
  uint64_t nsmall = 0, nbig = 0, ntasks = 0, front_deg = 0;
  if (root < N)
  {
    LA3G_CUDA(cudaMemcpyAsync(&rp, g.pos_of_id + root, 4, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    // init returns true for the root; regular and source vertices scatter.
    const bool scat = rp < g.nreg || (rp >= g.src_base() && rp < g.iso_base());
    if (rp >= g.src_base() && rp < g.iso_base()) src_root = rp;
    uint32_t re = 0, hp[2] = {0, 0};
    if (scat)
    {
      LA3G_CUDA(cudaMemcpyAsync(hp, g.out_ptr + rp, 8, cudaMemcpyDeviceToHost, s));
      LA3G_CUDA(cudaMemcpyAsync(&re, ss->reg_end + rp, 4, cudaMemcpyDeviceToHost, s));
      LA3G_CUDA(cudaStreamSynchronize(s));
      front_deg = re - hp[0];
    }
    const bool hub = front_deg > kBigDeg;
    k_sssp_root<<<1, 1, 0, s>>>(rp, scat ? 1 : 0, ss->dist, ss->msg, hub ? ss->big[0] : ss->small[0],
                                ss->big_task0[0]);
    LA3G_LAUNCHED();
    tls_launches++;
    if (scat) (hub ? nbig : nsmall) = 1;
    if (scat && hub) ntasks = (front_deg + kHubTask - 1) / kHubTask;
  }
  uint32_t iter = 0;
  int cur = 0;
  uint64_t examined = 0;
  const unsigned blocks = num_sms() * 8;
  for (;;)
  {
    if (iter > 1000000) return set_error(LA3G_ETIMEOUT, "sssp did not converge");
    iter++;
    if (nsmall + nbig == 0) break;
    LA3G_CUDA(cudaMemsetAsync(ss->ctr, 0, 4 * sizeof(unsigned long long), s));
    if (iter > 1 && ss->max_w <= 0x80000000u && (double) front_deg * kPullDivisor > (double) ss->reg_in)
    {
      // in-edges of every regular row (index + weight), stamps and
      // messages of their columns, one dist read per row
      ProfileScope p("sssp_pull", s, 8.0 * ss->reg_in + 8.0 * ss->reg_in + 8.0 * g.nreg);
      // warps split between long-row tasks and short rows in proportion to their in-edges
      const uint32_t all_warps = num_sms() * 8 * 8;
      const uint32_t task_warps =
          ss->ntasks ? std::min<uint32_t>(ss->ntasks, std::max<uint32_t>(1, (uint32_t) ((double) all_warps *
                                                                                          ss->task_edges /
                                                                                          std::max<uint64_t>(ss->reg_in, 1))))
                     : 0;
      k_fill_inf<<<grid_for(N, 256), 256, 0, s>>>(N, ss->fmsg);
      LA3G_LAUNCHED();
      k_sssp_fmsg<<<grid_for(nsmall + nbig, 256), 256, 0, s>>>(ss->small[cur], (uint32_t) nsmall, ss->big[cur],
                                                               (uint32_t) nbig, ss->msg, ss->fmsg);
      LA3G_LAUNCHED();
      tls_launches += 2;
      k_sssp_pull<<<num_sms() * 8, 256, 0, s>>>(g.in_ptr, g.in_col, g.in_w, g.nreg, ss->task_row, ss->task_begin,
                                            ss->ntasks, task_warps, ss->ymin, ss->fmsg, ss->msg, ss->dist, ss->raw,
                                            ss->ctr);
      LA3G_LAUNCHED();
      tls_launches++;
      if (ss->nlong)
      {
        k_sssp_pull_long<<<grid_for(ss->nlong, 256), 256, 0, s>>>(ss->long_rows, ss->nlong, ss->ymin, ss->dist,
                                                                  ss->raw, ss->ctr);
        LA3G_LAUNCHED();
        tls_launches++;
      }
      examined += ss->reg_in;
    }
    else
    {
      ProfileScope p("sssp_push", s, 8.0 * front_deg + 12.0 * (nsmall + nbig));
      k_sssp_push<<<blocks, 256, 0, s>>>(g.out_ptr, ss->reg_end, g.out_row, g.out_w, ss->small[cur], (uint32_t) nsmall,
                                         ss->big[cur], ss->big_task0[cur], (uint32_t) nbig, (uint32_t) ntasks, ss->msg,
                                         ss->dist, ss->stamp, iter, ss->raw, ss->ctr);
      LA3G_LAUNCHED();
      examined += front_deg;
    }
    k_sssp_apply<<<num_sms() * 4, 256, 0, s>>>(g.out_ptr, ss->reg_end, ss->raw, ss->dist, ss->msg, ss->stamp, iter,
                                         ss->small[cur ^ 1], ss->big[cur ^ 1], ss->big_task0[cur ^ 1], ss->ctr);
    LA3G_LAUNCHED();
    tls_launches++;
    LA3G_CUDA(cudaMemcpyAsync(ss->hctr, ss->ctr, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    const uint64_t nn = ss->hctr[0];
    nsmall = ss->hctr[2];
    nbig = ss->hctr[3] >> kHubSlotShift;
    ntasks = ss->hctr[3] & ((1ull << kHubSlotShift) - 1);
    front_deg = ss->hctr[1];
    cur ^= 1;
    // A vertex lowered only into sink-free regular rows with no regular
    // out-edges is activated but has nothing to relax; the loop still runs
    // the next iteration only if something was activated.
    if (nn == 0) break;
    if (nsmall + nbig == 0)
    {
      iter++;  // the next iteration runs with messages that reach no regular row
      break;
    }
  }
  if (g.nsink)
  {
    // the sink rows' in-edges only (index + weight, and the column's
    // distance), their offsets and the distance read and written
    const double sink_in = (double) (g.nent - ss->reg_in);
    ProfileScope p("sssp_sinks", s, 12.0 * sink_in + 12.0 * g.nsink);
    k_sssp_sinks<<<grid_for(g.nsink, 256), 256, 0, s>>>(g.in_ptr, g.in_col, g.in_w, g.nreg, g.nsink, src_root, ss->dist);
    LA3G_LAUNCHED();
  }
  if (st)
  {
    st->iterations = iter;
    st->edges_examined = examined;
  }
  return LA3G_OK;
}

}  // namespace la3g

using namespace la3g;

extern "C" int la3g_sssp(la3g_graph* G, uint32_t root, uint32_t* dist_out, la3g_stats* st)
{
  if (!G) return set_error(LA3G_EINVAL, "null graph");
  DevGraph& g = G->g;
  if (!g.directed() || !g.weighted() || (g.flags & (LA3G_REVERSE | LA3G_ACYCLIC | LA3G_BIPARTITE)))
    return set_error(LA3G_EINVAL, "sssp needs a graph loaded with LA3G_DIRECTED | LA3G_WEIGHTED");
  CallTimer T(G, st);
  LA3G_TRY(build_push_csr(G));
  SsspScratch* ss = nullptr;
  LA3G_TRY(sssp_scratch(G, &ss));
  cudaStream_t s = G->stream;
  const uint32_t N = g.nslots;
  T.device_begin();
  LA3G_TRY(sssp_run(G, ss, root, st));
  T.device_end();
  if (st)
  {
    LA3G_CUDA(cudaMemsetAsync(ss->ctr + 2, 0, 8, s));
    k_reached_outdeg<<<grid_for(N, 256), 256, 0, s>>>(g.out_ptr, ss->dist, N, ss->ctr + 2);
    LA3G_LAUNCHED();
    LA3G_CUDA(cudaMemcpyAsync(ss->hctr + 2, ss->ctr + 2, 8, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    st->teps_edges = ss->hctr[2];
    st->algo_bytes = st->edges_examined * 8 + (uint64_t) N * 8;
  }
  if (dist_out)
  {
    // the graph's own reorder buffer: no allocation per call
    k_u32_by_id<<<grid_for(N, 256), 256, 0, s>>>(N, g.id_of_pos, ss->dist, ss->by_id);
    LA3G_LAUNCHED();
    LA3G_CUDA(cudaMemcpyAsync(dist_out, ss->by_id, (size_t) N * 4, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
  }
  return T.finish();
}
