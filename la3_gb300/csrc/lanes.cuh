// Kernels shared by the batched SSSP (la3g_sssp_batch) and the serving
// loop's SSSP lanes: distances are kept [vertex][root] (uint32, INF =
// 2^31 - 1) with one frontier bit per (vertex, root) packed 64 roots to a
// word; an iteration relaxes the out-edges of every active (vertex, word)
// pair.  Everything here has internal linkage so that each translation unit
// that includes it gets its own copy.
#ifndef LA3G_LANES_CUH
#define LA3G_LANES_CUH

#include <cstdint>
#include <cstdlib>

#include <algorithm>
#include <vector>

#include "frontier.cuh"
#include "la3g_internal.h"

namespace la3g {

static constexpr uint32_t kInfD = 0x7FFFFFFFu;

// Active (vertex, word) pairs of the batched SSSP are kept as a split
// frontier: pairs whose vertex has at most kBigDeg regular out-edges are
// listed for one warp each; the edges of bigger ones are cut into tasks of
// kHubTask edges that warps take one at a time.
struct PairList
{
  uint32_t* small;
  uint32_t* hub;
  uint32_t* hub_t0;
  unsigned long long* nsmall;
  unsigned long long* packed;
};

static __device__ __forceinline__ void bs_list_pair(uint32_t i, uint32_t deg, const PairList& L)
{
  if (deg <= kBigDeg) L.small[atomicAdd(L.nsmall, 1ull)] = i;
  else hub_append(i, deg, L.hub, L.hub_t0, L.packed);
}

// Relaxes edges [k0, k1) of the vertex of pair i: lane l handles roots
// 64w + l and 64w + l + 32, so the distances of one edge's target are read
// contiguously; the roots an edge improved are ORed into the target's
// next-frontier word at once.
static __device__ __forceinline__ void bs_relax_range(uint32_t i, uint32_t k0, uint32_t k1, int lane, uint32_t R, uint32_t W,
                                               const uint32_t* __restrict__ row, const uint32_t* __restrict__ wgt,
                                               const uint64_t* __restrict__ front, uint64_t* next,
                                               const uint32_t* __restrict__ msg, uint32_t* dist)
{
  const uint32_t u = i / W, w = i % W;
  const uint64_t f = front[i];
  const uint32_t r0 = w * 64 + lane, r1 = r0 + 32;
  const bool h0 = (f >> lane) & 1ull, h1 = (f >> (lane + 32)) & 1ull;
  const uint32_t m0 = h0 ? msg[(uint64_t) u * R + r0] : 0, m1 = h1 ? msg[(uint64_t) u * R + r1] : 0;
  for (uint32_t k = k0; k < k1; k++)
  {
    const uint32_t v = row[k], wt = wgt[k];
    bool i0 = false, i1 = false;
    if (h0)
    {
      const uint32_t cand = m0 + wt;
      uint32_t* p = &dist[(uint64_t) v * R + r0];
      i0 = cand < *p && cand < atomicMin(p, cand);
    }
    if (h1)
    {
      const uint32_t cand = m1 + wt;
      uint32_t* p = &dist[(uint64_t) v * R + r1];
      i1 = cand < *p && cand < atomicMin(p, cand);
    }
    const uint64_t mask = (uint64_t) __ballot_sync(0xffffffffu, i0) | ((uint64_t) __ballot_sync(0xffffffffu, i1) << 32);
    if (lane == 0 && mask) atomicOr((unsigned long long*) &next[(uint64_t) v * W + w], (unsigned long long) mask);
  }
}

static __global__ void __launch_bounds__(256)
k_bs_relax(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ reg_end, const uint32_t* __restrict__ row,
           const uint32_t* __restrict__ wgt, uint32_t R, uint32_t W, const uint64_t* __restrict__ front, PairList L,
           uint64_t* next, const uint32_t* __restrict__ msg, uint32_t* dist)
{
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t ns = (uint32_t) *L.nsmall;
  const unsigned long long pk = *L.packed;
  const uint32_t nbig = hub_count(pk), ntasks = hub_tasks(pk);
  for (uint32_t a = warp; a < ntasks + ns; a += nwarps)
  {
    if (a < ntasks)
    {
      const uint32_t slot = hub_of_task(L.hub_t0, nbig, a);
      const uint32_t i = L.hub[slot], u = i / W;
      const uint32_t k0 = ptr[u] + (a - L.hub_t0[slot]) * kHubTask;
      bs_relax_range(i, k0, min(k0 + kHubTask, reg_end[u]), lane, R, W, row, wgt, front, next, msg, dist);
    }
    else
    {
      const uint32_t i = L.small[a - ntasks], u = i / W;
      bs_relax_range(i, ptr[u], reg_end[u], lane, R, W, row, wgt, front, next, msg, dist);
    }
  }
}

// After a relaxation: the old frontier words are cleared (they become the
// next "next" buffer); messages = current distances of the newly lowered
// roots; the words holding them form the next active list.  alive (W words,
// optional) collects the roots that still have a frontier.
static __global__ void k_bs_apply(uint32_t N, uint32_t R, uint32_t W, const uint32_t* __restrict__ ptr,
                                  const uint32_t* __restrict__ reg_end, const uint64_t* __restrict__ next,
                                  const uint32_t* __restrict__ dist, uint32_t* msg, PairList out, uint64_t* front_old,
                                  PairList old, uint64_t* alive = nullptr, unsigned long long* degsum = nullptr)
{
  unsigned long long dsum = 0;
  const uint64_t tid = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x, nth = (uint64_t) gridDim.x * blockDim.x;
  const uint64_t ns = *old.nsmall, nb = hub_count(*old.packed);
  for (uint64_t k = tid; k < ns; k += nth) front_old[old.small[k]] = 0;
  for (uint64_t k = tid; k < nb; k += nth) front_old[old.hub[k]] = 0;
  const uint64_t NW = (uint64_t) N * W;
  for (uint64_t i = tid; i < NW; i += nth)
  {
    uint64_t f = next[i];
    if (!f) continue;
    const uint32_t v = (uint32_t) (i / W), w = (uint32_t) (i % W);
    const uint32_t deg = reg_end[v] - ptr[v];
    bs_list_pair((uint32_t) i, deg, out);
    dsum += deg;
    if (alive && (alive[w] & f) != f) atomicOr((unsigned long long*) &alive[w], (unsigned long long) f);
    while (f)
    {
      const int bpos = __ffsll((long long) f) - 1;
      f &= f - 1;
      const uint64_t j = (uint64_t) v * R + w * 64 + bpos;
      msg[j] = dist[j];
    }
  }
  if (degsum)
  {
    for (int o = 16; o > 0; o >>= 1) dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
    if ((threadIdx.x & 31) == 0 && dsum) atomicAdd(degsum, dsum);
  }
}

// Pull step over (regular vertex, word) pairs, for large frontiers: one warp
// per pair, lane l holding roots 64w + l and 64w + l + 32.  For each
// in-edge (u, v) whose frontier word has bits, every lane whose root is in
// u's frontier takes msg(u) + weight; the pair's new bits (roots lowered)
// are written to next directly (each pair has one writer), so no atomics are
// needed.  Edges go 8 at a time (indices, weights and frontier words loaded
// by 8 lanes and broadcast), so each lane has up to 16 independent message
// loads in flight.  The result per (vertex, root) is the min over the same
// messages a push step relaxes, so both directions give the same iteration.
static constexpr uint32_t kLanePullLong = 4096;  // in-edges per long-row task of a lane pull step

// min over 8 in-edges [e0, e0 + 8) of one (vertex, word) pair, into y0 / y1
static __device__ __forceinline__ void bs_pull8(uint32_t e0, uint32_t e, int lane, uint32_t w, uint32_t R, uint32_t W,
                                                uint32_t r0, uint32_t r1, const uint32_t* __restrict__ col,
                                                const uint32_t* __restrict__ wgt, const uint64_t* __restrict__ front,
                                                const uint32_t* __restrict__ msg, uint32_t& y0, uint32_t& y1)
{
  uint32_t u = 0, wt = 0;
  uint64_t f = 0;
  if (lane < 8 && e0 + lane < e)
  {
    u = col[e0 + lane];
    wt = wgt[e0 + lane];
    f = front[(uint64_t) u * W + w];
  }
  uint32_t m0[8], m1[8], ww[8];
  bool h0[8], h1[8];
#pragma unroll
  for (int j = 0; j < 8; j++)
  {
    const uint64_t fj = __shfl_sync(0xffffffffu, f, j);
    const uint32_t uj = __shfl_sync(0xffffffffu, u, j);
    ww[j] = __shfl_sync(0xffffffffu, wt, j);
    h0[j] = (fj >> lane) & 1ull;
    h1[j] = (fj >> (lane + 32)) & 1ull;
    m0[j] = h0[j] ? msg[(uint64_t) uj * R + r0] : 0u;
    m1[j] = h1[j] ? msg[(uint64_t) uj * R + r1] : 0u;
  }
#pragma unroll
  for (int j = 0; j < 8; j++)
  {
    if (h0[j]) y0 = min(y0, m0[j] + ww[j]);
    if (h1[j]) y1 = min(y1, m1[j] + ww[j]);
  }
}

// Pull step over (regular vertex, word) pairs, for large frontiers: one warp
// per pair, lane l holding roots 64w + l and 64w + l + 32.  For each
// in-edge (u, v) whose frontier word has bits, every lane whose root is in
// u's frontier takes msg(u) + weight.  Edges go 8 at a time (indices,
// weights and frontier words loaded by 8 lanes and broadcast), so each lane
// has up to 16 independent message loads in flight.  Rows with more than
// kLanePullLong in-edges are cut into tasks (task_row / task_b / task_e)
// taken by the first task_warps warps, which meet through atomicMin on dist
// and atomicOr on next; every other pair has one writer and stores its new
// bits directly.  The result per (vertex, root) is the min over the same
// messages a push step relaxes, so both directions give the same iteration.
// next must be all zero on entry (the apply step leaves it so).
static __global__ void __launch_bounds__(256)
k_bs_pull(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, const uint32_t* __restrict__ wgt,
          uint32_t nreg, uint32_t R, uint32_t W, const uint64_t* __restrict__ front, uint64_t* next,
          const uint32_t* __restrict__ msg, uint32_t* dist, const uint32_t* __restrict__ task_row,
          const uint32_t* __restrict__ task_b, const uint32_t* __restrict__ task_e, uint32_t ntasks,
          uint32_t task_warps)
{
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  if (warp < task_warps)
  {
    for (uint64_t t = warp; t < (uint64_t) ntasks * W; t += task_warps)
    {
      const uint32_t k = (uint32_t) (t / W), w = (uint32_t) (t % W);
      const uint32_t v = task_row[k];
      const uint32_t r0 = w * 64 + lane, r1 = r0 + 32;
      uint32_t y0 = kInfD, y1 = kInfD;
      for (uint32_t e0 = task_b[k]; e0 < task_e[k]; e0 += 8)
        bs_pull8(e0, task_e[k], lane, w, R, W, r0, r1, col, wgt, front, msg, y0, y1);
      bool l0 = false, l1 = false;
      if (y0 != kInfD) l0 = y0 < atomicMin(&dist[(uint64_t) v * R + r0], y0);
      if (y1 != kInfD) l1 = y1 < atomicMin(&dist[(uint64_t) v * R + r1], y1);
      const uint64_t mask = (uint64_t) __ballot_sync(0xffffffffu, l0) | ((uint64_t) __ballot_sync(0xffffffffu, l1) << 32);
      if (lane == 0 && mask) atomicOr((unsigned long long*) &next[(uint64_t) v * W + w], (unsigned long long) mask);
    }
    return;
  }
  const uint64_t NP = (uint64_t) nreg * W;
  for (uint64_t i = warp - task_warps; i < NP; i += nwarps - task_warps)
  {
    const uint32_t v = (uint32_t) (i / W), w = (uint32_t) (i % W);
    const uint32_t b = ptr[v], e = ptr[v + 1];
    if (e - b > kLanePullLong) continue;  // the tasks take it
    const uint32_t r0 = w * 64 + lane, r1 = r0 + 32;
    uint32_t y0 = kInfD, y1 = kInfD;
    for (uint32_t e0 = b; e0 < e; e0 += 8) bs_pull8(e0, e, lane, w, R, W, r0, r1, col, wgt, front, msg, y0, y1);
    bool l0 = false, l1 = false;
    if (y0 != kInfD)
    {
      uint32_t* p = &dist[(uint64_t) v * R + r0];
      if (y0 < *p)
      {
        *p = y0;
        l0 = true;
      }
    }
    if (y1 != kInfD)
    {
      uint32_t* p = &dist[(uint64_t) v * R + r1];
      if (y1 < *p)
      {
        *p = y1;
        l1 = true;
      }
    }
    const uint64_t mask = (uint64_t) __ballot_sync(0xffffffffu, l0) | ((uint64_t) __ballot_sync(0xffffffffu, l1) << 32);
    if (lane == 0) next[i] = mask;
  }
}

// Tasks over the regular rows with more than kLanePullLong in-edges (built
// once per graph on the host from the row offsets).
struct LanePullTasks
{
  uint32_t* row = nullptr;
  uint32_t* b = nullptr;
  uint32_t* e = nullptr;
  uint32_t n = 0;
  uint32_t reg_in = 0;  // in-edges of the regular rows
  bool ready = false;
};

static inline int lane_pull_tasks(la3g_graph* G, LanePullTasks* T)
{
  if (T->ready) return LA3G_OK;
  const DevGraph& g = G->g;
  std::vector<uint32_t> ptr((size_t) g.nreg + 1);
  LA3G_CUDA(cudaMemcpy(ptr.data(), g.in_ptr, ptr.size() * 4, cudaMemcpyDeviceToHost));
  T->reg_in = ptr[g.nreg] - ptr[0];
  std::vector<uint32_t> row, b, e;
  for (uint32_t v = 0; v < g.nreg; v++)
    if (ptr[v + 1] - ptr[v] > kLanePullLong)
      for (uint32_t x = ptr[v]; x < ptr[v + 1]; x += kLanePullLong)
      {
        row.push_back(v);
        b.push_back(x);
        e.push_back(std::min(x + kLanePullLong, ptr[v + 1]));
      }
  T->n = (uint32_t) row.size();
  const size_t n = std::max<size_t>(row.size(), 1);
  LA3G_TRY(galloc(G, &T->row, n));
  LA3G_TRY(galloc(G, &T->b, n));
  LA3G_TRY(galloc(G, &T->e, n));
  if (T->n)
  {
    LA3G_CUDA(cudaMemcpy(T->row, row.data(), row.size() * 4, cudaMemcpyHostToDevice));
    LA3G_CUDA(cudaMemcpy(T->b, b.data(), b.size() * 4, cudaMemcpyHostToDevice));
    LA3G_CUDA(cudaMemcpy(T->e, e.data(), e.size() * 4, cudaMemcpyHostToDevice));
  }
  T->ready = true;
  return LA3G_OK;
}

// Initial active list: the nonzero words of the root frontier.
static __global__ void k_bs_list(uint64_t NW, uint32_t W, const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ reg_end,
                          const uint64_t* __restrict__ front, PairList out)
{
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < NW; i += (uint64_t) gridDim.x * blockDim.x)
    if (front[i])
    {
      const uint32_t v = (uint32_t) (i / W);
      bs_list_pair((uint32_t) i, reg_end[v] - ptr[v], out);
    }
}

static __global__ void k_max_u32(const uint32_t* __restrict__ a, uint64_t n, unsigned int* out)
{
  unsigned int m = 0;
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
    m = max(m, a[i]);
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

static __global__ void k_reg_end(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ row, uint32_t N, uint32_t nreg,
                          uint32_t* reg_end)
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

// Pull when the active pairs' out-degree sum exceeds the regular rows'
// in-edges times the words over this divisor; 0 = always push, the default:
// on R-MAT s18-s23 with 64 roots per word the pull step costs about what the
// push step does (it is faster on s18, slower on s21 / s23), because a lane
// set's work is its roots' own relaxations either way.  LA3G_LANES_PULL sets
// the divisor.
static inline double lanes_pull_divisor()
{
  static double d = -1;
  if (d < 0)
  {
    const char* e = std::getenv("LA3G_LANES_PULL");
    d = e ? std::atof(e) : 0.0;
  }
  return d;
}

}  // namespace la3g

#endif
