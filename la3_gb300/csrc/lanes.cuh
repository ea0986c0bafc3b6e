// Kernels shared by the batched SSSP (la3g_sssp_batch) and the serving
// loop's SSSP lanes: distances are kept [vertex][root] (uint32, INF =
// 2^31 - 1) with one frontier bit per (vertex, root) packed 64 roots to a
// word; an iteration relaxes the out-edges of every active (vertex, word)
// pair.  Everything here has internal linkage so that each translation unit
// that includes it gets its own copy.
#ifndef LA3G_LANES_CUH
#define LA3G_LANES_CUH

#include <cstdint>

#include "frontier.cuh"

namespace la3g {

static constexpr uint32_t kInfD = 0x7FFFFFFFu;
static constexpr uint32_t kNoWindow = 0xFFFFFFFFu;  // relax every active root

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

// Position of the s-th (from 0) set bit of f; s < popcount(f).
static __device__ __forceinline__ int nth_set_bit(uint64_t f, int s)
{
  int pos = 0;
  uint32_t x = (uint32_t) f;
  int c = __popc(x);
  if (s >= c)
  {
    s -= c;
    x = (uint32_t) (f >> 32);
    pos = 32;
  }
  c = __popc(x & 0xFFFFu);
  if (s >= c) { s -= c; x >>= 16; pos += 16; }
  c = __popc(x & 0xFFu);
  if (s >= c) { s -= c; x >>= 8; pos += 8; }
  c = __popc(x & 0xFu);
  if (s >= c) { s -= c; x >>= 4; pos += 4; }
  c = __popc(x & 0x3u);
  if (s >= c) { s -= c; x >>= 2; pos += 2; }
  if (s >= (int) (x & 1u)) pos += 1;
  return pos;
}

// Pairs with at most 32 active roots: the k active roots are packed into
// groups of S = next power of two >= k lanes, so a warp step covers 32 / S
// edges (four steps unrolled, their target reads in flight together); a
// lowered root ORs its own bit into the target's next word.
static __device__ __forceinline__ void bs_relax_sparse(uint32_t k0, uint32_t k1, int lane, uint32_t R, uint32_t W,
                                                const uint32_t* __restrict__ row, const uint32_t* __restrict__ wgt,
                                                uint32_t u, uint32_t w, uint64_t f, int k, uint64_t* next, uint32_t* dist,
                                                uint32_t& lmin)
{
  const int S = k <= 1 ? 1 : 1 << (32 - __clz(k - 1));
  const uint32_t E = 32 / S;
  const int slot = lane & (S - 1);
  const uint32_t e = (uint32_t) lane / S;
  const bool act = slot < k;
  const int b = act ? nth_set_bit(f, slot) : 0;
  const uint32_t r = w * 64 + b;
  const uint32_t m = act ? __ldcg(&dist[(uint64_t) u * R + r]) : 0;
  const unsigned long long bit = 1ull << b;
  for (uint32_t kb = k0; kb < k1; kb += 4 * E)
  {
    uint32_t v[4], wt[4], d[4];
    bool live[4];
#pragma unroll
    for (int q = 0; q < 4; q++)
    {
      const uint32_t ke = kb + q * E + e;
      live[q] = act && ke < k1;
      v[q] = live[q] ? row[ke] : 0;
      wt[q] = live[q] ? wgt[ke] : 0;
    }
#pragma unroll
    for (int q = 0; q < 4; q++) d[q] = live[q] ? __ldcg(&dist[(uint64_t) v[q] * R + r]) : 0;
#pragma unroll
    for (int q = 0; q < 4; q++)
    {
      const uint32_t c = m + wt[q];
      if (live[q] && c < d[q])
      {
        atomicMin(&dist[(uint64_t) v[q] * R + r], c);
        atomicOr((unsigned long long*) &next[(uint64_t) v[q] * W + w], bit);
        lmin = min(lmin, c);
      }
    }
  }
}

// Pairs with more than 32 active roots: lane l handles roots 64w + l and
// 64w + l + 32, so the distances of one edge's target are read contiguously;
// the roots an edge lowered are ORed into the target's next-frontier word at
// once.  Edges go 8 at a time (targets and weights loaded by 8 lanes and
// broadcast) so that up to 16 target reads per lane are in flight.
static __device__ __forceinline__ void bs_relax_dense(uint32_t k0, uint32_t k1, int lane, uint32_t R, uint32_t W,
                                               const uint32_t* __restrict__ row, const uint32_t* __restrict__ wgt,
                                               uint32_t u, uint32_t w, uint64_t f, uint64_t* next, uint32_t* dist,
                                               uint32_t& lmin)
{
  constexpr int G = 8;
  const uint32_t r0 = w * 64 + lane, r1 = r0 + 32;
  const bool h0 = (f >> lane) & 1ull, h1 = (f >> (lane + 32)) & 1ull;
  const uint32_t m0 = h0 ? __ldcg(&dist[(uint64_t) u * R + r0]) : 0, m1 = h1 ? __ldcg(&dist[(uint64_t) u * R + r1]) : 0;
  for (uint32_t kb = k0; kb < k1; kb += G)
  {
    const uint32_t cnt = min((uint32_t) G, k1 - kb);
    uint32_t lv = 0, lw = 0;
    if ((uint32_t) lane < cnt)
    {
      lv = row[kb + lane];
      lw = wgt[kb + lane];
    }
    uint32_t v[G];
#pragma unroll
    for (int j = 0; j < G; j++) v[j] = __shfl_sync(0xffffffffu, lv, j);
    uint32_t d0[G], d1[G];
#pragma unroll
    for (int j = 0; j < G; j++)
    {
      const bool live = (uint32_t) j < cnt;
      d0[j] = live && h0 ? __ldcg(&dist[(uint64_t) v[j] * R + r0]) : 0u;
      d1[j] = live && h1 ? __ldcg(&dist[(uint64_t) v[j] * R + r1]) : 0u;
    }
    // lane j keeps edge j's new bits and ORs them into next once
    uint64_t mine = 0;
#pragma unroll
    for (int j = 0; j < G; j++)
    {
      if ((uint32_t) j >= cnt) break;
      const uint32_t wt = __shfl_sync(0xffffffffu, lw, j), c0 = m0 + wt, c1 = m1 + wt;
      const bool i0 = h0 && c0 < d0[j], i1 = h1 && c1 < d1[j];
      if (i0)
      {
        atomicMin(&dist[(uint64_t) v[j] * R + r0], c0);
        lmin = min(lmin, c0);
      }
      if (i1)
      {
        atomicMin(&dist[(uint64_t) v[j] * R + r1], c1);
        lmin = min(lmin, c1);
      }
      const uint64_t mask = (uint64_t) __ballot_sync(0xffffffffu, i0) | ((uint64_t) __ballot_sync(0xffffffffu, i1) << 32);
      if (lane == j) mine = mask;
    }
    if (mine) atomicOr((unsigned long long*) &next[(uint64_t) lv * W + w], (unsigned long long) mine);
  }
}

// Relaxes edges [k0, k1) of the vertex of pair i (a warp, all lanes).  A
// source's distances are read when its pair is taken, not as of the
// iteration's start: a value lowered earlier in the same iteration reaches its
// targets at once (Gauss-Seidel order), and the source is in the next frontier
// anyway; every order of relaxation ends at the same shortest distances.  A
// root's bit is set when its candidate is below the distance read through L2:
// distances only fall, so that read is at most the value the iteration
// started with and the bit means "lowered in this iteration", exactly as an
// atomic's returned old value would; the minimum itself is therefore a
// reduction whose result nobody waits for.
//
// With a window (limit != kNoWindow) only roots whose distance at u is at most
// limit relax; the others keep their bit, carried into the next frontier, as
// delta-stepping keeps a vertex in a later bucket.  lmin collects the smallest
// distance the next frontier will hold (carried distances and lowered
// candidates), from which the host sets the next window.  Every active bit is
// either relaxed or carried, so the shortest distances are the same.
static __device__ __forceinline__ void bs_relax_range(uint32_t i, uint32_t k0, uint32_t k1, int lane, uint32_t R, uint32_t W,
                                               const uint32_t* __restrict__ row, const uint32_t* __restrict__ wgt,
                                               const uint64_t* __restrict__ front, uint64_t* next, uint32_t* dist,
                                               uint32_t limit, uint32_t& lmin)
{
  const uint32_t u = i / W, w = i % W;
  uint64_t f = front[i];
  if (limit != kNoWindow)
  {
    const uint32_t r0 = w * 64 + lane;
    const bool h0 = (f >> lane) & 1ull, h1 = (f >> (lane + 32)) & 1ull;
    const uint32_t m0 = h0 ? __ldcg(&dist[(uint64_t) u * R + r0]) : 0u;
    const uint32_t m1 = h1 ? __ldcg(&dist[(uint64_t) u * R + r0 + 32]) : 0u;
    const bool far0 = h0 && m0 > limit, far1 = h1 && m1 > limit;
    const uint64_t far = (uint64_t) __ballot_sync(0xffffffffu, far0) | ((uint64_t) __ballot_sync(0xffffffffu, far1) << 32);
    if (far)
    {
      if (far0) lmin = min(lmin, m0);
      if (far1) lmin = min(lmin, m1);
      if (lane == 0) atomicOr((unsigned long long*) &next[i], (unsigned long long) far);
      f &= ~far;
      if (!f) return;
    }
  }
  const int k = __popcll(f);
  if (k > 32) bs_relax_dense(k0, k1, lane, R, W, row, wgt, u, w, f, next, dist, lmin);
  else bs_relax_sparse(k0, k1, lane, R, W, row, wgt, u, w, f, k, next, dist, lmin);
}

static __global__ void __launch_bounds__(256, 4)
k_bs_relax(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ reg_end, const uint32_t* __restrict__ row,
           const uint32_t* __restrict__ wgt, uint32_t R, uint32_t W, const uint64_t* __restrict__ front, PairList L,
           uint64_t* next, uint32_t* dist, uint32_t limit = kNoWindow, unsigned int* pend_min = nullptr)
{
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t ns = (uint32_t) *L.nsmall;
  const unsigned long long pk = *L.packed;
  const uint32_t nbig = hub_count(pk), ntasks = hub_tasks(pk);
  uint32_t lmin = 0xFFFFFFFFu;
  for (uint32_t a = warp; a < ntasks + ns; a += nwarps)
  {
    if (a < ntasks)
    {
      const uint32_t slot = hub_of_task(L.hub_t0, nbig, a);
      const uint32_t i = L.hub[slot], u = i / W;
      const uint32_t k0 = ptr[u] + (a - L.hub_t0[slot]) * kHubTask;
      bs_relax_range(i, k0, min(k0 + kHubTask, reg_end[u]), lane, R, W, row, wgt, front, next, dist, limit, lmin);
    }
    else
    {
      const uint32_t i = L.small[a - ntasks], u = i / W;
      bs_relax_range(i, ptr[u], reg_end[u], lane, R, W, row, wgt, front, next, dist, limit, lmin);
    }
  }
  if (pend_min)
  {
    for (int o = 16; o > 0; o >>= 1) lmin = min(lmin, __shfl_xor_sync(0xffffffffu, lmin, o));
    if (lane == 0 && lmin != 0xFFFFFFFFu) atomicMin(pend_min, lmin);
  }
}

// After a relaxation: the old frontier words are cleared (they become the
// next "next" buffer) and the words holding newly lowered roots form the next
// active list.  alive (W words, optional) collects the roots that still have
// a frontier.
static __global__ void k_bs_apply(uint32_t N, uint32_t W, const uint32_t* __restrict__ ptr,
                                  const uint32_t* __restrict__ reg_end, const uint64_t* __restrict__ next,
                                  PairList out, uint64_t* front_old, PairList old, uint64_t* alive = nullptr)
{
  const uint64_t tid = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x, nth = (uint64_t) gridDim.x * blockDim.x;
  const uint64_t ns = *old.nsmall, nb = hub_count(*old.packed);
  for (uint64_t k = tid; k < ns; k += nth) front_old[old.small[k]] = 0;
  for (uint64_t k = tid; k < nb; k += nth) front_old[old.hub[k]] = 0;
  const uint64_t NW = (uint64_t) N * W;
  for (uint64_t i = tid; i < NW; i += nth)
  {
    const uint64_t f = next[i];
    if (!f) continue;
    const uint32_t v = (uint32_t) (i / W), w = (uint32_t) (i % W);
    bs_list_pair((uint32_t) i, reg_end[v] - ptr[v], out);
    if (alive && (alive[w] & f) != f) atomicOr((unsigned long long*) &alive[w], (unsigned long long) f);
  }
}

// Top-down step of a multi-source BFS over a split list of frontier
// (vertex, word) pairs (small pairs a warp each, hub edges as kHubTask-edge
// tasks): each edge's target gets the word's bits that it has not visited,
// ORed into its next word (skipped when already there).
static __device__ __forceinline__ void ms_push_pairs(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col,
                                                     uint32_t W, const uint64_t* __restrict__ front,
                                                     const uint64_t* __restrict__ vis, uint64_t* next, const PairList& L)
{
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t ns = (uint32_t) *L.nsmall;
  const unsigned long long pk = *L.packed;
  const uint32_t nbig = hub_count(pk), ntasks = hub_tasks(pk);
  for (uint32_t a = warp; a < ntasks + ns; a += nwarps)
  {
    uint32_t i, k0, k1;
    if (a < ntasks)
    {
      const uint32_t slot = hub_of_task(L.hub_t0, nbig, a);
      i = L.hub[slot];
      const uint32_t u = i / W;
      k0 = ptr[u] + (a - L.hub_t0[slot]) * kHubTask;
      k1 = min(k0 + kHubTask, ptr[u + 1]);
    }
    else
    {
      i = L.small[a - ntasks];
      const uint32_t u = i / W;
      k0 = ptr[u];
      k1 = ptr[u + 1];
    }
    const uint32_t w = i % W;
    const uint64_t f = front[i];
    for (uint32_t e = k0 + lane; e < k1; e += 32)
    {
      const uint64_t j = (uint64_t) col[e] * W + w;
      const uint64_t nb = f & ~vis[j];
      if (nb && (next[j] & nb) != nb) atomicOr((unsigned long long*) &next[j], (unsigned long long) nb);
    }
  }
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

}  // namespace la3g

#endif
