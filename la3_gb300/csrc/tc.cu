// Triangle counting: the reference tc app (src/apps/graph_analytics/
// tc.cpp:11-52, tc.h:47-99) on the device.
//
// The reference orients every edge from the lower to the higher original id
// (remove_cycles, graph.hpp:174-179), collects for each vertex v the list
// N<(v) of its lower neighbours (GnVertex), and for every oriented edge
// (u, v), u < v, adds |N<(u) ∩ N<(v)| to u, accumulating in uint32 (CtVertex).
// Each triangle a < b < c is therefore counted once, at its middle vertex b.
//
// Here the triangles are found once each by the usual degree ordering
// instead: rank(x) = (degree, id), N+(x) = neighbours of higher rank (sorted
// by id), and every triangle x < y < w in rank order is found while scanning
// the edge (x, y) as w ∈ N+(x) ∩ N+(y).  The middle vertex BY ID is then the
// median of the three ids; since y and w both lie in N+(x), the warp that
// owns x keeps one shared-memory counter per element of N+(x) (plus one for
// x) and adds every found triangle to the counter of its middle vertex,
// flushing them to the global uint32 counts once per x.  The per-vertex
// counts are those of the reference (sums are order-free); the lists stay
// short (max |N+| is about sqrt(2m)), which is what makes this fast on
// skewed graphs.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "la3g_internal.h"

namespace la3g {

static constexpr uint32_t kTcCap = 1024;     // N+(x) held in shared memory up to this length
static constexpr uint32_t kTcSmall = 192;    // lists up to this length use the high-occupancy variant
static constexpr uint32_t kTcWalkFactor = 16;  // heavy x: N+(y) is walked unless > 16 |N+(x)| (then searched)
static constexpr uint32_t kTcHubMin = 32;    // N+(y) longer than this (and than N+(x)) is a hub list:
static constexpr uint32_t kTcHubCap = 1024;  // ... small x's pairs with it go to the hub kernel, up to this length
static constexpr int kTcHubLanes = 8;        // lanes per hub pair in k_tc_hub

// A pair (x, y) of a list N+(x) (at most kTcCap long) with a longer list
// N+(y) of moderate length: instead of walking N+(y) against N+(x), or
// binary-searching N+(y) in global memory for every element of N+(x), the
// pair is handled hub-centrically (k_tc_hub walks the shorter N+(x)).
__device__ __forceinline__ bool tc_is_hub_pair(uint32_t d, uint32_t ylen)
{
  return ylen > d && ylen > kTcHubMin && ylen <= kTcHubCap;
}

struct TcScratch
{
  uint32_t* plus_ptr = nullptr;  // [nslots + 1] by original id
  uint32_t* plus_col = nullptr;  // [nent] ids, each row ascending
  uint32_t* plus_col_r = nullptr;  // [nent] the same rows ordered by rank (ids stored)
  uint32_t* order = nullptr;     // ids with 0 < |N+| <= kTcSmall, heaviest first
  uint32_t* order_mid = nullptr; // ids with kTcSmall < |N+| <= kTcCap, heaviest first
  uint32_t* big = nullptr;       // ids with |N+| > kTcCap
  uint32_t norder = 0, nmid = 0, nbig = 0;
  uint32_t* ntri = nullptr;      // [nslots] by id
  unsigned int* next = nullptr;  // dynamic work counter
  unsigned long long* total = nullptr;
  double work = 0;               // sum over x of |N+(x)| + sum_y |N+(y)| (list elements read)
  double work_mid = 0, work_big = 0;  // the part of it in the block-per-x and the global-search classes
  // hub-centric pairs: small x with y in N+(x), |N+(y)| > max(|N+(x)|, kTcHubMin)
  uint32_t* hub_ptr = nullptr;   // [nslots + 1] by id of y
  uint32_t* hub_x = nullptr;     // the x's of each hub y
  uint32_t* hub_j = nullptr;     // ... and the index of y in x's rank-ordered row
  uint32_t* hubs = nullptr;      // hub ids, heaviest first
  uint32_t nhubs = 0;
  uint32_t hub_pairs = 0;
  double hub_items = 0;          // sum over hub pairs of the part of N+(x) ranked above y
  double hub_lists = 0;          // sum over hubs of |N+(y)|
};

static void tc_scratch_free(void* p) { delete (TcScratch*) p; }

// Undirected degree by id: lower + higher neighbours.
__global__ void k_tc_deg(const uint32_t* __restrict__ iptr, const uint32_t* __restrict__ optr,
                         const uint32_t* __restrict__ id_of_pos, uint32_t N, uint32_t* deg)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x)
    deg[id_of_pos[p]] = (iptr[p + 1] - iptr[p]) + (optr[p + 1] - optr[p]);
}

// Every undirected edge once (push CSR of the id-oriented graph), emitted as
// (lower rank, higher rank) = id(x) << 32 | id(y).
__global__ void k_tc_rank_edges(const uint32_t* __restrict__ optr, const uint32_t* __restrict__ orow, uint32_t N,
                                const uint32_t* __restrict__ id_of_pos, const uint32_t* __restrict__ deg,
                                uint64_t* keys)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x)
  {
    const uint32_t a = id_of_pos[p];
    const uint32_t da = deg[a];
    for (uint32_t e = optr[p]; e < optr[p + 1]; e++)
    {
      const uint32_t b = id_of_pos[orow[e]];
      const uint32_t db = deg[b];
      const bool a_low = da < db || (da == db && a < b);
      keys[e] = a_low ? ((uint64_t) a << 32 | b) : ((uint64_t) b << 32 | a);
    }
  }
}

__global__ void k_tc_split_keys(const uint64_t* __restrict__ keys, uint64_t m, uint32_t* col)
{
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t) gridDim.x * blockDim.x)
    col[i] = (uint32_t) keys[i];
}

__global__ void k_tc_rows(const uint64_t* __restrict__ k, uint64_t m, uint32_t N, uint32_t* ptr)
{
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i <= m; i += (uint64_t) gridDim.x * blockDim.x)
  {
    int64_t r = i < m ? (int64_t) (k[i] >> 32) : (int64_t) N;
    int64_t rp = i == 0 ? -1 : (int64_t) (k[i - 1] >> 32);
    for (int64_t q = rp + 1; q <= r; q++) ptr[q] = (uint32_t) i;
  }
}

// Vertex ranks for the rank-ordered rows: keys (degree, id) sorted give
// rank -> id; rank_of_id is its inverse.
__global__ void k_tc_vkeys(uint32_t N, const uint32_t* __restrict__ deg, uint64_t* keys)
{
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x)
    keys[v] = (uint64_t) deg[v] << 32 | v;
}

__global__ void k_tc_ranks(uint32_t N, const uint64_t* __restrict__ sorted, uint32_t* rank_of_id, uint32_t* id_of_rank)
{
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < N; r += gridDim.x * blockDim.x)
  {
    const uint32_t v = (uint32_t) sorted[r];
    rank_of_id[v] = r;
    id_of_rank[r] = v;
  }
}

// (x, id) keys of the id-ordered rows -> (x, rank) keys, and back to ids
// once sorted.
__global__ void k_tc_rank_keys(const uint64_t* __restrict__ k, uint64_t m, const uint32_t* __restrict__ rank_of_id,
                               uint64_t* out)
{
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t) gridDim.x * blockDim.x)
    out[i] = (k[i] & 0xFFFFFFFF00000000ull) | rank_of_id[(uint32_t) k[i]];
}

__global__ void k_tc_rank_ids(const uint64_t* __restrict__ k, uint64_t m, const uint32_t* __restrict__ id_of_rank,
                              uint32_t* col)
{
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t) gridDim.x * blockDim.x)
    col[i] = id_of_rank[(uint32_t) k[i]];
}

// Work estimate per vertex and the lists of vertices to process.
__global__ void k_tc_work(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, uint32_t N,
                          uint32_t* wkey, uint32_t* wid, uint32_t* big, unsigned long long* counts)
{
  for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < N; x += gridDim.x * blockDim.x)
  {
    const uint32_t b = ptr[x], e = ptr[x + 1];
    if (b == e) continue;
    uint64_t w = e - b;
    const uint32_t d = e - b;
    for (uint32_t i = b; i < e; i++)
    {
      const uint32_t ylen = ptr[col[i] + 1] - ptr[col[i]];
      // a hub pair is walked by k_tc_hub (|N+(x)| elements, counted there)
      if (d <= kTcCap && tc_is_hub_pair(d, ylen)) continue;
      w += ylen;
    }
    if (e - b > kTcCap)
    {
      big[atomicAdd(&counts[1], 1ull)] = x;
      atomicAdd(&counts[5], (unsigned long long) w);
    }
    else
    {
      // keys: class bit on top (small lists first), then ~work (heaviest first)
      const uint32_t cls = (e - b) > kTcSmall ? 1u : 0u;
      const unsigned long long slot = atomicAdd(&counts[0], 1ull);
      const uint32_t wq = (uint32_t) (w < 0x7FFFFFFFull ? w : 0x7FFFFFFFull);
      wkey[slot] = (cls << 31) | (0x7FFFFFFFu - wq);
      wid[slot] = x;
      if (cls)
      {
        atomicAdd(&counts[3], 1ull);
        atomicAdd(&counts[4], (unsigned long long) w);
      }
    }
    atomicAdd(&counts[2], (unsigned long long) w);
  }
}

// Shared-memory set of N+(x) for O(1) membership: open addressing with
// linear probing over a power-of-two table of at least 2 |N+(x)| slots;
// each slot holds a vertex id and its index in N+(x).
static constexpr uint32_t kEmpty = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t tc_slot(uint32_t w, int lg) { return (w * 0x9E3779B1u) >> (32 - lg); }

__host__ __device__ constexpr uint32_t tc_pow2(uint32_t v) { return v <= 32 ? 32 : 2 * tc_pow2((v + 1) / 2); }

__device__ __forceinline__ int tc_lg(uint32_t d)
{
  int lg = 5;
  while ((1u << lg) < 2 * d) lg++;
  return lg;
}

// Counts the triangle {x, y, w} (w found at index pw of N+(x), y at index
// jy) at its middle id: x through cx, the others through their counters.
__device__ __forceinline__ void tc_attribute(uint32_t x, uint32_t y, uint32_t w, uint32_t jy, uint32_t pw,
                                             uint32_t* Cn, uint32_t& cx)
{
  // the middle id of {x, y, w}: w itself, or the larger / smaller of x, y;
  // x's count stays in a register (one shared word would serialise lanes)
  const uint32_t mn = min(x, y), mx = max(x, y);
  const uint32_t mid = w < mn ? mn : (w > mx ? mx : w);
  if (mid == x) cx++;
  else atomicAdd(&Cn[mid == w ? pw : jy], 1u);
}

// x's walk with lane groups of G lanes: group g takes y = L[jy] for jy = g,
// g + ngroups, ...; its lanes walk N+(y) (coalesced loads, each element
// probed in the hash set of N+(x)) unless N+(y) is more than walk_factor
// times longer than N+(x), in which case they walk N+(x) and binary-search
// each element in N+(y).
// Bloom bits of N+(x) (one hash, kBloomBits bits): most candidates that
// are not in N+(x) are rejected by one shared load, before the probe loop.
static constexpr uint32_t kBloomBits = 1u << 16;
__device__ __forceinline__ uint32_t tc_bloom(uint32_t w) { return (w * 0x85EBCA6Bu) >> 16; }

template <int G, class IDX>
__device__ __forceinline__ void tc_walk(uint32_t x, uint32_t d, const uint32_t* L, uint32_t* Cn, const uint32_t* key,
                                        const IDX* idx, int lg, uint32_t* cx, const uint32_t* __restrict__ ptr,
                                        const uint32_t* __restrict__ col, uint32_t walk_factor, uint32_t g,
                                        uint32_t ngroups, uint32_t glane, const uint32_t* bloom = nullptr)
{
  const uint32_t mask = (1u << lg) - 1;
  uint32_t cxr = 0;  // triangles counted at x by this lane
  for (uint32_t jy = g; jy < d; jy += ngroups)
  {
    const uint32_t y = L[jy];
    const uint32_t yb = ptr[y], ylen = ptr[y + 1] - yb;
    if (tc_is_hub_pair(d, ylen)) continue;  // k_tc_hub walks this pair
    if (ylen <= walk_factor * d)
    {
      // four independent list loads in flight per lane, then the probes
      for (uint32_t r0 = glane; r0 < ylen; r0 += 4 * G)
      {
        uint32_t wv[4];
#pragma unroll
        for (int u = 0; u < 4; u++) wv[u] = r0 + u * G < ylen ? col[yb + r0 + u * G] : kEmpty;
#pragma unroll
        for (int u = 0; u < 4; u++)
        {
          const uint32_t w = wv[u];
          if (w == kEmpty) continue;
          if (bloom)
          {
            const uint32_t bb = tc_bloom(w);
            if (!((bloom[bb >> 5] >> (bb & 31)) & 1u)) continue;
          }
          uint32_t sl = tc_slot(w, lg);
          for (;;)
          {
            const uint32_t kk = key[sl];
            if (kk == w)
            {
              tc_attribute(x, y, w, jy, idx[sl], Cn, cxr);
              break;
            }
            if (kk == kEmpty) break;
            sl = (sl + 1) & mask;
          }
        }
      }
    }
    else
    {
      for (uint32_t r = glane; r < d; r += G)
      {
        const uint32_t w = L[r];
        uint32_t a = yb, c = yb + ylen;
        while (a < c)
        {
          const uint32_t mid = (a + c) >> 1;
          if (col[mid] < w) a = mid + 1;
          else c = mid;
        }
        if (a < yb + ylen && col[a] == w) tc_attribute(x, y, w, jy, r, Cn, cxr);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) cxr += __shfl_xor_sync(0xffffffffu, cxr, o);
  if ((threadIdx.x & 31) == 0 && cxr) atomicAdd(cx, cxr);
}

template <class IDX>
__device__ __forceinline__ void tc_insert_t(uint32_t* key, IDX* idx, int lg, uint32_t w, uint32_t j)
{
  const uint32_t mask = (1u << lg) - 1;
  uint32_t sl = tc_slot(w, lg);
  while (atomicCAS(&key[sl], kEmpty, w) != kEmpty) sl = (sl + 1) & mask;
  idx[sl] = (IDX) j;
}

__device__ __forceinline__ uint32_t lower_bound_s(const uint32_t* s, uint32_t n, uint32_t key)
{
  uint32_t lo = 0, hi = n;
  while (lo < hi)
  {
    uint32_t mid = (lo + hi) >> 1;
    if (s[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// One warp per vertex x (fetched dynamically, heaviest first).  Shared
// memory holds N+(x), the prefix offsets of the per-y work, and one counter
// per element of N+(x).  For each y in N+(x) the shorter of N+(y) and N+(x)
// is walked and its elements looked up in the other (a shared-memory binary
// search into N+(x), or a global one into N+(y)); lanes share the
// concatenated work of all y.  A hit w closes the triangle {x, y, w}, which
// is counted at its middle id.
// Counts, per hub y, the x's (|N+(x)| <= kTcCap) pointing at it and the
// part of their rows a walk reads: only the elements ranked above y (after y
// in the rank-ordered row) can lie in N+(y).
__global__ void k_tc_hub_count(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ colr, uint32_t N,
                               uint32_t* cnt, unsigned long long* work)
{
  for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < N; x += gridDim.x * blockDim.x)
  {
    const uint32_t b = ptr[x], d = ptr[x + 1] - b;
    if (d == 0 || d > kTcCap) continue;
    for (uint32_t i = b; i < b + d; i++)
    {
      const uint32_t y = colr[i];
      if (tc_is_hub_pair(d, ptr[y + 1] - ptr[y]))
      {
        atomicAdd(&cnt[y], 1u);
        atomicAdd(&work[y], (unsigned long long) (b + d - i - 1));
      }
    }
  }
}

__global__ void k_tc_hub_fill(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ colr, uint32_t N,
                              const uint32_t* __restrict__ hub_ptr, uint32_t* fill, uint32_t* hub_x, uint32_t* hub_j)
{
  for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < N; x += gridDim.x * blockDim.x)
  {
    const uint32_t b = ptr[x], d = ptr[x + 1] - b;
    if (d == 0 || d > kTcCap) continue;
    for (uint32_t i = b; i < b + d; i++)
    {
      const uint32_t y = colr[i];
      if (tc_is_hub_pair(d, ptr[y + 1] - ptr[y]))
      {
        const uint32_t slot = hub_ptr[y] + atomicAdd(&fill[y], 1u);
        hub_x[slot] = x;
        hub_j[slot] = i - b;
      }
    }
  }
}

// Totals for the algorithmic byte count: sum of |N+(x)| over hub pairs and
// of |N+(y)| over hubs.
__global__ void k_tc_hub_sums(const uint32_t* __restrict__ ptr, uint32_t N, const uint32_t* __restrict__ cnt,
                              const unsigned long long* __restrict__ work, unsigned long long* out)
{
  unsigned long long a = 0, b = 0;
  for (uint32_t y = blockIdx.x * blockDim.x + threadIdx.x; y < N; y += gridDim.x * blockDim.x)
    if (cnt[y])
    {
      a += work[y];
      b += ptr[y + 1] - ptr[y];
    }
  for (int o = 16; o > 0; o >>= 1)
  {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if ((threadIdx.x & 31) == 0)
  {
    if (a) atomicAdd(&out[0], a);
    if (b) atomicAdd(&out[1], b);
  }
}

// Hub keys for sorting: ~work so that heavier hubs come first.
__global__ void k_tc_hub_keys(uint32_t N, const uint32_t* __restrict__ cnt, const unsigned long long* __restrict__ work,
                              uint32_t* keys, uint32_t* ids, unsigned long long* n)
{
  for (uint32_t y = blockIdx.x * blockDim.x + threadIdx.x; y < N; y += gridDim.x * blockDim.x)
    if (cnt[y])
    {
      const unsigned long long k = atomicAdd(n, 1ull);
      const unsigned long long w = work[y];
      keys[k] = 0xFFFFFFFFu - (uint32_t) (w < 0xFFFFFFFFull ? w : 0xFFFFFFFFull);
      ids[k] = y;
    }
}

// One block per hub y (heaviest first): N+(y) is staged in shared memory
// with a hash set and Bloom bits; warps take the x's pointing at y, their
// lanes walk the part of x's rank-ordered row after y (coalesced; the rest
// is ranked below y and cannot lie in N+(y)) and probe N+(y).  A hit w closes the
// triangle {x, y, w}, counted at its middle id: y and w in shared counters
// (flushed once per hub), x through a warp sum per x.  (A flattened walk
// over chunks of x's, which fills the lanes better for short N+(x), measured
// slower: its staging and barriers cost more than the idle lanes.)
template <uint32_t CAP, int THREADS, int G>
__global__ void __launch_bounds__(THREADS)
k_tc_hub(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ colr, const uint32_t* __restrict__ hubs, uint32_t nhubs, const uint32_t* __restrict__ hub_ptr,
         const uint32_t* __restrict__ hub_x, const uint32_t* __restrict__ hub_j, unsigned int* next, uint32_t* ntri)
{
  __shared__ uint32_t L[CAP], Cn[CAP], key[2 * CAP];
  __shared__ uint16_t idx[2 * CAP];
  __shared__ uint32_t bloom[kBloomBits / 32];
  __shared__ uint32_t s_k, s_y;
  const int lane = threadIdx.x & 31;
  for (uint32_t i = threadIdx.x; i < kBloomBits / 32; i += THREADS) bloom[i] = 0;
  for (;;)
  {
    if (threadIdx.x == 0) s_k = atomicAdd(next, 1u);
    __syncthreads();
    const uint32_t k = s_k;
    if (k >= nhubs) break;
    const uint32_t y = hubs[k];
    const uint32_t yb = ptr[y], d = ptr[y + 1] - yb;
    const int lg = tc_lg(d);
    const uint32_t mask = (1u << lg) - 1;
    for (uint32_t i = threadIdx.x; i < (1u << lg); i += THREADS) key[i] = kEmpty;
    if (threadIdx.x == 0) s_y = 0;
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < d; j += THREADS)
    {
      const uint32_t w = colr[yb + j];  // set order is free: read the rows the walks read
      L[j] = w;
      Cn[j] = 0;
      tc_insert_t(key, idx, lg, w, j);
      const uint32_t bb = tc_bloom(w);
      atomicOr(&bloom[bb >> 5], 1u << (bb & 31));
    }
    __syncthreads();
    const uint32_t h0 = hub_ptr[y], h1 = hub_ptr[y + 1];
    // G lanes per pair (THREADS / G pairs at a time): the walked suffixes are
    // short, so whole warps per pair left most lanes idle
    const int gl = lane % G;
    const unsigned gmask = (G == 32 ? 0xffffffffu : ((1u << G) - 1) << (lane - gl));
    for (uint32_t h = h0 + threadIdx.x / G; h < h1; h += THREADS / G)
    {
      const uint32_t x = hub_x[h];
      const uint32_t j1 = hub_j[h] + 1;
      const uint32_t xb = ptr[x] + j1, xd = ptr[x + 1] - xb;
      const uint32_t mn = min(x, y), mx = max(x, y);
      uint32_t cnt_x = 0, cnt_y = 0;
      for (uint32_t r0 = gl; r0 < xd; r0 += 4 * G)
      {
        uint32_t wv[4];
#pragma unroll
        for (int u = 0; u < 4; u++) wv[u] = r0 + u * G < xd ? colr[xb + r0 + u * G] : kEmpty;
#pragma unroll
        for (int u = 0; u < 4; u++)
        {
          const uint32_t w = wv[u];
          if (w == kEmpty) continue;
          const uint32_t bb = tc_bloom(w);
          if (!((bloom[bb >> 5] >> (bb & 31)) & 1u)) continue;
          uint32_t sl = tc_slot(w, lg);
          for (;;)
          {
            const uint32_t kk = key[sl];
            if (kk == w)
            {
              const uint32_t mid = w < mn ? mn : (w > mx ? mx : w);
              if (mid == x) cnt_x++;
              else if (mid == y) cnt_y++;
              else atomicAdd(&Cn[idx[sl]], 1u);
              break;
            }
            if (kk == kEmpty) break;
            sl = (sl + 1) & mask;
          }
        }
      }
      for (int o = G / 2; o > 0; o >>= 1)
      {
        cnt_x += __shfl_xor_sync(gmask, cnt_x, o);
        cnt_y += __shfl_xor_sync(gmask, cnt_y, o);
      }
      if (gl == 0)
      {
        if (cnt_x) atomicAdd(&ntri[x], cnt_x);
        if (cnt_y) atomicAdd(&s_y, cnt_y);
      }
    }
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < d; j += THREADS)
    {
      if (Cn[j]) atomicAdd(&ntri[L[j]], Cn[j]);
      const uint32_t bb = tc_bloom(L[j]);
      bloom[bb >> 5] = 0;
    }
    if (threadIdx.x == 0 && s_y) atomicAdd(&ntri[y], s_y);
    __syncthreads();
  }
}

template <uint32_t CAP, int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
k_tc_rank_flat(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, const uint32_t* __restrict__ order,
          uint32_t norder, unsigned int* next, uint32_t* ntri)
{
  __shared__ uint32_t s_list[WARPS][CAP];
  __shared__ uint32_t s_off[WARPS][CAP + 1];
  __shared__ uint32_t s_cnt[WARPS][CAP];
  __shared__ uint32_t s_x[WARPS];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  uint32_t* L = s_list[wib];
  uint32_t* O = s_off[wib];
  uint32_t* Cn = s_cnt[wib];
  for (;;)
  {
    uint32_t k = 0;
    if (lane == 0) k = atomicAdd(next, 1u);
    k = __shfl_sync(0xffffffffu, k, 0);
    if (k >= norder) break;
    const uint32_t x = order[k];
    const uint32_t xb = ptr[x], d = ptr[x + 1] - xb;
    // stage N+(x), the work offsets (min(|N+(y)|, d) per y) and zeroed counters
    uint32_t base = 0;
    for (uint32_t j0 = 0; j0 < d; j0 += 32)
    {
      const uint32_t j = j0 + lane;
      uint32_t len = 0;
      if (j < d)
      {
        const uint32_t y = col[xb + j];
        const uint32_t ylen = ptr[y + 1] - ptr[y];
        // pairs with a hub list are walked by k_tc_hub instead
        len = tc_is_hub_pair(d, ylen) ? 0u : min(ylen, d);
        L[j] = y;
        Cn[j] = 0;
      }
      uint32_t incl = len;
      for (int o = 1; o < 32; o <<= 1)
      {
        uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      if (j < d) O[j] = base + incl - len;
      base += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0)
    {
      O[d] = base;
      s_x[wib] = 0;
    }
    __syncwarp();
    const uint32_t total = base;
    for (uint32_t t0 = 0; t0 < total; t0 += 32)
    {
      const uint32_t t = t0 + lane;
      if (t < total)
      {
        // y-index: the last j with O[j] <= t
        uint32_t lo = 0, hi = d;
        while (hi - lo > 1)
        {
          uint32_t mid = (lo + hi) >> 1;
          if (O[mid] <= t) lo = mid;
          else hi = mid;
        }
        const uint32_t jy = lo;
        const uint32_t y = L[jy];
        const uint32_t yb = ptr[y], ylen = ptr[y + 1] - yb;
        const uint32_t r = t - O[jy];
        uint32_t w, pw;
        bool hit;
        if (ylen <= d)
        {
          w = col[yb + r];
          pw = lower_bound_s(L, d, w);
          hit = pw < d && L[pw] == w;
        }
        else
        {
          pw = r;
          w = L[r];
          uint32_t a = yb, c = yb + ylen;
          while (a < c)
          {
            uint32_t mid = (a + c) >> 1;
            if (col[mid] < w) a = mid + 1;
            else c = mid;
          }
          hit = a < yb + ylen && col[a] == w;
        }
        if (hit)
        {
          const uint32_t mn = min(x, y), mx = max(x, y);
          if (w < mn) { if (mn == x) atomicAdd(&s_x[wib], 1u); else atomicAdd(&Cn[jy], 1u); }
          else if (w > mx) { if (mx == x) atomicAdd(&s_x[wib], 1u); else atomicAdd(&Cn[jy], 1u); }
          else atomicAdd(&Cn[pw], 1u);
        }
      }
    }
    __syncwarp();
    for (uint32_t j = lane; j < d; j += 32)
      if (Cn[j]) atomicAdd(&ntri[L[j]], Cn[j]);
    if (lane == 0 && s_x[wib]) atomicAdd(&ntri[x], s_x[wib]);
    __syncwarp();
  }
}

// Heavy vertices (kTcSmall < |N+(x)| <= kTcCap): a whole block per x, its
// threads in groups of G lanes.
template <uint32_t CAP, int THREADS, int G>
__global__ void __launch_bounds__(THREADS)
k_tc_rank_block(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, const uint32_t* __restrict__ order,
                uint32_t norder, unsigned int* next, uint32_t* ntri, uint32_t walk_factor)
{
  __shared__ uint32_t L[CAP], Cn[CAP], key[2 * CAP];
  __shared__ uint16_t idx[2 * CAP];
  __shared__ uint32_t bloom[kBloomBits / 32];
  __shared__ uint32_t s_k, s_x;
  for (uint32_t i = threadIdx.x; i < kBloomBits / 32; i += THREADS) bloom[i] = 0;
  for (;;)
  {
    if (threadIdx.x == 0) s_k = atomicAdd(next, 1u);
    __syncthreads();
    const uint32_t k = s_k;
    if (k >= norder) break;
    const uint32_t x = order[k];
    const uint32_t xb = ptr[x], d = ptr[x + 1] - xb;
    const int lg = tc_lg(d);
    for (uint32_t i = threadIdx.x; i < (1u << lg); i += THREADS) key[i] = kEmpty;
    if (threadIdx.x == 0) s_x = 0;
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < d; j += THREADS)
    {
      const uint32_t y = col[xb + j];
      L[j] = y;
      Cn[j] = 0;
      tc_insert_t(key, idx, lg, y, j);
      const uint32_t bb = tc_bloom(y);
      atomicOr(&bloom[bb >> 5], 1u << (bb & 31));
    }
    __syncthreads();
    tc_walk<G>(x, d, L, Cn, key, idx, lg, &s_x, ptr, col, walk_factor, threadIdx.x / G, THREADS / G, threadIdx.x % G,
               bloom);
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < d; j += THREADS)
    {
      if (Cn[j]) atomicAdd(&ntri[L[j]], Cn[j]);
      const uint32_t bb = tc_bloom(L[j]);
      bloom[bb >> 5] = 0;  // clears the words this x set (others are zero already)
    }
    if (threadIdx.x == 0 && s_x) atomicAdd(&ntri[x], s_x);
    __syncthreads();
  }
}

// Vertices whose N+ exceeds kTcCap: one warp each, lists read from global
// memory, every hit added with a global atomic.
__global__ void __launch_bounds__(256)
k_tc_rank_big(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, const uint32_t* __restrict__ big,
              uint32_t nbig, uint32_t* ntri)
{
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t k = warp; k < nbig; k += nwarps)
  {
    const uint32_t x = big[k];
    const uint32_t xb = ptr[x], xe = ptr[x + 1];
    for (uint32_t j = xb; j < xe; j++)
    {
      const uint32_t y = col[j];
      const uint32_t mn = min(x, y), mx = max(x, y);
      for (uint32_t i = ptr[y] + lane; i < ptr[y + 1]; i += 32)
      {
        const uint32_t w = col[i];
        uint32_t lo = xb, hi = xe;
        while (lo < hi)
        {
          uint32_t mid = (lo + hi) >> 1;
          if (col[mid] < w) lo = mid + 1;
          else hi = mid;
        }
        if (lo < xe && col[lo] == w) atomicAdd(&ntri[w < mn ? mn : (w > mx ? mx : w)], 1u);
      }
    }
  }
}

__global__ void k_tc_sum(uint32_t N, const uint32_t* __restrict__ ntri, unsigned long long* total)
{
  unsigned long long s = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x) s += ntri[v];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(total, s);
}

static int tc_prepare(la3g_graph* G, TcScratch* ts)
{
  DevGraph& g = G->g;
  cudaStream_t s = G->stream;
  const uint32_t N = g.nslots;
  const uint64_t m = g.nent;
  LA3G_TRY(galloc(G, &ts->plus_ptr, N + 1));
  LA3G_TRY(galloc(G, &ts->plus_col, m + 1));
  LA3G_TRY(galloc(G, &ts->ntri, N));
  LA3G_TRY(galloc(G, &ts->total, 1));
  LA3G_TRY(galloc(G, &ts->next, 4));
  DevBuf deg, k1, k2, tmp, wkey, wid, wkey2, cnt;
  LA3G_TRY(deg.alloc((size_t) N * 4));
  LA3G_TRY(k1.alloc(m * 8 + 8));
  LA3G_TRY(k2.alloc(m * 8 + 8));
  k_tc_deg<<<grid_for(N, 256), 256, 0, s>>>(g.in_ptr, g.out_ptr, g.id_of_pos, N, deg.as<uint32_t>());
  LA3G_LAUNCHED();
  if (m)
  {
    k_tc_rank_edges<<<grid_for(N, 256), 256, 0, s>>>(g.out_ptr, g.out_row, N, g.id_of_pos, deg.as<uint32_t>(),
                                                     k1.as<uint64_t>());
    LA3G_LAUNCHED();
    size_t tb = 0;
    int end_bit = 33;
    while (end_bit < 64 && ((uint64_t) N >> (end_bit - 32)) != 0) end_bit++;
    LA3G_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, tb, k1.as<uint64_t>(), k2.as<uint64_t>(), m, 0, end_bit, s));
    LA3G_TRY(tmp.alloc(tb));
    LA3G_CUDA(cub::DeviceRadixSort::SortKeys(tmp.p, tb, k1.as<uint64_t>(), k2.as<uint64_t>(), m, 0, end_bit, s));
    k_tc_split_keys<<<grid_for(m, 256), 256, 0, s>>>(k2.as<uint64_t>(), m, ts->plus_col);
    LA3G_LAUNCHED();
    // the same rows ordered by rank (degree, id), for the hub walks
    DevBuf vk, vk2, rk, ir, k3, t3;
    LA3G_TRY(vk.alloc((size_t) N * 8));
    LA3G_TRY(vk2.alloc((size_t) N * 8));
    LA3G_TRY(rk.alloc((size_t) N * 4));
    LA3G_TRY(ir.alloc((size_t) N * 4));
    LA3G_TRY(k3.alloc(m * 8 + 8));
    k_tc_vkeys<<<grid_for(N, 256), 256, 0, s>>>(N, deg.as<uint32_t>(), vk.as<uint64_t>());
    LA3G_LAUNCHED();
    size_t tv = 0;
    LA3G_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, tv, vk.as<uint64_t>(), vk2.as<uint64_t>(), N, 0, 64, s));
    LA3G_TRY(t3.alloc(std::max(tv, tb)));
    LA3G_CUDA(cub::DeviceRadixSort::SortKeys(t3.p, tv, vk.as<uint64_t>(), vk2.as<uint64_t>(), N, 0, 64, s));
    k_tc_ranks<<<grid_for(N, 256), 256, 0, s>>>(N, vk2.as<uint64_t>(), rk.as<uint32_t>(), ir.as<uint32_t>());
    LA3G_LAUNCHED();
    k_tc_rank_keys<<<grid_for(m, 256), 256, 0, s>>>(k2.as<uint64_t>(), m, rk.as<uint32_t>(), k3.as<uint64_t>());
    LA3G_LAUNCHED();
    LA3G_CUDA(cub::DeviceRadixSort::SortKeys(t3.p, tb, k3.as<uint64_t>(), k1.as<uint64_t>(), m, 0, end_bit, s));
    LA3G_TRY(galloc(G, &ts->plus_col_r, m + 1));
    k_tc_rank_ids<<<grid_for(m, 256), 256, 0, s>>>(k1.as<uint64_t>(), m, ir.as<uint32_t>(), ts->plus_col_r);
    LA3G_LAUNCHED();
    LA3G_CUDA(cudaStreamSynchronize(s));
  }
  else LA3G_TRY(galloc(G, &ts->plus_col_r, 1));
  k_tc_rows<<<grid_for(m + 1, 256), 256, 0, s>>>(k2.as<uint64_t>(), m, N, ts->plus_ptr);
  LA3G_LAUNCHED();
  LA3G_TRY(wkey.alloc((size_t) N * 4));
  LA3G_TRY(wid.alloc((size_t) N * 4));
  LA3G_TRY(wkey2.alloc((size_t) N * 4));
  LA3G_TRY(cnt.alloc(8 * 8));
  LA3G_TRY(galloc(G, &ts->order, N));
  LA3G_TRY(galloc(G, &ts->big, N));
  LA3G_CUDA(cudaMemsetAsync(cnt.p, 0, 64, s));
  k_tc_work<<<grid_for(N, 256), 256, 0, s>>>(ts->plus_ptr, ts->plus_col, N, wkey.as<uint32_t>(), wid.as<uint32_t>(),
                                             ts->big, cnt.as<unsigned long long>());
  LA3G_LAUNCHED();
  unsigned long long hc[8];
  LA3G_CUDA(cudaMemcpyAsync(hc, cnt.p, 64, cudaMemcpyDeviceToHost, s));
  LA3G_CUDA(cudaStreamSynchronize(s));
  ts->nmid = (uint32_t) hc[3];
  ts->norder = (uint32_t) hc[0];  // small + mid, sorted: small first
  ts->nbig = (uint32_t) hc[1];
  ts->work = (double) hc[2];
  ts->work_mid = (double) hc[4];
  ts->work_big = (double) hc[5];
  if (ts->norder)
  {
    size_t tb = 0;
    LA3G_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, wkey.as<uint32_t>(), wkey2.as<uint32_t>(), wid.as<uint32_t>(),
                                              ts->order, ts->norder, 0, 32, s));
    DevBuf t2;
    LA3G_TRY(t2.alloc(tb));
    LA3G_CUDA(cub::DeviceRadixSort::SortPairs(t2.p, tb, wkey.as<uint32_t>(), wkey2.as<uint32_t>(), wid.as<uint32_t>(),
                                              ts->order, ts->norder, 0, 32, s));
  }
  LA3G_CUDA(cudaStreamSynchronize(s));
  ts->order_mid = ts->order + (ts->norder - ts->nmid);
  ts->norder -= ts->nmid;

  // hub-centric pairs (small x, moderate hub y): CSR by y, hubs heaviest first
  DevBuf hcnt, hwork, hkeys, hkeys2, hids, hn;
  LA3G_TRY(hcnt.alloc((size_t) (N + 1) * 4));
  LA3G_TRY(hwork.alloc((size_t) N * 8));
  LA3G_CUDA(cudaMemsetAsync(hcnt.p, 0, (size_t) (N + 1) * 4, s));
  LA3G_CUDA(cudaMemsetAsync(hwork.p, 0, (size_t) N * 8, s));
  k_tc_hub_count<<<grid_for(N, 256), 256, 0, s>>>(ts->plus_ptr, ts->plus_col_r, N, hcnt.as<uint32_t>(),
                                                  hwork.as<unsigned long long>());
  LA3G_LAUNCHED();
  LA3G_TRY(galloc(G, &ts->hub_ptr, N + 1));
  {
    size_t tb = 0;
    LA3G_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, hcnt.as<uint32_t>(), ts->hub_ptr, N + 1, s));
    DevBuf t;
    LA3G_TRY(t.alloc(tb));
    LA3G_CUDA(cub::DeviceScan::ExclusiveSum(t.p, tb, hcnt.as<uint32_t>(), ts->hub_ptr, N + 1, s));
  }
  uint32_t npairs = 0;
  LA3G_CUDA(cudaMemcpyAsync(&npairs, ts->hub_ptr + N, 4, cudaMemcpyDeviceToHost, s));
  LA3G_CUDA(cudaStreamSynchronize(s));
  LA3G_TRY(galloc(G, &ts->hub_x, std::max<uint32_t>(npairs, 1)));
  LA3G_TRY(galloc(G, &ts->hub_j, std::max<uint32_t>(npairs, 1)));
  ts->hub_pairs = npairs;
  LA3G_TRY(galloc(G, &ts->hubs, N));
  if (npairs)
  {
    DevBuf fill;
    LA3G_TRY(fill.alloc((size_t) N * 4));
    LA3G_CUDA(cudaMemsetAsync(fill.p, 0, (size_t) N * 4, s));
    k_tc_hub_fill<<<grid_for(N, 256), 256, 0, s>>>(ts->plus_ptr, ts->plus_col_r, N, ts->hub_ptr, fill.as<uint32_t>(),
                                                   ts->hub_x, ts->hub_j);
    LA3G_LAUNCHED();
    LA3G_TRY(hkeys.alloc((size_t) N * 4));
    LA3G_TRY(hkeys2.alloc((size_t) N * 4));
    LA3G_TRY(hids.alloc((size_t) N * 4));
    LA3G_TRY(hn.alloc(8));
    LA3G_CUDA(cudaMemsetAsync(hn.p, 0, 8, s));
    k_tc_hub_keys<<<grid_for(N, 256), 256, 0, s>>>(N, hcnt.as<uint32_t>(), hwork.as<unsigned long long>(),
                                                   hkeys.as<uint32_t>(), hids.as<uint32_t>(),
                                                   hn.as<unsigned long long>());
    LA3G_LAUNCHED();
    DevBuf hsum;
    LA3G_TRY(hsum.alloc(16));
    LA3G_CUDA(cudaMemsetAsync(hsum.p, 0, 16, s));
    k_tc_hub_sums<<<grid_for(N, 256), 256, 0, s>>>(ts->plus_ptr, N, hcnt.as<uint32_t>(), hwork.as<unsigned long long>(),
                                                   hsum.as<unsigned long long>());
    LA3G_LAUNCHED();
    unsigned long long hs[2] = {0, 0};
    LA3G_CUDA(cudaMemcpyAsync(hs, hsum.p, 16, cudaMemcpyDeviceToHost, s));
    unsigned long long nh = 0;
    LA3G_CUDA(cudaMemcpyAsync(&nh, hn.p, 8, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    ts->nhubs = (uint32_t) nh;
    ts->hub_items = (double) hs[0];
    ts->hub_lists = (double) hs[1];
    size_t tb = 0;
    LA3G_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, hkeys.as<uint32_t>(), hkeys2.as<uint32_t>(),
                                              hids.as<uint32_t>(), ts->hubs, ts->nhubs, 0, 32, s));
    DevBuf t;
    LA3G_TRY(t.alloc(tb));
    LA3G_CUDA(cub::DeviceRadixSort::SortPairs(t.p, tb, hkeys.as<uint32_t>(), hkeys2.as<uint32_t>(),
                                              hids.as<uint32_t>(), ts->hubs, ts->nhubs, 0, 32, s));
  }
  LA3G_CUDA(cudaStreamSynchronize(s));
  return LA3G_OK;
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
    LA3G_TRY(tc_prepare(G, ts));
  }
  cudaStream_t s = G->stream;
  const uint32_t N = g.nslots;
  T.device_begin();
  LA3G_CUDA(cudaMemsetAsync(ts->ntri, 0, (size_t) N * 4, s));
  LA3G_CUDA(cudaMemsetAsync(ts->total, 0, 8, s));
  LA3G_CUDA(cudaMemsetAsync(ts->next, 0, 16, s));
  if (ts->nmid)
  {
    // list reads (N+(x) once, N+(y) per oriented edge) + the x's two offsets
    ProfileScope p("tc_rank_mid", s, 4.0 * ts->work_mid + 8.0 * ts->nmid);
    k_tc_rank_block<kTcCap, 256, 32><<<kSMs * 8, 256, 0, s>>>(ts->plus_ptr, ts->plus_col, ts->order_mid, ts->nmid,
                                                              ts->next + 1, ts->ntri, kTcWalkFactor);
    LA3G_LAUNCHED();
  }
  if (ts->norder)
  {
    ProfileScope p("tc_rank", s, 4.0 * (ts->work - ts->work_mid - ts->work_big) + 8.0 * ts->norder);
    // short lists: the flattened walk keeps all 32 lanes busy across the y's
    k_tc_rank_flat<kTcSmall, 8><<<kSMs * 8, 8 * 32, 0, s>>>(ts->plus_ptr, ts->plus_col, ts->order, ts->norder, ts->next,
                                                            ts->ntri);
    LA3G_LAUNCHED();
  }
  if (ts->nhubs)
  {
    // the walked part of N+(x) of every hub pair + each hub's N+(y) once + the
    // pair's x, index and two offsets
    ProfileScope p("tc_hub", s, 4.0 * ts->hub_items + 4.0 * ts->hub_lists + 16.0 * (double) ts->hub_pairs);
    k_tc_hub<kTcHubCap, 256, kTcHubLanes><<<kSMs * 6, 256, 0, s>>>(ts->plus_ptr, ts->plus_col_r, ts->hubs, ts->nhubs,
                                                      ts->hub_ptr, ts->hub_x, ts->hub_j, ts->next + 2, ts->ntri);
    LA3G_LAUNCHED();
  }
  if (ts->nbig)
  {
    k_tc_rank_big<<<grid_for((uint64_t) ts->nbig * 32, 256), 256, 0, s>>>(ts->plus_ptr, ts->plus_col, ts->big, ts->nbig,
                                                                           ts->ntri);
    LA3G_LAUNCHED();
    tls_launches++;
  }
  k_tc_sum<<<grid_for(N, 256), 256, 0, s>>>(N, ts->ntri, ts->total);
  LA3G_LAUNCHED();
  tls_launches++;
  T.device_end();
  unsigned long long total = 0;
  LA3G_CUDA(cudaMemcpyAsync(&total, ts->total, 8, cudaMemcpyDeviceToHost, s));
  if (per_vertex_out) LA3G_CUDA(cudaMemcpyAsync(per_vertex_out, ts->ntri, (size_t) N * 4, cudaMemcpyDeviceToHost, s));
  LA3G_TRY(T.finish());
  if (total_out) *total_out = total;
  if (st)
  {
    st->iterations = 2;
    st->teps_edges = g.nent;
    st->edges_examined = (uint64_t) ts->work;
    st->algo_bytes = (uint64_t) (4.0 * ts->work + 8.0 * N);
  }
  return LA3G_OK;
}
