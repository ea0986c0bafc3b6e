// Triangle counting: the reference tc app (src/apps/graph_analytics/
// tc.cpp:11-52, tc.h:47-99) on the device.
//
// The reference orients every edge from the lower to the higher original id
// (remove_cycles, graph.hpp:174-179), collects for each vertex v the list
// N<(v) of its lower neighbours (GnVertex, pass 1), and for every oriented
// edge (u, v), u < v, adds |N<(u) ∩ N<(v)| to u, accumulating in uint32
// (CtVertex, pass 2).  Each triangle a < b < c is therefore counted once, at
// its middle vertex b.  Both passes are inside the reference's timed window,
// and both are inside every call here.
//
// Here every triangle is found once by degree ordering instead, and counted
// at the middle vertex BY ID (the median of its three ids), which gives the
// reference's per-vertex counts (sums are order-free, uint32 wraps alike):
//
//   rank(v) = position of v after sorting by (undirected degree, position);
//   N+(x)   = neighbours of higher rank, kept as ranks, each row ascending;
//   a triangle x < y < w in rank order has y, w in N+(x) and w in N+(y),
//   and w lies in the part of N+(x) ranked above y (a suffix of the row).
//
// Pass 1 (list building, every call): degrees, ranks (one radix sort of the
// vertices), N+ rows by an edge-parallel count / scan / fill, a segmented
// sort of the rows, and the transposed pair lists: for each y the pairs
// (x, start of the suffix of N+(x) after y), i.e. every oriented edge once.
//
// Pass 2 (counting) is y-centric: a task is a vertex y and a slice of its
// pairs; N+(y) goes into a shared-memory hash table (rank -> index, at least
// four slots per element) with the ids of its elements, and a warp walks the
// suffixes of 32 pairs at a time concatenated, 64 list elements per step,
// each probed in the table; an element's pair is found from the window's
// pair-start bits (one OR-reduction) and its address by a shuffle from the
// pair's lane.  A hit w closes {x, y, w}; its middle id takes the count: x
// in a per-pair shared counter, y in a register, w in a shared counter per
// element of N+(y); all are flushed once per round or task.  On R-MAT this
// walks the shorter side of almost every pair (the suffix), and the lists
// stay L2-resident.  N+(y) up to kTcWarpCap: one warp per task; longer: one
// block per task with a block-wide table, its warps taking the rounds from a
// shared counter; beyond kTcBlockCap (no such rows on R-MAT up to scale 24):
// a binary search in the sorted row in global memory.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_segmented_sort.cuh>

#include "la3g_internal.h"

namespace la3g {

static constexpr uint32_t kTcEdgesPerThread = 8;  // edge-parallel passes: contiguous edges per thread
static constexpr uint32_t kTcWarpCap = 128;       // |N+(y)| up to this: a warp per task
static constexpr uint32_t kTcWarpSlots = 512;     // hash slots of a warp table (>= 4 kTcWarpCap)
static constexpr uint32_t kTcWarpPairs = 256;     // pairs per warp task
static constexpr uint32_t kTcMidCap = 512;        // |N+(y)| up to this: a small block per task
static constexpr uint32_t kTcMidSlots = 2048;     // hash slots of its table (>= 4 kTcMidCap)
static constexpr uint32_t kTcBlockCap = 2048;     // |N+(y)| up to this: a large block table; longer: global search
static constexpr uint32_t kTcBlockSlots = 8192;   // hash slots of a large block table (>= 4 kTcBlockCap)
static constexpr uint32_t kTcBlockPairs = 1024;   // pairs per block task (both block sizes; R-MAT s20 call: 4096 4.96 ms, 2048 4.83, 1024 4.73, 512 4.74, 256 5.01)
static constexpr int kTcWarpKernelWarps = 8;
static constexpr int kTcMidThreads = 256;
static constexpr int kTcBlockThreads = 512;
static constexpr uint32_t kTcSortWarpCap = 1024;  // N+ rows up to this are sorted by one warp
static constexpr uint32_t kTcSortBlockCap = 16384;  // ... up to this by one block; longer: library sort
static constexpr uint32_t kEmpty = 0xFFFFFFFFu;
static constexpr int kTcCounters = 12;

struct TcScratch
{
  uint32_t N = 0;
  uint64_t m = 0;
  uint32_t* deg = nullptr;          // [N] undirected degree by position
  uint32_t* iota = nullptr;         // [N] 0..N-1
  uint32_t* deg_of_rank = nullptr;  // [N]
  uint32_t* pos_of_rank = nullptr;  // [N]
  uint32_t* rank_of_pos = nullptr;  // [N]
  uint32_t* id_of_rank = nullptr;   // [N]
  uint32_t* dplus = nullptr;        // [N + 1] |N+| by rank, then the row offsets' input
  uint32_t* pptr = nullptr;         // [N + 1] N+ row offsets (rows = ranks)
  uint32_t* fill = nullptr;         // [N] fill cursors
  uint32_t* pcol_raw = nullptr;     // [m] N+ rows as filled (ranks)
  uint32_t* pcol = nullptr;         // [m] N+ rows, each ascending
  uint32_t* mcount = nullptr;       // [N + 1] pairs per y
  uint32_t* mptr = nullptr;         // [N + 1] pair offsets per y
  uint2* pairs = nullptr;           // [m] (suffix start in pcol, x) grouped by y
  unsigned long long* tcount = nullptr;  // [N + 1] tasks per y: small block << 32 | warp
  unsigned long long* toff = nullptr;    // [N + 1] their exclusive sums
  uint32_t* tcount2 = nullptr;      // [N + 1] large-block tasks per y
  uint32_t* toff2 = nullptr;        // [N + 1] their exclusive sums
  uint2* wtasks = nullptr;          // (y, first pair) of the warp tasks
  uint2* mtasks = nullptr;          // ... of the small-block tasks
  uint2* btasks = nullptr;          // ... and of the large-block tasks
  uint32_t* ntri = nullptr;         // [N] by id
  uint32_t* big_rows = nullptr;     // [N] N+ rows too long for a warp's sort
  // [0] warp-task cursor [1] large-block-task cursor [2] walked [3] table
  // builds [4] triangles [5] self-check failures [6] big rows [7] rows too
  // long for the block sort [8] small-block-task cursor
  unsigned long long* ctr = nullptr;
  unsigned long long* hctr = nullptr;  // pinned mirror
  void* temp = nullptr;
  size_t temp_bytes = 0;
  void* seg_temp = nullptr;         // the library segmented sort's storage (oversize rows only)
  size_t seg_bytes = 0;
  int end_bit = 32;
};

static void tc_scratch_free(void* p)
{
  TcScratch* s = (TcScratch*) p;
  if (s->hctr) cudaFreeHost(s->hctr);
  delete s;
}

// ---------------------------------------------------------------- pass 1

__global__ void k_tc_deg(const uint32_t* __restrict__ iptr, const uint32_t* __restrict__ optr, uint32_t N,
                         uint32_t* deg, uint32_t* iota)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x)
  {
    deg[p] = (iptr[p + 1] - iptr[p]) + (optr[p + 1] - optr[p]);
    iota[p] = p;
  }
}

__global__ void k_tc_ranks(uint32_t N, const uint32_t* __restrict__ pos_of_rank, const uint32_t* __restrict__ id_of_pos,
                           uint32_t* rank_of_pos, uint32_t* id_of_rank)
{
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < N; r += gridDim.x * blockDim.x)
  {
    const uint32_t p = pos_of_rank[r];
    rank_of_pos[p] = r;
    id_of_rank[r] = id_of_pos[p];
  }
}

// Row of entry e: the largest r < nrows with ptr[r] <= e (e < ptr[nrows]).
__device__ __forceinline__ uint32_t tc_row_of(const uint32_t* __restrict__ ptr, uint32_t nrows, uint64_t e)
{
  uint32_t lo = 0, hi = nrows;
  while (hi - lo > 1)
  {
    const uint32_t mid = (lo + hi) >> 1;
    if (ptr[mid] <= e) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Every undirected edge once (the pull CSR of the id-oriented graph: row =
// higher id, column = lower id); each thread takes kTcEdgesPerThread
// consecutive entries, so a hub row spreads over many threads.  PLUS = false
// counts |N+| per lower-rank end; PLUS = true writes the higher-rank end into
// the lower end's row.
template <bool FILL>
__global__ void __launch_bounds__(256)
k_tc_orient(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, uint32_t nrows, uint64_t m,
            const uint32_t* __restrict__ rank_of_pos, uint32_t* count_or_fill, const uint32_t* __restrict__ pptr,
            uint32_t* pcol)
{
  const uint64_t e0 = ((uint64_t) blockIdx.x * blockDim.x + threadIdx.x) * kTcEdgesPerThread;
  if (e0 >= m) return;
  const uint64_t e1 = min(e0 + kTcEdgesPerThread, m);
  uint32_t r = tc_row_of(ptr, nrows, e0);
  uint32_t rr = rank_of_pos[r];
  uint64_t rend = ptr[r + 1];
  for (uint64_t e = e0; e < e1; e++)
  {
    if (e >= rend)  // the next non-empty row (runs of empty rows are skipped by the search)
    {
      r = tc_row_of(ptr, nrows, e);
      rr = rank_of_pos[r];
      rend = ptr[r + 1];
    }
    const uint32_t ru = rank_of_pos[col[e]];
    const uint32_t lo = min(rr, ru), hi = max(rr, ru);
    if (FILL) pcol[pptr[lo] + atomicAdd(&count_or_fill[lo], 1u)] = hi;
    else atomicAdd(&count_or_fill[lo], 1u);
  }
}

// Pairs per y (a y with an empty N+(y) closes no triangle as the middle
// rank) and the tasks they form.
__global__ void k_tc_pair_counts(uint32_t N, const uint32_t* __restrict__ pptr, const uint32_t* __restrict__ deg_of_rank,
                                 uint32_t* mcount, unsigned long long* tcount, uint32_t* tcount2)
{
  for (uint32_t y = blockIdx.x * blockDim.x + threadIdx.x; y <= N; y += gridDim.x * blockDim.x)
  {
    uint32_t c = 0, t2 = 0;
    unsigned long long t = 0;
    if (y < N)
    {
      const uint32_t dp = pptr[y + 1] - pptr[y];
      c = dp ? deg_of_rank[y] - dp : 0u;
      if (c)
      {
        if (dp <= kTcWarpCap) t = (c + kTcWarpPairs - 1) / kTcWarpPairs;
        else if (dp <= kTcMidCap) t = (unsigned long long) ((c + kTcBlockPairs - 1) / kTcBlockPairs) << 32;
        else t2 = (c + kTcBlockPairs - 1) / kTcBlockPairs;
      }
    }
    mcount[y] = c;
    tcount[y] = t;
    tcount2[y] = t2;
  }
}

// Index of rank y in the ascending row [b, e) (y is known to be there).
__device__ __forceinline__ uint32_t tc_find_in_row(const uint32_t* __restrict__ pcol, uint32_t b, uint32_t e, uint32_t y)
{
  while (b < e)
  {
    const uint32_t mid = (b + e) >> 1;
    if (pcol[mid] < y) b = mid + 1;
    else e = mid;
  }
  return b;
}

// Pair lists by y, built from each y's own adjacency (its in- and out-rows in
// the id-oriented graph), so that a hub's many pairs come from consecutive
// entries: the lanes of a warp that hold the same y reserve their slots with
// one atomic.  A neighbour x of lower rank gives the pair (s, x), s the
// index after y in the sorted row N+(x).  Thread chunks [0, m8) cover the
// in-rows' m entries, [m8, m8 + m) the out-rows' (m8 = m rounded up to the
// chunk size, so that no chunk straddles the two).
__global__ void __launch_bounds__(256)
k_tc_pairs(const uint32_t* __restrict__ iptr, const uint32_t* __restrict__ icol, const uint32_t* __restrict__ optr,
           const uint32_t* __restrict__ orow, uint32_t nrows, uint32_t N, uint64_t m,
           const uint32_t* __restrict__ rank_of_pos, const uint32_t* __restrict__ pptr,
           const uint32_t* __restrict__ pcol, const uint32_t* __restrict__ mptr, uint32_t* fill, uint2* pairs)
{
  const int lane = threadIdx.x & 31;
  const uint64_t m8 = (m + kTcEdgesPerThread - 1) / kTcEdgesPerThread * kTcEdgesPerThread;
  const uint64_t e0 = ((uint64_t) blockIdx.x * blockDim.x + threadIdx.x) * kTcEdgesPerThread;
  const bool in_part = e0 < m8;
  const uint32_t* ptr = in_part ? iptr : optr;
  const uint32_t* col = in_part ? icol : orow;
  const uint64_t base = in_part ? 0 : m8;
  const uint64_t lim = in_part ? m : m8 + m;
  const bool live = e0 < lim;
  uint32_t r = 0, ry = 0;
  uint64_t rend = 0;
  if (live)
  {
    r = tc_row_of(ptr, in_part ? nrows : N, e0 - base);
    ry = rank_of_pos[r];
    rend = ptr[r + 1] + base;
  }
  for (uint32_t u = 0; u < kTcEdgesPerThread; u++)
  {
    const uint64_t e = e0 + u;
    bool emit = false;
    uint32_t x = 0;
    if (live && e < lim)
    {
      if (e >= rend)  // the next non-empty row (sinks' out-rows are empty, in runs)
      {
        r = tc_row_of(ptr, in_part ? nrows : N, e - base);
        ry = rank_of_pos[r];
        rend = ptr[r + 1] + base;
      }
      x = rank_of_pos[col[e - base]];
      emit = x < ry && pptr[ry + 1] > pptr[ry];
    }
    const unsigned want = __ballot_sync(0xffffffffu, emit);
    if (!want) continue;
    const unsigned grp = __match_any_sync(0xffffffffu, emit ? ry : 0xFFFFFFFFu);
    if (emit)
    {
      const int leader = __ffs(grp) - 1;
      uint32_t slot = 0;
      if (lane == leader) slot = atomicAdd(&fill[ry], (uint32_t) __popc(grp));
      slot = __shfl_sync(grp, slot, leader) + __popc(grp & ((1u << lane) - 1));
      const uint32_t sidx = tc_find_in_row(pcol, pptr[x], pptr[x + 1], ry);
      pairs[mptr[ry] + slot] = make_uint2(sidx + 1, x);
    }
  }
}

__global__ void k_tc_tasks(uint32_t N, const unsigned long long* __restrict__ toff, const uint32_t* __restrict__ toff2,
                           const uint32_t* __restrict__ mptr, uint2* wtasks, uint2* mtasks, uint2* btasks)
{
  for (uint32_t y = blockIdx.x * blockDim.x + threadIdx.x; y < N; y += gridDim.x * blockDim.x)
  {
    const unsigned long long c = toff[y + 1] - toff[y];
    const uint32_t nw = (uint32_t) c, nm = (uint32_t) (c >> 32), nb = toff2[y + 1] - toff2[y];
    const uint32_t wo = (uint32_t) toff[y], mo = (uint32_t) (toff[y] >> 32), bo = toff2[y];
    for (uint32_t k = 0; k < nw; k++) wtasks[wo + k] = make_uint2(y, mptr[y] + k * kTcWarpPairs);
    for (uint32_t k = 0; k < nm; k++) mtasks[mo + k] = make_uint2(y, mptr[y] + k * kTcBlockPairs);
    for (uint32_t k = 0; k < nb; k++) btasks[bo + k] = make_uint2(y, mptr[y] + k * kTcBlockPairs);
  }
}

// ---------------------------------------------------------------- row sort

// Sorts every N+ row ascending (pass 1 fills them in arbitrary order): up to
// 32 elements in a warp's registers (a bitonic network over shuffles), up to
// kTcSortWarpCap in a warp's shared buffer; longer rows are listed for
// k_tc_sort_big.
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
k_tc_sort_rows(const uint32_t* __restrict__ pptr, uint32_t N, const uint32_t* __restrict__ raw, uint32_t* out,
               uint32_t* big_rows, unsigned long long* nbig)
{
  __shared__ uint32_t s_buf[WARPS][kTcSortWarpCap];
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
  uint32_t* buf = s_buf[wi];
  const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t x = gw; x < N; x += nw)
  {
    const uint32_t b = pptr[x], d = pptr[x + 1] - b;
    if (d <= 1)
    {
      if (d == 1 && lane == 0) out[b] = raw[b];
      continue;
    }
    if (d <= 32)
    {
      uint32_t v = (uint32_t) lane < d ? raw[b + lane] : kEmpty;
#pragma unroll
      for (int k = 2; k <= 32; k <<= 1)
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1)
        {
          const uint32_t o = __shfl_xor_sync(0xffffffffu, v, j);
          const bool asc = (lane & k) == 0, low = (lane & j) == 0;
          v = (low == asc) ? min(v, o) : max(v, o);
        }
      if ((uint32_t) lane < d) out[b + lane] = v;
      continue;
    }
    if (d > kTcSortWarpCap)
    {
      if (lane == 0) big_rows[atomicAdd(nbig, 1ull)] = x;
      continue;
    }
    uint32_t n = 64;
    while (n < d) n <<= 1;
    for (uint32_t i = lane; i < n; i += 32) buf[i] = i < d ? raw[b + i] : kEmpty;
    __syncwarp();
    for (uint32_t k = 2; k <= n; k <<= 1)
      for (uint32_t j = k >> 1; j > 0; j >>= 1)
      {
        for (uint32_t q = lane; q < n / 2; q += 32)
        {
          const uint32_t i = 2 * j * (q / j) + (q % j), l = i + j;
          const uint32_t a = buf[i], c = buf[l];
          if ((a > c) == ((i & k) == 0))
          {
            buf[i] = c;
            buf[l] = a;
          }
        }
        __syncwarp();
      }
    for (uint32_t i = lane; i < d; i += 32) out[b + i] = buf[i];
    __syncwarp();
  }
}

// Rows longer than kTcSortWarpCap, one block each, in dynamic shared memory
// (up to kTcSortBlockCap elements); longer ones are counted in *over so that
// the call sorts with the library's segmented sort instead.
__global__ void __launch_bounds__(1024)
k_tc_sort_big(const uint32_t* __restrict__ pptr, const uint32_t* __restrict__ raw, uint32_t* out,
              const uint32_t* __restrict__ big_rows, const unsigned long long* __restrict__ nbig,
              unsigned long long* over)
{
  extern __shared__ uint32_t sbig[];
  const uint32_t nrows = (uint32_t) *nbig;
  for (uint32_t r = blockIdx.x; r < nrows; r += gridDim.x)
  {
    const uint32_t x = big_rows[r];
    const uint32_t b = pptr[x], d = pptr[x + 1] - b;
    if (d > kTcSortBlockCap)
    {
      if (threadIdx.x == 0) atomicAdd(over, 1ull);
      continue;
    }
    uint32_t n = 64;
    while (n < d) n <<= 1;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) sbig[i] = i < d ? raw[b + i] : kEmpty;
    __syncthreads();
    for (uint32_t k = 2; k <= n; k <<= 1)
      for (uint32_t j = k >> 1; j > 0; j >>= 1)
      {
        for (uint32_t q = threadIdx.x; q < n / 2; q += blockDim.x)
        {
          const uint32_t i = 2 * j * (q / j) + (q % j), l = i + j;
          const uint32_t a = sbig[i], c = sbig[l];
          if ((a > c) == ((i & k) == 0))
          {
            sbig[i] = c;
            sbig[l] = a;
          }
        }
        __syncthreads();
      }
    for (uint32_t i = threadIdx.x; i < d; i += blockDim.x) out[b + i] = sbig[i];
    __syncthreads();
  }
}

// ---------------------------------------------------------------- pass 2

__device__ __forceinline__ uint32_t tc_mid3(uint32_t a, uint32_t b, uint32_t c)
{
  return max(min(a, b), min(max(a, b), c));
}

__device__ __forceinline__ uint32_t tc_hash(uint32_t w, int lg) { return (w * 0x9E3779B1u) >> (32 - lg); }

// The table of one task's N+(y): open addressing (rank -> index in the row)
// with at least 4 slots per element, so that nearly every probe ends at its
// first slot; the ids of the row's elements (lid) and one counter per
// element (cn).
template <class IDX>
struct TcTable
{
  const uint32_t* key;
  const IDX* idx;
  const uint32_t* lid;
  uint32_t* cn;
  uint32_t mask;
  int lg;
};

// Per-warp round state (shared memory): the compacted pairs' (suffix start
// minus walk offset), walk offset and x id, and the triangles counted at
// each pair's x.
struct TcRound
{
  uint32_t so[32];
  uint32_t off[32];
  uint32_t xid[32];
  uint32_t cx[32];
};

// Counts the element w (of the suffix of the pair at lane k of this round)
// against N+(y): a hit closes {x, y, w}; its middle id takes the count - x
// in the round's cx[k], y in cy, w in cn[j].  SEARCH: N+(y) too long for a
// table, binary search in the sorted global row, w's count straight to ntri.
template <class IDX, bool SEARCH>
__device__ __forceinline__ void tc_probe(uint32_t w, uint32_t k, uint32_t xo, uint32_t yid, const TcTable<IDX>& T,
                                         const uint32_t* __restrict__ row, uint32_t d,
                                         const uint32_t* __restrict__ id_of_rank, TcRound& R, uint32_t& cy,
                                         uint32_t* ntri)
{
  if (w == kEmpty) return;
  int j = -1;
  if (SEARCH)
  {
    uint32_t lo = 0, hi = d;
    while (lo < hi)
    {
      const uint32_t mid = (lo + hi) >> 1;
      if (row[mid] < w) lo = mid + 1;
      else hi = mid;
    }
    if (lo < d && row[lo] == w) j = (int) lo;
  }
  else
  {
    uint32_t sl = tc_hash(w, T.lg), kk = T.key[sl];
    while (kk != w && kk != kEmpty)
    {
      sl = (sl + 1) & T.mask;
      kk = T.key[sl];
    }
    if (kk == w) j = T.idx[sl];
  }
  if (j < 0) return;
  const uint32_t wid = SEARCH ? id_of_rank[w] : T.lid[j];
  const uint32_t mid = tc_mid3(xo, yid, wid);
  cy += mid == yid;
  uint32_t* const at_w = SEARCH ? &ntri[wid] : &T.cn[j];
  if (mid != yid) atomicAdd(mid == xo ? &R.cx[k] : at_w, 1u);
}

// One warp walks one round: pairs [p0, p1) (at most 32) of y.  The pairs'
// suffixes are concatenated and read 64 elements per step (two 32-element
// windows whose loads are in flight together).  Element t belongs to the
// compacted pair k whose walk offset is the last at or below t: k = (pairs
// started before the window) + (pairs starting in the window at or below
// the lane) - 1, from one OR-reduction of the window's start bits; the
// owner's (start - offset) and x id come from its lane by shuffle, so the
// address of element t is so[k] + t.
template <class IDX, bool SEARCH>
__device__ __forceinline__ void tc_round(uint32_t p0, uint32_t p1, const uint2* __restrict__ pairs,
                                         const uint32_t* __restrict__ pptr, const uint32_t* __restrict__ pcol,
                                         const uint32_t* __restrict__ id_of_rank, uint32_t yid, const TcTable<IDX>& T,
                                         const uint32_t* __restrict__ row, uint32_t d, TcRound& R, uint32_t& cy,
                                         unsigned long long& walked, uint32_t* ntri, unsigned long long* err)
{
  const uint32_t lane = threadIdx.x & 31;
  const unsigned full = 0xffffffffu;
  const unsigned lt = (1u << lane) - 1, le = lane == 31 ? full : ((2u << lane) - 1);
  const uint32_t p = p0 + lane;
  uint32_t s = 0, L = 0, xid = 0;
  if (p < p1)
  {
    const uint2 px = pairs[p];
    s = px.x;
    L = pptr[px.y + 1] - s;
    xid = id_of_rank[px.y];
  }
  const unsigned nz = __ballot_sync(full, L > 0);
  uint32_t incl = L;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    const uint32_t v = __shfl_up_sync(full, incl, o);
    if (lane >= (uint32_t) o) incl += v;
  }
  const uint32_t total = __shfl_sync(full, incl, 31);
  if (L > 0)
  {
    const uint32_t k = __popc(nz & lt);
    R.so[k] = s - (incl - L);
    R.off[k] = incl - L;
    R.xid[k] = xid;
  }
  __syncwarp();
  const uint32_t np = __popc(nz);
  // lane k holds the k-th compacted pair
  const uint32_t pk = lane < np ? R.off[lane] : kEmpty;
  const uint32_t my_so = lane < np ? R.so[lane] : 0u;
  const uint32_t my_x = lane < np ? R.xid[lane] : 0u;
  R.cx[lane] = 0;
  __syncwarp();
  uint32_t before = 0;
  bool slip = false;
  for (uint32_t w0 = 0; w0 < total; w0 += 64)
  {
    const uint32_t ra = pk - w0, rb = pk - (w0 + 32);
    const unsigned sa = __reduce_or_sync(full, ra < 32 ? 1u << ra : 0u);
    const unsigned sb = __reduce_or_sync(full, rb < 32 ? 1u << rb : 0u);
    const uint32_t ka = (before + __popc(sa & le) - 1u) & 31u;
    before += __popc(sa);
    const uint32_t kb = (before + __popc(sb & le) - 1u) & 31u;
    before += __popc(sb);
    const uint32_t ta = w0 + lane, tb = ta + 32;
    const uint32_t soa = __shfl_sync(full, my_so, ka), sob = __shfl_sync(full, my_so, kb);
    const uint32_t xa = __shfl_sync(full, my_x, ka), xb = __shfl_sync(full, my_x, kb);
    // by construction every element below total has an owner in this round;
    // checked all the same, so that a slip reads nothing outside the lists
    const bool va = ta < total, vb = tb < total;
    slip |= (va && ka >= np) || (vb && kb >= np);
    const uint32_t wa = (va && ka < np) ? pcol[soa + ta] : kEmpty;
    const uint32_t wb = (vb && kb < np) ? pcol[sob + tb] : kEmpty;
    tc_probe<IDX, SEARCH>(wa, ka, xa, yid, T, row, d, id_of_rank, R, cy, ntri);
    tc_probe<IDX, SEARCH>(wb, kb, xb, yid, T, row, d, id_of_rank, R, cy, ntri);
  }
  if (slip) atomicAdd(err, 1ull);
  walked += total;
  __syncwarp();
  if (lane < np && R.cx[lane]) atomicAdd(&ntri[my_x], R.cx[lane]);
  __syncwarp();
}

// Builds the table of N+(y) (d elements at row) with `nthreads` threads
// starting at thread `tid`; the caller clears the keys and synchronises
// before and after.
template <class IDX>
__device__ __forceinline__ void tc_build(const uint32_t* __restrict__ row, uint32_t d, int lg,
                                         const uint32_t* __restrict__ id_of_rank, uint32_t* key, IDX* idx,
                                         uint32_t* lid, uint32_t* cn, uint32_t tid, uint32_t nthreads)
{
  const uint32_t mask = (1u << lg) - 1;
  for (uint32_t j = tid; j < d; j += nthreads)
  {
    const uint32_t w = row[j];
    lid[j] = id_of_rank[w];
    cn[j] = 0;
    uint32_t sl = tc_hash(w, lg);
    while (atomicCAS(&key[sl], kEmpty, w) != kEmpty) sl = (sl + 1) & mask;
    idx[sl] = (IDX) j;
  }
}

// log2 of the table size: at least 4 slots per element, at least 32 slots.
__device__ __forceinline__ int tc_lg(uint32_t d)
{
  int lg = 5;
  while ((1u << lg) < 4 * d) lg++;
  return lg;
}

// Warp tasks: |N+(y)| <= kTcWarpCap, one table per warp in static shared
// memory (indices fit a byte), rounds of 32 pairs in turn.
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32, 5)
k_tc_count_warp(const uint32_t* __restrict__ pptr, const uint32_t* __restrict__ pcol, const uint2* __restrict__ pairs,
                const uint32_t* __restrict__ mptr, const uint2* __restrict__ tasks,
                const uint32_t* __restrict__ ntasks_ptr, const uint32_t* __restrict__ id_of_rank,
                uint32_t* ntri, unsigned long long* ctr)
{
  __shared__ uint32_t s_key[WARPS][kTcWarpSlots];
  __shared__ uint8_t s_idx[WARPS][kTcWarpSlots];
  __shared__ uint32_t s_lid[WARPS][kTcWarpCap];
  __shared__ uint32_t s_cn[WARPS][kTcWarpCap];
  __shared__ TcRound s_r[WARPS];
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
  uint32_t* key = s_key[wi];
  uint8_t* idx = s_idx[wi];
  uint32_t* lid = s_lid[wi];
  uint32_t* cn = s_cn[wi];
  const uint32_t ntasks = *ntasks_ptr;
  unsigned long long walked = 0, built = 0;
  for (;;)
  {
    uint32_t t = 0;
    if (lane == 0) t = (uint32_t) atomicAdd(&ctr[0], 1ull);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= ntasks) break;
    const uint2 tk = tasks[t];
    const uint32_t y = tk.x, p0 = tk.y, p1 = min(p0 + kTcWarpPairs, mptr[y + 1]);
    const uint32_t yb = pptr[y], d = pptr[y + 1] - yb;
    if (d == 0 || d > kTcWarpCap) continue;  // not a warp task (never built so)
    const int lg = tc_lg(d);
    for (uint32_t i = lane; i < (1u << lg); i += 32) key[i] = kEmpty;
    __syncwarp();
    tc_build<uint8_t>(pcol + yb, d, lg, id_of_rank, key, idx, lid, cn, lane, 32);
    __syncwarp();
    built += d;
    const TcTable<uint8_t> T{key, idx, lid, cn, (1u << lg) - 1, lg};
    const uint32_t yid = id_of_rank[y];
    uint32_t cy = 0;
    for (uint32_t q = p0; q < p1; q += 32)
      tc_round<uint8_t, false>(q, min(q + 32u, p1), pairs, pptr, pcol, id_of_rank, yid, T, nullptr, d, s_r[wi], cy,
                               walked, ntri, ctr + 5);
    for (int o = 16; o > 0; o >>= 1) cy += __shfl_xor_sync(0xffffffffu, cy, o);
    if (lane == 0 && cy) atomicAdd(&ntri[yid], cy);
    __syncwarp();
    for (uint32_t j = lane; j < d; j += 32)
      if (cn[j]) atomicAdd(&ntri[lid[j]], cn[j]);
    __syncwarp();
  }
  if (lane == 0)
  {
    atomicAdd(&ctr[2], walked);
    atomicAdd(&ctr[3], built);
  }
}

// Block tasks: |N+(y)| > kTcWarpCap; one table per block in dynamic shared
// memory (CAP elements, SLOTS slots; rows longer than CAP fall back to a
// global binary search), the warps taking the task's 32-pair rounds from a
// shared counter.  Two sizes: small blocks with small tables for rows up to
// kTcMidCap, so that many tasks run on an SM at once, and large ones.  The
// per-warp round state stays in static shared memory.
template <int THREADS, uint32_t SLOTS, uint32_t CAP, int CURSOR>
__global__ void __launch_bounds__(THREADS, 1536 / THREADS)
k_tc_count_block(const uint32_t* __restrict__ pptr, const uint32_t* __restrict__ pcol, const uint2* __restrict__ pairs,
                 const uint32_t* __restrict__ mptr, const uint2* __restrict__ tasks,
                 const uint32_t* __restrict__ ntasks_ptr, const uint32_t* __restrict__ id_of_rank,
                 uint32_t* ntri, unsigned long long* ctr)
{
  constexpr int WARPS = THREADS / 32;
  extern __shared__ __align__(16) uint32_t tc_smem[];
  uint32_t* key = tc_smem;                          // [SLOTS]
  uint32_t* lid = key + SLOTS;                      // [CAP]
  uint32_t* cn = lid + CAP;                         // [CAP]
  uint16_t* idx = (uint16_t*) (cn + CAP);           // [SLOTS]
  __shared__ TcRound s_r[WARPS];
  __shared__ uint32_t s_t, s_cy, s_round;
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
  const uint32_t ntasks = *ntasks_ptr;
  unsigned long long walked = 0, built = 0;
  for (;;)
  {
    if (threadIdx.x == 0)
    {
      s_t = (uint32_t) atomicAdd(&ctr[CURSOR], 1ull);
      s_cy = 0;
      s_round = 0;
    }
    __syncthreads();
    const uint32_t t = s_t;
    if (t >= ntasks) break;
    const uint2 tk = tasks[t];
    const uint32_t y = tk.x, p0 = tk.y, p1 = min(p0 + kTcBlockPairs, mptr[y + 1]);
    const uint32_t yb = pptr[y], d = pptr[y + 1] - yb;
    const bool search = d > CAP;
    const int lg = search ? 5 : tc_lg(d);
    if (!search)
    {
      for (uint32_t i = threadIdx.x; i < (1u << lg); i += THREADS) key[i] = kEmpty;
      __syncthreads();
      tc_build<uint16_t>(pcol + yb, d, lg, id_of_rank, key, idx, lid, cn, threadIdx.x, THREADS);
      if (threadIdx.x == 0) built += d;
    }
    __syncthreads();
    const TcTable<uint16_t> T{key, idx, lid, cn, (1u << lg) - 1, lg};
    const uint32_t yid = id_of_rank[y];
    uint32_t cy = 0;
    for (;;)
    {
      uint32_t r = 0;
      if (lane == 0) r = atomicAdd(&s_round, 1u);
      r = __shfl_sync(0xffffffffu, r, 0);
      const uint32_t q = p0 + 32u * r;
      if (q >= p1) break;
      if (search)
        tc_round<uint16_t, true>(q, min(q + 32u, p1), pairs, pptr, pcol, id_of_rank, yid, T, pcol + yb, d, s_r[wi],
                                 cy, walked, ntri, ctr + 5);
      else
        tc_round<uint16_t, false>(q, min(q + 32u, p1), pairs, pptr, pcol, id_of_rank, yid, T, nullptr, d, s_r[wi],
                                  cy, walked, ntri, ctr + 5);
    }
    for (int o = 16; o > 0; o >>= 1) cy += __shfl_xor_sync(0xffffffffu, cy, o);
    if (lane == 0 && cy) atomicAdd(&s_cy, cy);
    __syncthreads();
    if (threadIdx.x == 0 && s_cy) atomicAdd(&ntri[yid], s_cy);
    if (!search)
      for (uint32_t j = threadIdx.x; j < d; j += THREADS)
        if (cn[j]) atomicAdd(&ntri[lid[j]], cn[j]);
    __syncthreads();
  }
  // every lane of a warp holds the warp's walked count
  if (lane == 0 && walked) atomicAdd(&ctr[2], walked);
  if (threadIdx.x == 0 && built) atomicAdd(&ctr[3], built);
}

static constexpr size_t kTcBlockSmem = (size_t) kTcBlockSlots * 4 + 2 * (size_t) kTcBlockCap * 4 +
                                       (size_t) kTcBlockSlots * 2;
static constexpr size_t kTcMidSmem = (size_t) kTcMidSlots * 4 + 2 * (size_t) kTcMidCap * 4 + (size_t) kTcMidSlots * 2;
#define TC_MID_KERNEL k_tc_count_block<kTcMidThreads, kTcMidSlots, kTcMidCap, 8>
#define TC_BIG_KERNEL k_tc_count_block<kTcBlockThreads, kTcBlockSlots, kTcBlockCap, 1>
static constexpr size_t kTcSortBigSmem = (size_t) kTcSortBlockCap * 4;

__global__ void k_tc_sum(uint32_t N, const uint32_t* __restrict__ ntri, unsigned long long* total)
{
  unsigned long long s = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x) s += ntri[v];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(total, s);
}

static int tc_scratch(la3g_graph* G, TcScratch** out)
{
  TcScratch* ts = (TcScratch*) G->slot[kSlotTc];
  if (ts) { *out = ts; return LA3G_OK; }
  ts = new (std::nothrow) TcScratch();
  if (!ts) return set_error(LA3G_ENOMEM, "out of host memory");
  G->slot[kSlotTc] = ts;
  G->slot_free[kSlotTc] = tc_scratch_free;
  const uint32_t N = G->g.nslots;
  const uint64_t m = G->g.nent;
  ts->N = N;
  ts->m = m;
  LA3G_TRY(galloc(G, &ts->deg, N));
  LA3G_TRY(galloc(G, &ts->iota, N));
  LA3G_TRY(galloc(G, &ts->deg_of_rank, N));
  LA3G_TRY(galloc(G, &ts->pos_of_rank, N));
  LA3G_TRY(galloc(G, &ts->rank_of_pos, N));
  LA3G_TRY(galloc(G, &ts->id_of_rank, N));
  LA3G_TRY(galloc(G, &ts->dplus, (size_t) N + 1));
  LA3G_TRY(galloc(G, &ts->pptr, (size_t) N + 1));
  LA3G_TRY(galloc(G, &ts->fill, N));
  LA3G_TRY(galloc(G, &ts->pcol_raw, m + 1));
  LA3G_TRY(galloc(G, &ts->pcol, m + 1));
  LA3G_TRY(galloc(G, &ts->mcount, (size_t) N + 1));
  LA3G_TRY(galloc(G, &ts->mptr, (size_t) N + 1));
  LA3G_TRY(galloc(G, &ts->pairs, m + 1));
  LA3G_TRY(galloc(G, &ts->tcount, (size_t) N + 1));
  LA3G_TRY(galloc(G, &ts->toff, (size_t) N + 1));
  LA3G_TRY(galloc(G, &ts->tcount2, (size_t) N + 1));
  LA3G_TRY(galloc(G, &ts->toff2, (size_t) N + 1));
  LA3G_TRY(galloc(G, &ts->wtasks, m / kTcWarpPairs + N + 1));
  LA3G_TRY(galloc(G, &ts->mtasks, m / kTcBlockPairs + N + 1));
  LA3G_TRY(galloc(G, &ts->btasks, m / kTcBlockPairs + N + 1));
  LA3G_TRY(galloc(G, &ts->ntri, N));
  LA3G_TRY(galloc(G, &ts->big_rows, N));
  LA3G_TRY(galloc(G, &ts->ctr, kTcCounters));
  LA3G_CUDA(cudaHostAlloc(&ts->hctr, kTcCounters * sizeof(unsigned long long), cudaHostAllocDefault));
  // degrees are at most N - 1: the rank sort needs bit_width(N) key bits
  ts->end_bit = 1;
  while (ts->end_bit < 32 && ((uint64_t) N >> ts->end_bit) != 0) ts->end_bit++;
  size_t a = 0, b = 0, c = 0;
  LA3G_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, a, ts->deg, ts->deg_of_rank, ts->iota, ts->pos_of_rank, (int) N, 0,
                                            ts->end_bit));
  LA3G_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, b, ts->dplus, ts->pptr, (int) N + 1));
  LA3G_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, c, ts->tcount, ts->toff, (int) N + 1));
  size_t c2 = 0;
  LA3G_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, c2, ts->tcount2, ts->toff2, (int) N + 1));
  ts->temp_bytes = std::max(std::max(a, b), std::max(c, c2));
  LA3G_TRY(galloc_bytes(G, &ts->temp, ts->temp_bytes));
  *out = ts;
  return LA3G_OK;
}

// Pass 1: the rank-ordered N+ rows and the per-y pair lists and tasks.
// library_sort: sort the rows with the library's segmented sort (for rows
// longer than kTcSortBlockCap, which this build's sort kernels leave).
static int tc_lists(la3g_graph* G, TcScratch* ts, bool library_sort)
{
  DevGraph& g = G->g;
  cudaStream_t s = G->stream;
  const uint32_t N = ts->N;
  const uint64_t m = ts->m;
  const unsigned eblocks = (unsigned) std::max<uint64_t>(1, (m + 256ull * kTcEdgesPerThread - 1) /
                                                                (256ull * kTcEdgesPerThread));
  size_t tb = ts->temp_bytes;
  LA3G_CUDA(cudaMemsetAsync(ts->dplus, 0, ((size_t) N + 1) * 4, s));
  LA3G_CUDA(cudaMemsetAsync(ts->fill, 0, (size_t) N * 4, s));
  LA3G_CUDA(cudaMemsetAsync(ts->ctr, 0, kTcCounters * sizeof(unsigned long long), s));
  k_tc_deg<<<grid_for(N, 256), 256, 0, s>>>(g.in_ptr, g.out_ptr, N, ts->deg, ts->iota);
  LA3G_LAUNCHED();
  LA3G_CUDA(cub::DeviceRadixSort::SortPairs(ts->temp, tb, ts->deg, ts->deg_of_rank, ts->iota, ts->pos_of_rank, (int) N,
                                            0, ts->end_bit, s));
  k_tc_ranks<<<grid_for(N, 256), 256, 0, s>>>(N, ts->pos_of_rank, g.id_of_pos, ts->rank_of_pos, ts->id_of_rank);
  LA3G_LAUNCHED();
  tls_launches += 2;
  if (m)
  {
    k_tc_orient<false><<<eblocks, 256, 0, s>>>(g.in_ptr, g.in_col, g.nrows(), m, ts->rank_of_pos, ts->dplus, nullptr,
                                               nullptr);
    LA3G_LAUNCHED();
    tls_launches++;
  }
  tb = ts->temp_bytes;
  LA3G_CUDA(cub::DeviceScan::ExclusiveSum(ts->temp, tb, ts->dplus, ts->pptr, (int) N + 1, s));
  if (m)
  {
    k_tc_orient<true><<<eblocks, 256, 0, s>>>(g.in_ptr, g.in_col, g.nrows(), m, ts->rank_of_pos, ts->fill, ts->pptr,
                                              ts->pcol_raw);
    LA3G_LAUNCHED();
    tls_launches++;
    if (library_sort)
    {
      if (!ts->seg_temp)
      {
        LA3G_CUDA(cub::DeviceSegmentedSort::SortKeys(nullptr, ts->seg_bytes, ts->pcol_raw, ts->pcol, (int64_t) m,
                                                     (int64_t) N, ts->pptr, ts->pptr + 1, s));
        LA3G_TRY(galloc_bytes(G, &ts->seg_temp, ts->seg_bytes));
      }
      tb = ts->seg_bytes;
      LA3G_CUDA(cub::DeviceSegmentedSort::SortKeys(ts->seg_temp, tb, ts->pcol_raw, ts->pcol, (int64_t) m, (int64_t) N,
                                                   ts->pptr, ts->pptr + 1, s));
    }
    else
    {
      k_tc_sort_rows<8><<<num_sms() * 8, 256, 0, s>>>(ts->pptr, N, ts->pcol_raw, ts->pcol, ts->big_rows, ts->ctr + 6);
      LA3G_LAUNCHED();
      k_tc_sort_big<<<num_sms(), 1024, kTcSortBigSmem, s>>>(ts->pptr, ts->pcol_raw, ts->pcol, ts->big_rows, ts->ctr + 6,
                                                       ts->ctr + 7);
      LA3G_LAUNCHED();
      tls_launches += 2;
    }
  }
  k_tc_pair_counts<<<grid_for((uint64_t) N + 1, 256), 256, 0, s>>>(N, ts->pptr, ts->deg_of_rank, ts->mcount,
                                                                   ts->tcount, ts->tcount2);
  LA3G_LAUNCHED();
  tls_launches++;
  tb = ts->temp_bytes;
  LA3G_CUDA(cub::DeviceScan::ExclusiveSum(ts->temp, tb, ts->mcount, ts->mptr, (int) N + 1, s));
  tb = ts->temp_bytes;
  LA3G_CUDA(cub::DeviceScan::ExclusiveSum(ts->temp, tb, ts->tcount, ts->toff, (int) N + 1, s));
  tb = ts->temp_bytes;
  LA3G_CUDA(cub::DeviceScan::ExclusiveSum(ts->temp, tb, ts->tcount2, ts->toff2, (int) N + 1, s));
  if (m)
  {
    LA3G_CUDA(cudaMemsetAsync(ts->fill, 0, (size_t) N * 4, s));
    const uint64_t m8 = (m + kTcEdgesPerThread - 1) / kTcEdgesPerThread * kTcEdgesPerThread;
    const unsigned pblocks = (unsigned) ((m8 + m + 256ull * kTcEdgesPerThread - 1) / (256ull * kTcEdgesPerThread));
    k_tc_pairs<<<pblocks, 256, 0, s>>>(g.in_ptr, g.in_col, g.out_ptr, g.out_row, g.nrows(), N, m, ts->rank_of_pos,
                                       ts->pptr, ts->pcol, ts->mptr, ts->fill, ts->pairs);
    LA3G_LAUNCHED();
    tls_launches++;
  }
  k_tc_tasks<<<grid_for(N, 256), 256, 0, s>>>(N, ts->toff, ts->toff2, ts->mptr, ts->wtasks, ts->mtasks, ts->btasks);
  LA3G_LAUNCHED();
  tls_launches++;
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
  if (g.nent >= 0xFFFFFFFFull) return set_error(LA3G_EINVAL, "tc: more than 2^32 - 2 edges");
  CallTimer T(G, st);
  LA3G_TRY(build_push_csr(G));
  TcScratch* ts = nullptr;
  LA3G_TRY(tc_scratch(G, &ts));
  static bool smem_set = false;  // the opt-ins are per function and device; idempotent
  if (!smem_set)
  {
    LA3G_CUDA(cudaFuncSetAttribute(TC_BIG_KERNEL, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) kTcBlockSmem));
    LA3G_CUDA(cudaFuncSetAttribute(TC_MID_KERNEL, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) kTcMidSmem));
    LA3G_CUDA(cudaFuncSetAttribute(k_tc_sort_big, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) kTcSortBigSmem));
    smem_set = true;
  }
  cudaStream_t s = G->stream;
  const uint32_t N = g.nslots;
  const double m = (double) g.nent;
  // rows longer than the block sort's capacity (none on R-MAT up to scale
  // 24): the whole call runs again with the library's segmented sort
  for (int attempt = 0; attempt < 2; attempt++)
  {
    T.device_begin();
    {
      // pass 1: degrees, ranks, N+ rows (count, fill, sort), pair lists,
      // tasks; compulsory bytes: the edge list read by the count and fill
      // passes, the rows written, sorted (read + write), the adjacency read
      // once more for the pair lists (8 B per pair), plus the per-vertex
      // arrays (about 48 B per vertex)
      ProfileScope p("tc_lists", s, 4.0 * m + 8.0 * m + 8.0 * m + 8.0 * m + 8.0 * m + 48.0 * N);
      LA3G_TRY(tc_lists(G, ts, attempt == 1));
    }
    LA3G_CUDA(cudaMemsetAsync(ts->ntri, 0, (size_t) N * 4, s));
    {
      // pass 2; its bytes (walked list elements, pairs, tables) are added below
      ProfileScope p("tc_count", s, 0.0);
      // task counts on the device: warp and small-block counts are the two
      // halves of the packed total (little-endian), large-block the other
      const uint32_t* nw = (const uint32_t*) (ts->toff + N);
      k_tc_count_warp<kTcWarpKernelWarps><<<num_sms() * 5, kTcWarpKernelWarps * 32, 0, s>>>(
          ts->pptr, ts->pcol, ts->pairs, ts->mptr, ts->wtasks, nw, ts->id_of_rank, ts->ntri, ts->ctr);
      LA3G_LAUNCHED();
      TC_MID_KERNEL<<<num_sms() * 8, kTcMidThreads, kTcMidSmem, s>>>(ts->pptr, ts->pcol, ts->pairs, ts->mptr, ts->mtasks,
                                                                 nw + 1, ts->id_of_rank, ts->ntri, ts->ctr);
      LA3G_LAUNCHED();
      TC_BIG_KERNEL<<<num_sms() * 3, kTcBlockThreads, kTcBlockSmem, s>>>(ts->pptr, ts->pcol, ts->pairs, ts->mptr,
                                                                     ts->btasks, ts->toff2 + N, ts->id_of_rank,
                                                                     ts->ntri, ts->ctr);
      LA3G_LAUNCHED();
      tls_launches += 2;
    }
    k_tc_sum<<<grid_for(N, 256), 256, 0, s>>>(N, ts->ntri, ts->ctr + 4);
    LA3G_LAUNCHED();
    tls_launches++;
    T.device_end();
    LA3G_CUDA(cudaMemcpyAsync(ts->hctr, ts->ctr, kTcCounters * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    if (ts->hctr[5]) return set_error(LA3G_ECUDA, "tc: %llu internal consistency checks failed",
                                      (unsigned long long) ts->hctr[5]);
    if (!ts->hctr[7]) break;
  }
  if (per_vertex_out) LA3G_CUDA(cudaMemcpyAsync(per_vertex_out, ts->ntri, (size_t) N * 4, cudaMemcpyDeviceToHost, s));
  LA3G_TRY(T.finish());
  const double walked = (double) ts->hctr[2], built = (double) ts->hctr[3];
  // walked suffix elements (4 B), each pair's entry, row end and x id (16 B),
  // each table's row and its ids (8 B per element)
  profile_add_bytes("tc_count", 4.0 * walked + 16.0 * m + 8.0 * built);
  if (total_out) *total_out = ts->hctr[4];
  if (st)
  {
    st->iterations = 2;
    st->teps_edges = g.nent;
    st->edges_examined = (uint64_t) walked;
    st->algo_bytes = (uint64_t) (4.0 * walked + 16.0 * m + 8.0 * built + 36.0 * m + 48.0 * N);
  }
  return LA3G_OK;
}
