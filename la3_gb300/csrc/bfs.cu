// BFS: the reference bfs app (src/apps/graph_analytics/bfs.cpp:11-37,
// bfs.h:11-49) on the device, direction-optimising.
//
// Reference semantics kept exactly (np = 1):
//   * hops are uint8 with 255 = unvisited; apply at iteration i sets
//     hops = (uint8)(i + 1) on a touched vertex whose hops are 255
//     (bfs.h:41-48); the loop stops after the first iteration that activates
//     nothing (execute_non_opt, vertex_program_execute.hpp:166-248);
//   * parent: gather returns edge.src (the hashed id of the column) and
//     combine keeps the last value written (bfs.h:39-40).  The SpMV walks the
//     active columns in ascending position = ascending hashed id, so the
//     last writer of a row is its frontier neighbour with the LARGEST hashed
//     id.  Top-down keeps it with atomicMax; bottom-up scans a vertex's
//     neighbours from the highest position down and stops at the first one
//     in the frontier, which is that same neighbour.
//
// Direction switching follows Beamer et al. (alpha = 14, beta = 24): go
// bottom-up when the frontier's edges exceed the unvisited edges / alpha,
// back top-down when the frontier holds fewer than n / beta vertices.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "frontier.cuh"
#include "la3g_internal.h"

namespace la3g {

struct BfsCounters
{
  unsigned long long next_count;   // vertices activated this iteration
  unsigned long long next_degsum;  // their degrees
};

// Frontier counters of la3g_bfs: a frontier is kept as two lists, vertices
// of degree <= kBigDeg ("small", one warp each) and hubs ("big", whose edges
// the whole grid shares), so that no warp serialises on a hub.
struct FrontierCounters
{
  unsigned long long raw;      // vertices touched by the expansion
  unsigned long long degsum;   // degrees of the next frontier
  unsigned long long nsmall;   // next frontier: small list length
  unsigned long long packed;   // next frontier: hub slots and hub tasks (frontier.cuh)
};

struct BfsScratch
{
  uint8_t* hops = nullptr;
  uint32_t* parent = nullptr;
  uint32_t* cand = nullptr;        // top-down parent candidate + 1 (0 = none)
  uint32_t* raw = nullptr;         // touched vertices of a top-down step
  uint32_t* small[2] = {nullptr, nullptr};
  uint32_t* big[2] = {nullptr, nullptr};
  uint32_t* big_task0[2] = {nullptr, nullptr};
  uint32_t* bits[2] = {nullptr, nullptr};
  // [2] device: ctr[c] holds the sizes of the frontier in small[c] / big[c]
  // and, after a step from buffer c, ctr[c ^ 1] the touched count and the
  // degree sum of the next frontier
  FrontierCounters* ctr = nullptr;
  unsigned long long* state = nullptr;   // the level loop's state (kB* slots), device side
  unsigned long long* hstate = nullptr;  // pinned host mirror
  unsigned long long* red = nullptr;  // reduction scratch
  uint32_t* by_id = nullptr;          // [nslots] outputs reordered by id before they leave the device
  uint32_t words = 0;
  DeviceLoop* loop = nullptr;         // the device-driven level loop (built on first use)
};

// Level-loop state slots (unsigned long long each).
enum : int {
  kBIter = 0,    // levels, counted as the reference counts iterations
  kBPulls,       // bottom-up levels
  kBExamined,    // edges examined
  kBStatus,      // 1: the level limit was reached
  kBFirst,       // 1 until the first decision (the root's frontier is in ctr[0])
  kBMode,        // the body chosen last (kBDone: the loop has ended)
  kBCur,         // which buffer pair holds the current frontier
  kBBottomUp,    // direction of the last level
  kBList,        // 1: the current frontier is in the split lists, 0: only in bits[cur]
  kBUnvisited,   // degree sum of the vertices not yet visited
  kBFrontDeg,    // degree sum of the current frontier
  kBNfront,      // size of the current frontier
  kBCount,       // [8] levels run per body
  kBSlots = kBCount + 8
};
// Bodies: variant * 2 + the current buffer pair.
enum : unsigned { kTdList = 0, kTdBits = 1, kBuList = 2, kBuBits = 3, kBDone = 8 };
static constexpr double kAlpha = 14.0, kBeta = 24.0;

static void bfs_scratch_free(void* p)
{
  BfsScratch* s = (BfsScratch*) p;
  if (s->hstate) cudaFreeHost(s->hstate);
  delete s->loop;
  delete s;
}

__global__ void k_bfs_init(uint32_t N, uint8_t* hops, uint32_t* parent, uint32_t* cand)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x)
  {
    hops[p] = 255;
    parent[p] = 0;
    cand[p] = 0;
  }
}

// Top-down: one warp per frontier vertex, lanes over its neighbours.
__global__ void __launch_bounds__(256)
k_bfs_td(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, const uint32_t* __restrict__ hash_of_pos,
         uint32_t N, const uint32_t* __restrict__ front, uint32_t nfront, const uint8_t* __restrict__ hops,
         uint32_t* cand, uint32_t* next, BfsCounters* ctr)
{
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t f = warp; f < nfront; f += nwarps)
  {
    const uint32_t u = front[f];
    const uint32_t hu = hash_of_pos[u] + 1;
    const uint32_t b = ptr[u], e = ptr[u + 1];
    for (uint32_t i0 = b; i0 < e; i0 += 32)
    {
      const uint32_t i = i0 + lane;
      bool add = false;
      uint32_t v = 0;
      if (i < e)
      {
        v = col[i];
        if (v < N && hops[v] == 255)  // a neighbour id outside the graph is skipped
        {
          uint32_t old = atomicMax(&cand[v], hu);
          add = old == 0;
        }
      }
      const unsigned mask = __ballot_sync(0xffffffffu, add);
      if (mask)
      {
        uint32_t base = 0;
        if (lane == 0) base = (uint32_t) atomicAdd(&ctr->next_count, (unsigned long long) __popc(mask));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (add) next[base + __popc(mask & ((1u << lane) - 1))] = v;
      }
    }
  }
}

// Top-down apply: the newly touched vertices take hops and parent.
__global__ void k_bfs_td_apply(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ next, uint32_t n,
                               uint8_t hop, uint8_t* hops, uint32_t* parent, uint32_t* cand, BfsCounters* ctr)
{
  unsigned long long deg = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
  {
    uint32_t v = next[i];
    hops[v] = hop;
    parent[v] = cand[v] - 1;
    cand[v] = 0;
    deg += ptr[v + 1] - ptr[v];
  }
  for (int o = 16; o > 0; o >>= 1) deg += __shfl_xor_sync(0xffffffffu, deg, o);
  if ((threadIdx.x & 31) == 0 && deg) atomicAdd(&ctr->next_degsum, deg);
}

// Bottom-up: one thread per unvisited vertex, neighbours from the highest
// position down; the first frontier neighbour is the parent.
__global__ void __launch_bounds__(256)
k_bfs_bu(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, const uint32_t* __restrict__ hash_of_pos,
         uint32_t nrows, const uint32_t* __restrict__ fbits, uint32_t* nbits, uint8_t hop, uint8_t* hops,
         uint32_t* parent, BfsCounters* ctr)
{
  unsigned long long cnt = 0, deg = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nrows; v += gridDim.x * blockDim.x)
  {
    if (hops[v] != 255) continue;
    const uint32_t b = ptr[v], e = ptr[v + 1];
    for (uint32_t i = e; i > b; i--)
    {
      const uint32_t u = col[i - 1];
      if (u < nrows && (fbits[u >> 5] & (1u << (u & 31))))  // ids outside the graph are skipped
      {
        hops[v] = hop;
        parent[v] = hash_of_pos[u];
        atomicOr(&nbits[v >> 5], 1u << (v & 31));
        cnt++;
        deg += e - b;
        break;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1)
  {
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    deg += __shfl_xor_sync(0xffffffffu, deg, o);
  }
  if ((threadIdx.x & 31) == 0 && cnt)
  {
    atomicAdd(&ctr->next_count, cnt);
    atomicAdd(&ctr->next_degsum, deg);
  }
}

__global__ void k_list_to_bits(const uint32_t* __restrict__ list, uint32_t n, uint32_t* bits)
{
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
  {
    uint32_t v = list[i];
    atomicOr(&bits[v >> 5], 1u << (v & 31));
  }
}

__global__ void k_bits_to_list(const uint32_t* __restrict__ bits, uint32_t words, uint32_t* list, unsigned long long* count)
{
  const int lane = threadIdx.x & 31;
  for (uint32_t w0 = blockIdx.x * blockDim.x; w0 < words; w0 += gridDim.x * blockDim.x)
  {
    uint32_t w = w0 + threadIdx.x;
    uint32_t x = w < words ? bits[w] : 0;
    uint32_t c = __popc(x);
    uint32_t incl = c;
    for (int o = 1; o < 32; o <<= 1)
    {
      uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    uint32_t base = 0;
    if (lane == 31 && total) base = (uint32_t) atomicAdd(count, (unsigned long long) total);
    base = __shfl_sync(0xffffffffu, base, 31);
    uint32_t o = base + incl - c;
    while (x)
    {
      int bpos = __ffs(x) - 1;
      x &= x - 1;
      list[o++] = w * 32 + bpos;
    }
  }
}

// Top-down over a split frontier.  Hubs first: every warp of the grid
// takes a slice of each hub's edges; then one warp per small vertex.  A
// touched unvisited vertex keeps the largest key + 1 in cand; the thread that
// moves cand away from 0 records the vertex in `raw`.
__device__ __forceinline__ void td_visit(uint32_t v, bool valid, uint32_t hu, const uint8_t* __restrict__ hops,
                                         uint32_t* cand, uint32_t* raw, FrontierCounters* ctr, int lane)
{
  bool add = false;
  if (valid && hops[v] == 255) add = atomicMax(&cand[v], hu) == 0;
  const unsigned mask = __ballot_sync(0xffffffffu, add);
  if (mask)
  {
    uint32_t base = 0;
    if (lane == 0) base = (uint32_t) atomicAdd(&ctr->raw, (unsigned long long) __popc(mask));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (add) raw[base + __popc(mask & ((1u << lane) - 1))] = v;
  }
}

__global__ void __launch_bounds__(256)
k_bfs_td_split(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, const uint32_t* __restrict__ key,
               const uint32_t* __restrict__ small, const uint32_t* __restrict__ big,
               const uint32_t* __restrict__ big_task0, const FrontierCounters* __restrict__ front,
               const uint8_t* __restrict__ hops, uint32_t* cand, uint32_t* raw, FrontierCounters* ctr)
{
  const uint32_t nsmall = (uint32_t) front->nsmall;
  const uint32_t nbig = hub_count(front->packed), ntasks = hub_tasks(front->packed);
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t t = warp; t < ntasks; t += nwarps)
  {
    const uint32_t slot = hub_of_task(big_task0, nbig, t);
    const uint32_t u = big[slot];
    const uint32_t hu = key[u] + 1;
    const uint32_t b = ptr[u] + (t - big_task0[slot]) * kHubTask;
    const uint32_t e = min(b + kHubTask, ptr[u + 1]);
    for (uint32_t i0 = b; i0 < e; i0 += 32)
    {
      const uint32_t i = i0 + lane;
      td_visit(i < e ? col[i] : 0, i < e, hu, hops, cand, raw, ctr, lane);
    }
  }
  for (uint32_t f = warp; f < nsmall; f += nwarps)
  {
    const uint32_t u = small[f];
    const uint32_t hu = key[u] + 1;
    const uint32_t b = ptr[u], e = ptr[u + 1];
    for (uint32_t i0 = b; i0 < e; i0 += 32)
    {
      const uint32_t i = i0 + lane;
      td_visit(i < e ? col[i] : 0, i < e, hu, hops, cand, raw, ctr, lane);
    }
  }
}

__device__ __forceinline__ void push_split(uint32_t v, uint32_t deg, uint32_t* small, uint32_t* big,
                                           uint32_t* big_task0, FrontierCounters* ctr)
{
  if (deg > kBigDeg) hub_append(v, deg, big, big_task0, &ctr->packed);
  else small[atomicAdd(&ctr->nsmall, 1ull)] = v;
}

// Top-down apply: touched vertices take hops and parent and form the next
// frontier, split by degree.
__global__ void k_bfs_td_apply_split(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ raw,
                                     const unsigned long long* __restrict__ state, uint8_t* hops, uint32_t* parent,
                                     uint32_t* cand, uint32_t* small, uint32_t* big, uint32_t* big_task0,
                                     FrontierCounters* ctr)
{
  const uint8_t hop = (uint8_t) (state[kBIter] + 1);
  unsigned long long deg = 0;
  const uint32_t n = (uint32_t) ctr->raw;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
  {
    uint32_t v = raw[i];
    hops[v] = hop;
    parent[v] = cand[v] - 1;
    cand[v] = 0;
    uint32_t d = ptr[v + 1] - ptr[v];
    deg += d;
    push_split(v, d, small, big, big_task0, ctr);
  }
  deg = block_sum_u64(deg);
  if (threadIdx.x == 0 && deg) atomicAdd(&ctr->degsum, deg);
}

// Bottom-up with the split counters (same scan as k_bfs_bu).
__global__ void __launch_bounds__(256)
k_bfs_bu_split(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, const uint32_t* __restrict__ key,
               uint32_t nrows, const uint32_t* __restrict__ fbits, uint32_t* nbits,
               const unsigned long long* __restrict__ state, uint8_t* hops, uint32_t* parent, FrontierCounters* ctr)
{
  const uint8_t hop = (uint8_t) (state[kBIter] + 1);
  unsigned long long cnt = 0, deg = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nrows; v += gridDim.x * blockDim.x)
  {
    if (hops[v] != 255) continue;
    const uint32_t b = ptr[v], e = ptr[v + 1];
    for (uint32_t i = e; i > b; i--)
    {
      const uint32_t u = col[i - 1];
      if (fbits[u >> 5] & (1u << (u & 31)))
      {
        hops[v] = hop;
        parent[v] = key[u];
        atomicOr(&nbits[v >> 5], 1u << (v & 31));
        cnt++;
        deg += e - b;
        break;
      }
    }
  }
  cnt = block_sum_u64(cnt);
  deg = block_sum_u64(deg);
  if (threadIdx.x == 0 && cnt)
  {
    atomicAdd(&ctr->raw, cnt);
    atomicAdd(&ctr->degsum, deg);
  }
}

// Split-list frontier (sizes in `front`) -> bitmap.
__global__ void k_front_to_bits(const uint32_t* __restrict__ small, const uint32_t* __restrict__ big,
                                const FrontierCounters* __restrict__ front, uint32_t* bits)
{
  const uint32_t ns = (uint32_t) front->nsmall, n = ns + hub_count(front->packed);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
  {
    const uint32_t v = i < ns ? small[i] : big[i - ns];
    atomicOr(&bits[v >> 5], 1u << (v & 31));
  }
}

// Bitmap frontier -> split lists.
__global__ void k_bits_to_split(const uint32_t* __restrict__ bits, uint32_t words, const uint32_t* __restrict__ ptr,
                                uint32_t* small, uint32_t* big, uint32_t* big_task0, FrontierCounters* ctr)
{
  for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < words; w += gridDim.x * blockDim.x)
  {
    uint32_t x = bits[w];
    while (x)
    {
      int b = __ffs(x) - 1;
      x &= x - 1;
      uint32_t v = w * 32 + b;
      push_split(v, ptr[v + 1] - ptr[v], small, big, big_task0, ctr);
    }
  }
}

__global__ void k_reached_degsum(const uint32_t* __restrict__ ptr, const uint8_t* __restrict__ hops, uint32_t nrows,
                                 unsigned long long* out)
{
  unsigned long long s = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nrows; v += gridDim.x * blockDim.x)
    if (hops[v] != 255) s += ptr[v + 1] - ptr[v];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, s);
}

template <class T>
__global__ void k_by_id(uint32_t N, const uint32_t* __restrict__ id_of_pos, const T* __restrict__ val, T* __restrict__ out)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) out[id_of_pos[p]] = val[p];
}

__global__ void k_bfs_root(uint32_t rp, uint8_t* hops, uint32_t* list) { hops[rp] = 0; list[0] = rp; }

// The root (an id below N): hops 0, and the first frontier in small[0] or
// big[0] with its sizes in ctr[0] (empty if the root has no edges); the
// loop state starts at level 0, top-down, from the lists.
__global__ void k_bfs_root_state(uint32_t root, const uint32_t* __restrict__ pos_of_id,
                                 const uint32_t* __restrict__ ptr, uint32_t nrows, uint64_t nent, uint8_t* hops,
                                 uint32_t* small, uint32_t* big, uint32_t* big_task0, FrontierCounters* ctr,
                                 unsigned long long* state)
{
  for (int k = 0; k < kBSlots; k++) state[k] = 0;
  state[kBFirst] = 1;
  state[kBList] = 1;
  const uint32_t rp = pos_of_id[root];
  hops[rp] = 0;
  uint64_t deg = 0;
  if (rp < nrows)
  {
    deg = ptr[rp + 1] - ptr[rp];
    if (deg > kBigDeg)
    {
      big[0] = rp;
      big_task0[0] = 0;
      ctr->packed = hub_pack_inc((uint32_t) ((deg + kHubTask - 1) / kHubTask));
    }
    else
    {
      small[0] = rp;
      ctr->nsmall = 1;
    }
    state[kBNfront] = 1;
  }
  state[kBFrontDeg] = deg;
  state[kBUnvisited] = nent - deg;
}

// Start of every level (one thread).  First folds in what the last level
// left in ctr[cur ^ 1] (as the reference's loop does after each SpMV: the
// next frontier's size and degree sum, the unvisited degree sum), then
// picks the direction (Beamer's alpha / beta test) and the body: top-down
// from the lists, top-down after turning the bottom-up bitmap into lists,
// bottom-up after turning the lists into a bitmap, or bottom-up from the
// bitmap.  An empty frontier ends the loop.
__global__ void k_bfs_decide(unsigned long long* S, FrontierCounters* ctr, uint32_t N, uint64_t limit,
                             cudaGraphConditionalHandle cont, cudaGraphConditionalHandle mode)
{
  unsigned long long it = S[kBIter];
  bool done = false, convert = false;
  if (S[kBFirst]) S[kBFirst] = 0;
  else
  {
    const unsigned cur = (unsigned) S[kBCur];
    const FrontierCounters c = ctr[cur ^ 1];
    const unsigned long long nn = c.raw;
    unsigned long long fdeg, nfront = nn;
    bool list = true;
    if (S[kBMode] / 2 >= kBuList)
    {
      fdeg = c.degsum;
      const bool next_bu = !((double) nn < (double) N / kBeta);
      if (nn && !next_bu) convert = true;  // the bitmap becomes lists before the top-down level
      else list = false;
    }
    else
    {
      nfront = nn ? c.nsmall + hub_count(c.packed) : 0;
      fdeg = nn ? c.degsum : 0;
    }
    S[kBUnvisited] -= min(S[kBUnvisited], fdeg);
    S[kBCur] = cur ^ 1;
    S[kBFrontDeg] = fdeg;
    S[kBNfront] = nfront;
    S[kBList] = list;
    it++;
    if (nfront == 0) done = true;
  }
  unsigned m = kBDone;
  if (!done)
  {
    if (it > limit) S[kBStatus] = 1;
    else
    {
      const unsigned long long nfront = S[kBNfront], fdeg = S[kBFrontDeg], unv = S[kBUnvisited];
      bool bu = S[kBBottomUp] != 0;
      if (!bu && (double) fdeg > (double) unv / kAlpha) bu = true;
      else if (bu && (double) nfront < (double) N / kBeta) bu = false;
      S[kBBottomUp] = bu;
      if (nfront == 0) it++;  // nothing active: this level activates nothing
      else
      {
        const unsigned variant = bu ? (S[kBList] && !convert ? kBuList : kBuBits) : (convert ? kTdBits : kTdList);
        m = variant * 2 + (unsigned) S[kBCur];
        if (bu)
        {
          S[kBExamined] += unv;
          S[kBPulls]++;
        }
        else S[kBExamined] += fdeg;
        S[kBCount + m]++;
        // the counters the body accumulates into start at zero (no memset
        // node between the levels): the next frontier's, and the list sizes
        // of a bitmap turned into lists
        const unsigned c = m & 1;
        ctr[c ^ 1] = FrontierCounters{0, 0, 0, 0};
        if (variant == kTdBits)
        {
          ctr[c].nsmall = 0;
          ctr[c].packed = 0;
        }
      }
    }
  }
  S[kBIter] = it;
  S[kBMode] = m;
  loop_set(cont, m != kBDone);
  loop_set(mode, m);
}

static int bfs_scratch(la3g_graph* G, BfsScratch** out)
{
  BfsScratch* bs = (BfsScratch*) G->slot[kSlotBfs];
  if (bs) { *out = bs; return LA3G_OK; }
  bs = new (std::nothrow) BfsScratch();
  if (!bs) return set_error(LA3G_ENOMEM, "out of host memory");
  G->slot[kSlotBfs] = bs;
  G->slot_free[kSlotBfs] = bfs_scratch_free;
  const uint32_t N = G->g.nslots;
  bs->words = (N + 31) / 32 + 1;
  LA3G_TRY(galloc(G, &bs->hops, N));
  LA3G_TRY(galloc(G, &bs->parent, N));
  LA3G_TRY(galloc(G, &bs->cand, N));
  LA3G_TRY(galloc(G, &bs->raw, N));
  LA3G_TRY(galloc(G, &bs->small[0], N));
  LA3G_TRY(galloc(G, &bs->small[1], N));
  LA3G_TRY(galloc(G, &bs->big[0], N));
  LA3G_TRY(galloc(G, &bs->big[1], N));
  LA3G_TRY(galloc(G, &bs->big_task0[0], N));
  LA3G_TRY(galloc(G, &bs->big_task0[1], N));
  LA3G_TRY(galloc(G, &bs->bits[0], bs->words));
  LA3G_TRY(galloc(G, &bs->bits[1], bs->words));
  LA3G_TRY(galloc(G, &bs->ctr, 2));
  LA3G_TRY(galloc(G, &bs->state, kBSlots));
  LA3G_TRY(galloc(G, &bs->red, 1));
  LA3G_TRY(galloc(G, &bs->by_id, N));
  LA3G_CUDA(cudaHostAlloc(&bs->hstate, kBSlots * sizeof(unsigned long long), cudaHostAllocDefault));
  *out = bs;
  return LA3G_OK;
}

// One level's body m = variant * 2 + c (c: the buffer pair holding the
// current frontier).  `fdeg`, `nfront` and `unv` (frontier degree sum and
// size, unvisited degree sum) only size the profile entries' bytes; the
// kernels read every count they need on the device.
static int bfs_body(la3g_graph* G, BfsScratch* bs, cudaStream_t s, unsigned m, double fdeg, double nfront, double unv)
{
  DevGraph& g = G->g;
  const uint32_t N = g.nslots, nrows = g.nrows();
  const unsigned variant = m / 2, c = m & 1;
  FrontierCounters* cur = bs->ctr + c;
  FrontierCounters* next = bs->ctr + (c ^ 1);  // zeroed by the decide kernel, as are cur's list sizes for kTdBits
  if (variant == kTdBits)
  {
    // the bottom-up level's bitmap becomes split lists (sizes into ctr[c])
    k_bits_to_split<<<grid_for(bs->words, 256), 256, 0, s>>>(bs->bits[c], bs->words, g.in_ptr, bs->small[c],
                                                              bs->big[c], bs->big_task0[c], cur);
    LA3G_LAUNCHED();
    tls_launches++;
  }
  if (variant == kTdList || variant == kTdBits)
  {
    {
      ProfileScope p("bfs_top_down", s, 4.0 * fdeg + 8.0 * nfront + 1.0 * fdeg);
      k_bfs_td_split<<<num_sms() * 8, 256, 0, s>>>(g.in_ptr, g.in_col, g.hash_of_pos, bs->small[c], bs->big[c],
                                                   bs->big_task0[c], cur, bs->hops, bs->cand, bs->raw, next);
      LA3G_LAUNCHED();
    }
    k_bfs_td_apply_split<<<num_sms() * 4, 256, 0, s>>>(g.in_ptr, bs->raw, bs->state, bs->hops, bs->parent, bs->cand,
                                                       bs->small[c ^ 1], bs->big[c ^ 1], bs->big_task0[c ^ 1], next);
    LA3G_LAUNCHED();
    tls_launches++;
    return LA3G_OK;
  }
  if (variant == kBuList)
  {
    LA3G_CUDA(cudaMemsetAsync(bs->bits[c], 0, (size_t) bs->words * 4, s));
    k_front_to_bits<<<num_sms() * 4, 256, 0, s>>>(bs->small[c], bs->big[c], cur, bs->bits[c]);
    LA3G_LAUNCHED();
    tls_launches++;
  }
  LA3G_CUDA(cudaMemsetAsync(bs->bits[c ^ 1], 0, (size_t) bs->words * 4, s));
  ProfileScope p("bfs_bottom_up", s, 4.0 * unv + 8.0 * nrows + N / 8.0);
  k_bfs_bu_split<<<grid_for(nrows, 256, num_sms() * 16), 256, 0, s>>>(g.in_ptr, g.in_col, g.hash_of_pos, nrows,
                                                                      bs->bits[c], bs->bits[c ^ 1], bs->state,
                                                                      bs->hops, bs->parent, next);
  LA3G_LAUNCHED();
  return LA3G_OK;
}

static int bfs_decide(la3g_graph* G, BfsScratch* bs, cudaStream_t s, cudaGraphConditionalHandle cont,
                      cudaGraphConditionalHandle mode)
{
  // every level visits at least one new vertex: N + 2 levels is a fault
  k_bfs_decide<<<1, 1, 0, s>>>(bs->state, bs->ctr, G->g.nslots, (uint64_t) G->g.nslots + 2, cont, mode);
  LA3G_LAUNCHED();
  tls_launches++;
  return LA3G_OK;
}

// Runs BFS from `root` with results left on the device (positions).  The
// levels run as one device-driven graph (no host round trip per level);
// with profiling on they are stepped from the host instead, so that each
// kernel is timed.
static int bfs_run(la3g_graph* G, BfsScratch* bs, uint32_t root, la3g_stats* st)
{
  DevGraph& g = G->g;
  cudaStream_t s = G->stream;
  const uint32_t N = g.nslots;
  k_bfs_init<<<grid_for(N, 256), 256, 0, s>>>(N, bs->hops, bs->parent, bs->cand);
  LA3G_LAUNCHED();
  tls_launches++;
  if (root >= N)
  {
    if (st) st->iterations = 1;
    return LA3G_OK;  // no vertex matches the root: every hop stays 255
  }
  LA3G_CUDA(cudaMemsetAsync(bs->ctr, 0, 2 * sizeof(FrontierCounters), s));
  k_bfs_root_state<<<1, 1, 0, s>>>(root, g.pos_of_id, g.in_ptr, g.nrows(), g.nent, bs->hops, bs->small[0], bs->big[0],
                                   bs->big_task0[0], bs->ctr, bs->state);
  LA3G_LAUNCHED();
  tls_launches++;
  unsigned long long* H = bs->hstate;
  if (!profile_enabled())
  {
    if (!bs->loop)
    {
      bs->loop = new (std::nothrow) DeviceLoop();
      if (!bs->loop) return set_error(LA3G_ENOMEM, "out of host memory");
      const int rc = device_loop_build(
          bs->loop, 8,
          [&](cudaStream_t c, cudaGraphConditionalHandle cont, cudaGraphConditionalHandle mode) {
            return bfs_decide(G, bs, c, cont, mode);
          },
          [&](cudaStream_t c, int k) { return bfs_body(G, bs, c, (unsigned) k, 0.0, 0.0, 0.0); });
      if (rc != LA3G_OK)
      {
        delete bs->loop;
        bs->loop = nullptr;
        return rc;
      }
    }
    LA3G_CUDA(cudaGraphLaunch(bs->loop->exec, s));
    LA3G_CUDA(cudaMemcpyAsync(H, bs->state, kBSlots * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    // the graph's launches: one decide per pass, each body's kernels per level
    uint64_t n = 1;
    for (int k = 0; k < 8; k++) n += H[kBCount + k] * (1 + bs->loop->body_launches[k]);
    tls_launches += (uint32_t) n;
  }
  else
  {
    for (;;)
    {
      LA3G_TRY(bfs_decide(G, bs, s, 0, 0));
      LA3G_CUDA(cudaMemcpyAsync(H, bs->state, kBSlots * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
      LA3G_CUDA(cudaStreamSynchronize(s));
      const unsigned m = (unsigned) H[kBMode];
      if (m == kBDone) break;
      LA3G_TRY(bfs_body(G, bs, s, m, (double) H[kBFrontDeg], (double) H[kBNfront], (double) H[kBUnvisited]));
    }
  }
  if (H[kBStatus]) return set_error(LA3G_ETIMEOUT, "bfs did not converge");
  if (st)
  {
    st->iterations = (uint32_t) H[kBIter];
    st->pull_iterations = (uint32_t) H[kBPulls];
    st->edges_examined = H[kBExamined];
  }
  return LA3G_OK;
}

}  // namespace la3g

using namespace la3g;

extern "C" int la3g_bfs(la3g_graph* G, uint32_t root, uint8_t* hops_out, uint32_t* parent_out, la3g_stats* st)
{
  if (!G) return set_error(LA3G_EINVAL, "null graph");
  DevGraph& g = G->g;
  if (g.directed()) return set_error(LA3G_EINVAL, "bfs needs an undirected graph (load without LA3G_DIRECTED)");
  CallTimer T(G, st);
  BfsScratch* bs = nullptr;
  LA3G_TRY(bfs_scratch(G, &bs));
  cudaStream_t s = G->stream;
  const uint32_t N = g.nslots;
  T.device_begin();
  LA3G_TRY(bfs_run(G, bs, root, st));
  T.device_end();
  if (st)
  {
    LA3G_CUDA(cudaMemsetAsync(bs->red, 0, 8, s));
    k_reached_degsum<<<grid_for(g.nrows(), 256), 256, 0, s>>>(g.in_ptr, bs->hops, g.nrows(), bs->red);
    LA3G_LAUNCHED();
    unsigned long long sum = 0;
    LA3G_CUDA(cudaMemcpyAsync(&sum, bs->red, 8, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    st->teps_edges = sum / 2;
    st->algo_bytes = st->edges_examined * 4 + (uint64_t) N * 6;
  }
  if (hops_out || parent_out)
  {
    // the graph's own reorder buffer: no allocation per call
    if (hops_out)
    {
      k_by_id<uint8_t><<<grid_for(N, 256), 256, 0, s>>>(N, g.id_of_pos, bs->hops, (uint8_t*) bs->by_id);
      LA3G_LAUNCHED();
      LA3G_CUDA(cudaMemcpyAsync(hops_out, bs->by_id, N, cudaMemcpyDeviceToHost, s));
      LA3G_CUDA(cudaStreamSynchronize(s));
    }
    if (parent_out)
    {
      k_by_id<uint32_t><<<grid_for(N, 256), 256, 0, s>>>(N, g.id_of_pos, bs->parent, bs->by_id);
      LA3G_LAUNCHED();
      LA3G_CUDA(cudaMemcpyAsync(parent_out, bs->by_id, (size_t) N * 4, cudaMemcpyDeviceToHost, s));
      LA3G_CUDA(cudaStreamSynchronize(s));
    }
  }
  return T.finish();
}

// ---------------------------------------------------------------------------
// la3g_bfs_noalloc: the same BFS kernels over a CSR the caller already holds
// in device memory, with every temporary in one fixed device array, so the
// call itself never allocates.
//
// The scratch lives in `g_bfs_noalloc_scratch`, a file-scope __device__
// array: each GPU that loads this library holds it (kNoAllocScratchBytes,
// about 12.8 MB) until the process exits.  Host code must not hand the
// array's name to a kernel (on the host it only names a stand-in object);
// every call looks up its device address on the current device with
// cudaGetSymbolAddress (which allocates nothing), so the address stays right
// for whichever device and context is current.
//
// All calls share the one array and it keeps whatever the last call left in
// it; the call clears what has to start at zero.  Two calls whose work
// overlaps on the GPU (different streams, or different host threads on one
// device) race on the array: serialise them.  The call waits for its stream
// at every BFS level (it reads the frontier size back), and before it
// returns, on success and on every error after its first launch, so no work
// of a finished call is left running on the array.
// ---------------------------------------------------------------------------

namespace la3g {

static constexpr uint32_t kNoAllocMaxVertices = 1u << 20;
static constexpr size_t kNaAlign = 256;
static constexpr size_t na_round(size_t b) { return (b + kNaAlign - 1) / kNaAlign * kNaAlign; }
static constexpr uint32_t kNaWords = kNoAllocMaxVertices / 32 + 1;
static constexpr size_t kNaCandOff = 0;
static constexpr size_t kNaList0Off = kNaCandOff + na_round(sizeof(uint32_t) * kNoAllocMaxVertices);
static constexpr size_t kNaList1Off = kNaList0Off + na_round(sizeof(uint32_t) * kNoAllocMaxVertices);
static constexpr size_t kNaBits0Off = kNaList1Off + na_round(sizeof(uint32_t) * kNoAllocMaxVertices);
static constexpr size_t kNaBits1Off = kNaBits0Off + na_round(sizeof(uint32_t) * kNaWords);
static constexpr size_t kNaCtrOff = kNaBits1Off + na_round(sizeof(uint32_t) * kNaWords);
static constexpr size_t kNaRedOff = kNaCtrOff + na_round(sizeof(BfsCounters));
static constexpr size_t kNoAllocScratchBytes = kNaRedOff + na_round(sizeof(unsigned long long));

static __device__ __align__(256) unsigned char g_bfs_noalloc_scratch[kNoAllocScratchBytes];

// Device address of the scratch array on the current device.
static int noalloc_scratch(unsigned char** out)
{
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_bfs_noalloc_scratch);
  if (e != cudaSuccess || !p)
  {
    cudaGetLastError();
    return set_error(LA3G_ECUDA, "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
  }
  *out = (unsigned char*) p;
  return LA3G_OK;
}

}  // namespace la3g

namespace la3g {

static int bfs_noalloc_run(const uint32_t* row_ptr, const uint32_t* col, const uint32_t* key, uint32_t nvertices,
                           uint32_t root, uint8_t* hops, uint32_t* parent, cudaStream_t s, la3g_stats* st,
                           bool* launched);

}  // namespace la3g

extern "C" int la3g_bfs_noalloc(const uint32_t* row_ptr, const uint32_t* col, const uint32_t* key,
                                uint32_t nvertices, uint32_t root, uint8_t* hops, uint32_t* parent,
                                void* cuda_stream, la3g_stats* st)
{
  using namespace la3g;
  if (st) std::memset(st, 0, sizeof *st);
  if (nvertices == 0 || nvertices > kNoAllocMaxVertices)
    return set_error(LA3G_EINVAL,
                     "la3g_bfs_noalloc: nvertices = %u; it must be between 1 and %u (the size of its fixed scratch)",
                     nvertices, kNoAllocMaxVertices);
  if (!row_ptr || !col || !key || !hops || !parent)
    return set_error(LA3G_EINVAL, "la3g_bfs_noalloc: row_ptr, col, key, hops and parent must be device pointers");
  cudaStream_t s = (cudaStream_t) cuda_stream;
  bool launched = false;
  const int rc = bfs_noalloc_run(row_ptr, col, key, nvertices, root, hops, parent, s, st, &launched);
  if (rc != LA3G_OK && launched)
  {
    // let the work already queued finish before the caller may reuse the array
    cudaStreamSynchronize(s);
    cudaGetLastError();
  }
  return rc;
}

namespace la3g {

static int bfs_noalloc_run(const uint32_t* row_ptr, const uint32_t* col, const uint32_t* key, uint32_t nvertices,
                           uint32_t root, uint8_t* hops, uint32_t* parent, cudaStream_t s, la3g_stats* st,
                           bool* launched)
{
  unsigned char* base = nullptr;
  LA3G_TRY(noalloc_scratch(&base));
  uint32_t* cand = (uint32_t*) (base + kNaCandOff);
  uint32_t* list[2] = {(uint32_t*) (base + kNaList0Off), (uint32_t*) (base + kNaList1Off)};
  uint32_t* bits[2] = {(uint32_t*) (base + kNaBits0Off), (uint32_t*) (base + kNaBits1Off)};
  BfsCounters* ctr = (BfsCounters*) (base + kNaCtrOff);
  unsigned long long* red = (unsigned long long*) (base + kNaRedOff);
  const uint32_t N = nvertices;
  const uint32_t words = (N + 31) / 32 + 1;
  double t0 = now_ms();

  // hops = 255, parent = 0 and the candidates cleared (they must start at 0)
  *launched = true;
  k_bfs_init<<<grid_for(N, 256), 256, 0, s>>>(N, hops, parent, cand);
  LA3G_LAUNCHED();
  uint32_t iter = 0, pull_iters = 0;
  if (root < N)
  {
    uint32_t m = 0, rp[2] = {0, 0};
    LA3G_CUDA(cudaMemcpyAsync(&m, row_ptr + N, 4, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaMemcpyAsync(rp, row_ptr + root, 8, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    k_bfs_root<<<1, 1, 0, s>>>(root, hops, list[0]);
    LA3G_LAUNCHED();
    uint64_t nfront = rp[1] > rp[0] ? 1 : 0;
    uint64_t front_deg = rp[1] - rp[0];
    uint64_t unvisited_deg = m - front_deg;
    bool bottom_up = false, front_is_list = true;
    int cur = 0;
    BfsCounters h;
    for (;;)
    {
      if (iter > 100000) return set_error(LA3G_ETIMEOUT, "la3g_bfs_noalloc did not converge");
      if (!bottom_up && (double) front_deg > (double) unvisited_deg / 14.0) bottom_up = true;
      else if (bottom_up && (double) nfront < (double) N / 24.0) bottom_up = false;
      const uint8_t hop = (uint8_t) (iter + 1);
      if (nfront == 0) { iter++; break; }
      LA3G_CUDA(cudaMemsetAsync(ctr, 0, sizeof(BfsCounters), s));
      if (bottom_up)
      {
        if (front_is_list)
        {
          LA3G_CUDA(cudaMemsetAsync(bits[cur], 0, (size_t) words * 4, s));
          k_list_to_bits<<<grid_for(nfront, 256), 256, 0, s>>>(list[cur], (uint32_t) nfront, bits[cur]);
          LA3G_LAUNCHED();
        }
        LA3G_CUDA(cudaMemsetAsync(bits[cur ^ 1], 0, (size_t) words * 4, s));
        k_bfs_bu<<<grid_for(N, 256, num_sms() * 16), 256, 0, s>>>(row_ptr, col, key, N, bits[cur], bits[cur ^ 1], hop, hops,
                                                            parent, ctr);
        LA3G_LAUNCHED();
        front_is_list = false;
        pull_iters++;
      }
      else
      {
        if (!front_is_list)
        {
          LA3G_CUDA(cudaMemsetAsync(red, 0, 8, s));
          k_bits_to_list<<<grid_for(words, 256), 256, 0, s>>>(bits[cur], words, list[cur], red);
          LA3G_LAUNCHED();
        }
        k_bfs_td<<<grid_for(nfront * 32, 256), 256, 0, s>>>(row_ptr, col, key, N, list[cur], (uint32_t) nfront, hops,
                                                            cand, list[cur ^ 1], ctr);
        LA3G_LAUNCHED();
        LA3G_CUDA(cudaMemcpyAsync(&h, ctr, sizeof h, cudaMemcpyDeviceToHost, s));
        LA3G_CUDA(cudaStreamSynchronize(s));
        if (h.next_count)
        {
          k_bfs_td_apply<<<grid_for(h.next_count, 256), 256, 0, s>>>(row_ptr, list[cur ^ 1], (uint32_t) h.next_count,
                                                                     hop, hops, parent, cand, ctr);
          LA3G_LAUNCHED();
        }
        front_is_list = true;
      }
      LA3G_CUDA(cudaMemcpyAsync(&h, ctr, sizeof h, cudaMemcpyDeviceToHost, s));
      LA3G_CUDA(cudaStreamSynchronize(s));
      nfront = h.next_count;
      front_deg = h.next_degsum;
      unvisited_deg -= std::min<uint64_t>(unvisited_deg, front_deg);
      cur ^= 1;
      iter++;
      if (nfront == 0) break;
    }
  }
  else
  {
    iter = 1;
  }
  LA3G_CUDA(cudaStreamSynchronize(s));
  if (st)
  {
    st->iterations = iter;
    st->pull_iterations = pull_iters;
    st->host_ms = now_ms() - t0;
  }
  return LA3G_OK;
}

}  // namespace la3g
