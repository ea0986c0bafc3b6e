// Split frontiers shared by the top-down BFS and the SSSP relaxation.
//
// A frontier is kept as two lists: "small" vertices (at most kBigDeg edges,
// one warp each) and hubs.  A hub's edges are cut into tasks of kHubTask
// edges; the tasks of all hubs are numbered consecutively and warps take
// tasks, so a hub with a million edges is spread over a thousand warps while
// a warp never loops over hubs it has no work in.
//
// Appending a hub reserves its list slot and its first task number with one
// 64-bit atomicAdd on a packed counter (slot in the high 24 bits, task count
// in the low 40), so task numbers ascend with list slots and a warp finds
// the hub of task t by a binary search over the slots' first tasks.
#ifndef LA3G_FRONTIER_CUH
#define LA3G_FRONTIER_CUH

#include <cstdint>

namespace la3g {

static constexpr uint32_t kBigDeg = 512;
static constexpr uint32_t kHubTask = 1024;
static constexpr int kHubSlotShift = 40;

__device__ __forceinline__ unsigned long long hub_pack_inc(uint32_t ntasks)
{
  return (1ull << kHubSlotShift) | (unsigned long long) ntasks;
}

// Appends hub v with `deg` edges; `packed` counts slots and tasks.
__device__ __forceinline__ void hub_append(uint32_t v, uint32_t deg, uint32_t* big, uint32_t* big_task0,
                                           unsigned long long* packed)
{
  const uint32_t ntasks = (deg + kHubTask - 1) / kHubTask;
  const unsigned long long old = atomicAdd(packed, hub_pack_inc(ntasks));
  const uint32_t slot = (uint32_t) (old >> kHubSlotShift);
  big[slot] = v;
  big_task0[slot] = (uint32_t) (old & ((1ull << kHubSlotShift) - 1));
}

__device__ __forceinline__ uint32_t hub_count(unsigned long long packed) { return (uint32_t) (packed >> kHubSlotShift); }
__device__ __forceinline__ uint32_t hub_tasks(unsigned long long packed)
{
  return (uint32_t) (packed & ((1ull << kHubSlotShift) - 1));
}

// Slot whose task range holds task t (task0 ascends with the slot).
__device__ __forceinline__ uint32_t hub_of_task(const uint32_t* __restrict__ task0, uint32_t nbig, uint32_t t)
{
  uint32_t lo = 0, hi = nbig;
  while (hi - lo > 1)
  {
    uint32_t mid = (lo + hi) >> 1;
    if (task0[mid] <= t) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Multi-source BFS hop bytes are kept vertex-major: the 64 roots of frontier
// word w of vertex v own bytes [64 (v W + w), 64 (v W + w) + 64), so the
// thread that owns a (vertex, word) pair writes its newly reached roots with
// at most eight aligned 8-byte read-modify-writes inside one 64-byte block.
// Byte k of group g takes `hop` when bit 8g + k of nb is set.
__device__ __forceinline__ uint64_t spread_bits_to_bytes(uint32_t m)
{
  uint64_t x = m & 0xFFu;
  x = (x | (x << 28)) & 0x0000000F0000000Full;
  x = (x | (x << 14)) & 0x0003000300030003ull;
  x = (x | (x << 7)) & 0x0101010101010101ull;
  return x * 0xFFu;
}

__device__ __forceinline__ void hops_record(uint8_t* block, uint64_t nb, uint8_t hop)
{
  uint64_t* q = reinterpret_cast<uint64_t*>(block);
  const uint64_t hx = 0x0101010101010101ull * hop;
#pragma unroll
  for (int g = 0; g < 8; g++)
  {
    const uint32_t m = (uint32_t) (nb >> (8 * g)) & 0xFFu;
    if (!m) continue;
    const uint64_t M = spread_bits_to_bytes(m);
    q[g] = (q[g] & ~M) | (hx & M);
  }
}

// Bottom-up scan of one (vertex, word) pair of a multi-source BFS: the OR of
// the frontier words front[u W + w] over the in-neighbours u of v, stopping
// once every bit of `want` is found.  Called by all 32 lanes of a warp with
// one pair each (want = 0 for lanes without work).  A lane scans its own
// first kPullOwn edges, four independent loads at a time; pairs still short
// of bits after that are finished one after another by the whole warp, 32
// edges a step with an OR-reduction, so a hub's list never sits on a single
// thread.  Returns acc & want.
static constexpr uint32_t kPullOwn = 32;

__device__ __forceinline__ uint64_t warp_or64(uint64_t a)
{
  const uint32_t lo = __reduce_or_sync(0xffffffffu, (uint32_t) a);
  const uint32_t hi = __reduce_or_sync(0xffffffffu, (uint32_t) (a >> 32));
  return ((uint64_t) hi << 32) | lo;
}

__device__ __forceinline__ uint64_t pull_scan(uint32_t v, uint32_t w, uint32_t W, uint64_t want,
                                              const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col,
                                              const uint64_t* __restrict__ front, int lane)
{
  uint64_t acc = 0;
  uint32_t e = 0, end = 0;
  if (want)
  {
    e = ptr[v];
    end = ptr[v + 1];
  }
  const uint32_t own = min(end, e + kPullOwn);
  while (e < own && (acc & want) != want)
  {
    uint32_t c[4];
#pragma unroll
    for (int u = 0; u < 4; u++) c[u] = e + u < own ? col[e + u] : 0xFFFFFFFFu;
#pragma unroll
    for (int u = 0; u < 4; u++)
      if (c[u] != 0xFFFFFFFFu) acc |= front[(uint64_t) c[u] * W + w];
    e += 4;
  }
  unsigned m = __ballot_sync(0xffffffffu, (acc & want) != want && own < end);
  while (m)
  {
    const int src = __ffs(m) - 1;
    m &= m - 1;
    const uint32_t ws = __shfl_sync(0xffffffffu, w, src);
    const uint32_t b0 = __shfl_sync(0xffffffffu, own, src), b1 = __shfl_sync(0xffffffffu, end, src);
    const uint64_t wants = __shfl_sync(0xffffffffu, want, src), accs = __shfl_sync(0xffffffffu, acc, src);
    uint64_t a = 0, tot = accs;
    for (uint32_t kb = b0; kb < b1; kb += 32)
    {
      const uint32_t k = kb + lane;
      if (k < b1) a |= front[(uint64_t) col[k] * W + ws];
      tot = accs | warp_or64(a);
      if ((tot & wants) == wants) break;
    }
    if (lane == src) acc = tot;
  }
  return acc & want;
}

}  // namespace la3g

#endif
