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
// iteration is min(old, min over messages) exactly as apply computes it.  A
// row is activated iff some relaxation lowered it, i.e. iff its distance is
// now below its message (the distance it scattered when it was last
// activated; INF if never): one dense pass over the regular rows after each
// iteration finds those rows, scatters their new distance and forms the next
// frontier, so the relaxations themselves only do a non-returning atomicMin.
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
  uint32_t* msg = nullptr;        // the distance each vertex scattered at its last activation (INF if never)
  uint32_t* reg_end = nullptr;   // [nslots] end of each vertex's out-edges into regular rows
  uint32_t* small[1] = {nullptr};      // push steps: the frontier's split lists
  uint32_t* big[1] = {nullptr};
  uint32_t* big_task0[1] = {nullptr};
  // [0] activated count, [1] their regular out-degree sum, [2] activated with regular out-edges,
  // [3] scratch, [4] scratch, [5] the next frontier's smallest message
  unsigned long long* ctr = nullptr;
  unsigned long long* hctr = nullptr;
  uint32_t* fbits = nullptr;      // [nslots / 32 + 1] the current frontier, one bit per vertex
  unsigned long long* fctr = nullptr;  // push steps: [0] small-list length, [1] hub slots and tasks
  uint32_t* fmsg = nullptr;       // pull steps: msg of the current frontier's vertices, INF elsewhere
  uint32_t* long_rows = nullptr;  // regular rows with more than kPullLong in-edges
  uint32_t nlong = 0;
  uint32_t* task_row = nullptr;   // pull tasks over the long rows: kPullChunk in-edges each
  uint32_t* task_begin = nullptr;
  uint32_t ntasks = 0;
  uint64_t task_edges = 0;        // in-edges of the long rows
  uint32_t* ymin = nullptr;       // [nlong] partial minima of the long rows (INF between steps)
  uint64_t reg_in = 0;            // in-edges of the regular rows
  uint32_t max_w = 0;             // largest weight: pull steps need INF + w to stay in uint32
  uint32_t min_w = 0;             // smallest weight of a regular row's in-edge
  uint32_t* by_id = nullptr;      // [nslots] distances reordered by id before they leave the device
  unsigned long long* state = nullptr;  // the iteration loop's state (kSt* slots), device side
  DeviceLoop* loop = nullptr;     // the device-driven loop graph (built on first use)
};

// Loop state slots (unsigned long long each).
enum : int {
  kStIter = 0,      // iterations, counted as the reference counts them
  kStExamined,      // edges relaxed or gathered
  kStStatus,        // 1: the iteration limit was reached
  kStFirst,         // 1 until the first decision (the root's frontier is in kStNlist0 / kStDeg0)
  kStNlist0,        // the root's frontier: 1 if it scatters
  kStDeg0,          // the root's regular out-degree
  kStMode,          // the body chosen last: kPull, kPush or kDone
  kStSrcRoot,       // the root's position if it is a source (the sink pass reads it), else ~0
  kStFrontDeg,      // the chosen step's frontier out-degree sum
  kStNlist,         // the chosen step's frontier: vertices with regular out-edges
  kStPulls,         // pull steps run
  kStPushes,        // push steps run
  kStFmin,          // the chosen step's frontier minimum (what the pull's settled test reads)
  kStSlots = 16
};
enum : unsigned { kPull = 0, kPush = 1, kDone = 2 };

static void sssp_scratch_free(void* p)
{
  SsspScratch* s = (SsspScratch*) p;
  if (s->hctr) cudaFreeHost(s->hctr);
  delete s->loop;
  delete s;
}

__global__ void k_sssp_init(uint32_t N, uint32_t* dist, uint32_t* msg, uint32_t* fmsg)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x)
  {
    dist[p] = kInf;
    msg[p] = kInf;
    fmsg[p] = kInf;
  }
}

// The root (an id; none if it is outside the graph): distance 0, scattered
// (msg 0); regular and source vertices scatter, so they form the first
// frontier (even with no regular out-edge: the first iteration runs).
__global__ void k_sssp_root(uint32_t root, uint32_t N, const uint32_t* __restrict__ pos_of_id,
                            const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ reg_end, uint32_t nreg,
                            uint32_t src_base, uint32_t iso_base, uint32_t* dist, uint32_t* msg, uint32_t* fbits,
                            unsigned long long* state)
{
  for (int k = 0; k < kStSlots; k++) state[k] = 0;
  state[kStFirst] = 1;
  state[kStSrcRoot] = ~0ull;
  if (root >= N) return;
  const uint32_t rp = pos_of_id[root];
  const bool src = rp >= src_base && rp < iso_base;
  dist[rp] = 0;
  msg[rp] = 0;
  if (src) state[kStSrcRoot] = rp;
  if (rp < nreg || src)
  {
    fbits[rp >> 5] = 1u << (rp & 31);
    state[kStNlist0] = 1;
    state[kStDeg0] = reg_end[rp] - ptr[rp];
  }
}

// Start of every iteration (one thread): reads the counters the last dense
// apply left (or the root's frontier), ends the loop as the reference's
// execute loop does (nothing activated; or activated vertices with no
// regular out-edge, which take one more, empty iteration), and otherwise
// counts the iteration and picks pull (frontier out-degree sum above the
// regular rows' in-edges / divisor, after the first iteration, with weights
// that keep INF + w in uint32) or push.
// It also clears the counters the step's kernels accumulate into (the dense
// apply's, keeping the frontier minimum for the pull in the state; the push
// split's), so that no memset node sits between the iterations.
__global__ void k_sssp_decide(unsigned long long* state, unsigned long long* ctr, unsigned long long* fctr,
                              uint64_t reg_in, uint32_t max_w, double divisor, uint64_t limit,
                              cudaGraphConditionalHandle cont, cudaGraphConditionalHandle mode)
{
  unsigned long long it = state[kStIter], nlist, deg;
  bool done = false;
  if (state[kStFirst])
  {
    state[kStFirst] = 0;
    nlist = state[kStNlist0];
    deg = state[kStDeg0];
  }
  else
  {
    deg = ctr[1];
    nlist = ctr[2];
    if (ctr[0] == 0) done = true;
    else if (nlist == 0)
    {
      it++;  // the next iteration runs with messages that reach no regular row
      done = true;
    }
  }
  unsigned m = kDone;
  if (!done)
  {
    if (it > limit) state[kStStatus] = 1;
    else
    {
      it++;
      if (nlist)
        m = it > 1 && max_w <= 0x80000000u && (double) deg * divisor > (double) reg_in ? kPull : kPush;
    }
  }
  state[kStIter] = it;
  state[kStMode] = m;
  state[kStFrontDeg] = deg;
  state[kStNlist] = nlist;
  state[kStFmin] = ctr[5];
  ctr[0] = ctr[1] = ctr[2] = 0;
  ctr[5] = ~0ull;  // the next frontier's minimum
  fctr[0] = fctr[1] = 0;
  if (m == kPull)
  {
    state[kStExamined] += reg_in;
    state[kStPulls]++;
  }
  else if (m == kPush)
  {
    state[kStExamined] += deg;
    state[kStPushes]++;
  }
  loop_set(cont, m != kDone);
  loop_set(mode, m);
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

__device__ __forceinline__ void relax(uint32_t v, uint32_t cand, bool valid, uint32_t* dist)
{
  if (valid && cand < dist[v]) atomicMin(&dist[v], cand);  // result unused: a reduction in L2
}

// Relaxation over a split frontier: hubs first (all warps share each hub's
// edges), then one warp per small vertex.  Messages are the distances the
// frontier vertices held when they were activated (msg), as the reference's
// scatter values are.
__global__ void __launch_bounds__(256)
k_sssp_push(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ reg_end, const uint32_t* __restrict__ row,
            const uint32_t* __restrict__ w, const uint32_t* __restrict__ small, const uint32_t* __restrict__ big,
            const uint32_t* __restrict__ big_task0, const unsigned long long* __restrict__ fctr,
            const uint32_t* __restrict__ msg, uint32_t* dist)
{
  const uint32_t nsmall = (uint32_t) fctr[0];
  const uint32_t nbig = hub_count(fctr[1]), ntasks = hub_tasks(fctr[1]);
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
    for (uint32_t i = b + lane; i < e; i += 32) relax(row[i], mu + w[i], true, dist);
  }
  for (uint32_t f = warp; f < nsmall; f += nwarps)
  {
    const uint32_t u = small[f];
    const uint32_t mu = msg[u];
    const uint32_t b = ptr[u], e = reg_end[u];
    for (uint32_t i = b + lane; i < e; i += 32) relax(row[i], mu + w[i], true, dist);
  }
}

// After an iteration: the regular rows whose distance fell below their
// message were activated.  They scatter (msg = dist) and form the next
// frontier: one bit per vertex (a warp writes a whole word, so every word of
// the bitmap is rewritten) and the pull step's message array (fmsg: msg for
// the frontier, INF elsewhere); the counters get the frontier's size, its
// regular out-degree sum, how many of it have regular out-edges, and its
// smallest message.
__global__ void __launch_bounds__(256)
k_sssp_dense_apply(uint32_t nreg, uint32_t words, const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ reg_end,
                   const uint32_t* __restrict__ dist, uint32_t* msg, uint32_t* fmsg, uint32_t* fbits,
                   unsigned long long* ctr)
{
  const uint32_t lane = threadIdx.x & 31;
  unsigned long long deg = 0, cnt = 0, out = 0;
  uint32_t fmin = 0xFFFFFFFFu;
  const uint32_t nth = gridDim.x * blockDim.x;
  for (uint32_t v0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); v0 < words * 32u; v0 += nth)
  {
    const uint32_t v = v0 + lane;
    bool act = false;
    if (v < nreg)
    {
      const uint32_t dv = dist[v];
      act = dv < msg[v];
      fmsg[v] = act ? dv : kInf;
      if (act)
      {
        msg[v] = dv;
        const uint32_t d = reg_end[v] - ptr[v];
        deg += d;
        cnt++;
        out += d != 0;
        fmin = min(fmin, dv);
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, act);
    if (lane == 0) fbits[v0 >> 5] = m;
  }
  cnt = block_sum_u64(cnt);
  deg = block_sum_u64(deg);
  out = block_sum_u64(out);
  fmin = block_min_u32(fmin);
  if (threadIdx.x == 0)
  {
    if (cnt) atomicAdd(&ctr[0], cnt);
    if (deg) atomicAdd(&ctr[1], deg);
    if (out) atomicAdd(&ctr[2], out);
    if (fmin != 0xFFFFFFFFu) atomicMin(&ctr[5], (unsigned long long) fmin);
  }
}

// Push steps only: the frontier bitmap into the split lists (vertices with
// up to kBigDeg regular out-edges, appended a warp at a time; hubs with their
// edge tasks).
__global__ void __launch_bounds__(256)
k_sssp_split(const uint32_t* __restrict__ fbits, uint32_t words, const uint32_t* __restrict__ ptr,
             const uint32_t* __restrict__ reg_end, uint32_t* small, uint32_t* big, uint32_t* big_task0,
             unsigned long long* fctr)
{
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nth = gridDim.x * blockDim.x;
  for (uint32_t w0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); w0 < words; w0 += nth)
  {
    const uint32_t w = w0 + lane;
    uint32_t bits = w < words ? fbits[w] : 0u, c = 0;
    for (uint32_t x = bits; x; x &= x - 1)
    {
      const uint32_t v = w * 32 + (__ffs(x) - 1);
      const uint32_t d = reg_end[v] - ptr[v];
      if (d > kBigDeg) hub_append(v, d, big, big_task0, &fctr[1]);
      else c += d != 0;
    }
    uint32_t incl = c;
    for (int o = 1; o < 32; o <<= 1)
    {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= (uint32_t) o) incl += t;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    if (!total) continue;
    uint32_t base = 0;
    if (lane == 31) base = (uint32_t) atomicAdd(&fctr[0], (unsigned long long) total);
    base = __shfl_sync(0xffffffffu, base, 31) + incl - c;
    for (uint32_t x = bits; x; x &= x - 1)
    {
      const uint32_t v = w * 32 + (__ffs(x) - 1);
      const uint32_t d = reg_end[v] - ptr[v];
      if (d && d <= kBigDeg) small[base++] = v;
    }
  }
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

__global__ void __launch_bounds__(256)
k_sssp_pull(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, const uint32_t* __restrict__ w,
            uint32_t nreg, const uint32_t* __restrict__ task_row, const uint32_t* __restrict__ task_begin,
            uint32_t ntasks, uint32_t task_warps, uint32_t* ymin, const uint32_t* __restrict__ fmsg,
            uint32_t* dist, const uint32_t* __restrict__ long_rows, const unsigned long long* __restrict__ fmin_ptr,
            uint32_t min_w)
{
  const unsigned long long fmin = *fmin_ptr;  // the frontier's smallest message
  // Every candidate of this step is a frontier message plus a weight, so at
  // least fmin + min_w: a row already at or below that cannot be lowered and
  // its in-edges are not read (the result is the same).
  const uint32_t settled =
      fmin == ~0ull ? 0u : (fmin + min_w < kInf ? (uint32_t) (fmin + min_w) : kInf);
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp < task_warps)
  {
    // long rows: each task's minimum goes to the row's partial slot
    for (uint32_t t = warp; t < ntasks; t += task_warps)
    {
      const uint32_t k = task_row[t];  // index into the long-row list
      if (dist[long_rows[k]] <= settled) continue;
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
    uint32_t y = kInf, dv = 0;
    bool mine = false;
    if (v < nreg)
    {
      const uint32_t b = ptr[v], e = ptr[v + 1];
      dv = dist[v];
      mine = e - b <= kPullLong && dv > settled;
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
    if (mine && sub == 0 && y < dv) dist[v] = y;
  }
}

// Long rows after a pull step: apply the partial minimum, reset it.
__global__ void k_sssp_pull_long(const uint32_t* __restrict__ long_rows, uint32_t nlong, uint32_t* ymin, uint32_t* dist)
{
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nlong; k += gridDim.x * blockDim.x)
  {
    const uint32_t y = ymin[k];
    if (y == kInf) continue;
    ymin[k] = kInf;
    const uint32_t v = long_rows[k];
    if (y < dist[v]) dist[v] = y;
  }
}

__global__ void k_sssp_long_rows(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ w, uint32_t nreg,
                                 uint32_t* list, unsigned long long* n, unsigned long long* edges, unsigned int* maxw,
                                 unsigned int* minw)
{
  unsigned long long s = 0;
  unsigned int mw = 0, lw = 0xFFFFFFFFu;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nreg; v += gridDim.x * blockDim.x)
  {
    const uint32_t d = ptr[v + 1] - ptr[v];
    s += d;
    for (uint32_t i = ptr[v]; i < ptr[v + 1]; i++)
    {
      mw = max(mw, w[i]);
      lw = min(lw, w[i]);
    }
    if (d > kPullLong) list[atomicAdd(n, 1ull)] = v;
  }
  for (int o = 16; o > 0; o >>= 1)
  {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    mw = max(mw, __shfl_xor_sync(0xffffffffu, mw, o));
    lw = min(lw, __shfl_xor_sync(0xffffffffu, lw, o));
  }
  if ((threadIdx.x & 31) == 0)
  {
    if (s) atomicAdd(edges, s);
    if (mw) atomicMax(maxw, mw);
    if (lw != 0xFFFFFFFFu) atomicMin(minw, lw);
  }
}

// A step pulls when its frontier's out-degree sum exceeds the regular rows'
// in-edges / kPullDivisor (measured on R-MAT s22: 2 and 4 give 1.90 ms per
// call, 6 to 16 give 2.16-2.18 ms).
static constexpr double kPullDivisor = 4.0;

// Sink pass: y = min over in-neighbours (regular: final dist; the root if it
// is a source: its message 0) of msg + w; dist = min(dist, y).
__global__ void k_sssp_sinks(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col,
                             const uint32_t* __restrict__ w, uint32_t nreg, uint32_t nsink,
                             const unsigned long long* __restrict__ state, uint32_t* dist)
{
  const uint32_t src_root = (uint32_t) state[kStSrcRoot];
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
  LA3G_TRY(galloc(G, &ss->reg_end, N));
  LA3G_TRY(galloc(G, &ss->small[0], N));
  LA3G_TRY(galloc(G, &ss->big[0], N));
  LA3G_TRY(galloc(G, &ss->big_task0[0], N));
  LA3G_TRY(galloc(G, &ss->ctr, 8));
  LA3G_TRY(galloc(G, &ss->fctr, 2));
  LA3G_TRY(galloc(G, &ss->fbits, (size_t) N / 32 + 2));
  LA3G_TRY(galloc(G, &ss->by_id, N));
  LA3G_TRY(galloc(G, &ss->state, kStSlots));
  LA3G_CUDA(cudaHostAlloc(&ss->hctr, kStSlots * sizeof(unsigned long long), cudaHostAllocDefault));
  k_sssp_reg_end<<<grid_for(N, 256), 256, 0, G->stream>>>(G->g.out_ptr, G->g.out_row, N, G->g.nreg, ss->reg_end);
  LA3G_LAUNCHED();
  LA3G_TRY(galloc(G, &ss->long_rows, std::max<uint32_t>(G->g.nreg, 1)));
  LA3G_TRY(galloc(G, &ss->fmsg, N));
  LA3G_CUDA(cudaMemsetAsync(ss->ctr, 0, 8 * sizeof(unsigned long long), G->stream));
  LA3G_CUDA(cudaMemsetAsync(ss->ctr + 3, 0xFF, sizeof(unsigned long long), G->stream));
  k_sssp_long_rows<<<grid_for(G->g.nreg, 256), 256, 0, G->stream>>>(G->g.in_ptr, G->g.in_w, G->g.nreg, ss->long_rows,
                                                                     ss->ctr, ss->ctr + 1, (unsigned int*) (ss->ctr + 2),
                                                                     (unsigned int*) (ss->ctr + 3));
  LA3G_LAUNCHED();
  LA3G_CUDA(cudaMemcpyAsync(ss->hctr, ss->ctr, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, G->stream));
  LA3G_CUDA(cudaStreamSynchronize(G->stream));
  ss->nlong = (uint32_t) ss->hctr[0];
  ss->reg_in = ss->hctr[1];
  ss->max_w = (uint32_t) ss->hctr[2];
  ss->min_w = (uint32_t) ss->hctr[3];
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

// One iteration's body, k = kPull or kPush: the relaxation step, then the
// dense apply that forms the next frontier and its counters.  `deg` and
// `nlist` (the frontier's out-degree sum and size) only size the profile
// entries' bytes; the kernels read every count they need on the device.
static int sssp_body(la3g_graph* G, SsspScratch* ss, cudaStream_t s, unsigned k, double deg, double nlist)
{
  DevGraph& g = G->g;
  const uint32_t words = g.nslots / 32 + 1;
  if (k == kPull)
  {
    // in-edges of every regular row (index + weight), the frontier
    // messages of their columns, one dist read per row
    ProfileScope p("sssp_pull", s, 8.0 * ss->reg_in + 8.0 * ss->reg_in + 8.0 * g.nreg);
    // warps split between long-row tasks and short rows in proportion to their in-edges
    const uint32_t all_warps = num_sms() * 8 * 8;
    const uint32_t task_warps =
        ss->ntasks ? std::min<uint32_t>(ss->ntasks, std::max<uint32_t>(1, (uint32_t) ((double) all_warps *
                                                                                        ss->task_edges /
                                                                                        std::max<uint64_t>(ss->reg_in, 1))))
                   : 0;
    k_sssp_pull<<<num_sms() * 8, 256, 0, s>>>(g.in_ptr, g.in_col, g.in_w, g.nreg, ss->task_row, ss->task_begin,
                                              ss->ntasks, task_warps, ss->ymin, ss->fmsg, ss->dist, ss->long_rows,
                                              ss->state + kStFmin, ss->min_w);
    LA3G_LAUNCHED();
    if (ss->nlong)
    {
      k_sssp_pull_long<<<grid_for(ss->nlong, 256), 256, 0, s>>>(ss->long_rows, ss->nlong, ss->ymin, ss->dist);
      LA3G_LAUNCHED();
      tls_launches++;
    }
  }
  else
  {
    k_sssp_split<<<grid_for(words, 256), 256, 0, s>>>(ss->fbits, words, g.out_ptr, ss->reg_end, ss->small[0],
                                                      ss->big[0], ss->big_task0[0], ss->fctr);
    LA3G_LAUNCHED();
    tls_launches++;
    ProfileScope p("sssp_push", s, 8.0 * deg + 12.0 * nlist);
    k_sssp_push<<<num_sms() * 8, 256, 0, s>>>(g.out_ptr, ss->reg_end, g.out_row, g.out_w, ss->small[0], ss->big[0],
                                              ss->big_task0[0], ss->fctr, ss->msg, ss->dist);
    LA3G_LAUNCHED();
  }
  k_sssp_dense_apply<<<grid_for((uint64_t) words * 32, 256, num_sms() * 4), 256, 0, s>>>(
      g.nreg, words, g.out_ptr, ss->reg_end, ss->dist, ss->msg, ss->fmsg, ss->fbits, ss->ctr);
  LA3G_LAUNCHED();
  tls_launches++;
  return LA3G_OK;
}

// Iteration limit: with non-negative weights every distance is final after
// at most N + 1 iterations (Bellman-Ford), so a loop past N + 2 is a fault.
static uint64_t sssp_limit(const DevGraph& g) { return (uint64_t) g.nslots + 2; }

static int sssp_decide(la3g_graph* G, SsspScratch* ss, cudaStream_t s, cudaGraphConditionalHandle cont,
                       cudaGraphConditionalHandle mode)
{
  k_sssp_decide<<<1, 1, 0, s>>>(ss->state, ss->ctr, ss->fctr, ss->reg_in, ss->max_w, kPullDivisor, sssp_limit(G->g),
                                cont, mode);
  LA3G_LAUNCHED();
  tls_launches++;
  return LA3G_OK;
}

// Runs SSSP from `root` with the distances left on the device (positions).
// The iterations run as one device-driven graph (no host round trip per
// iteration); with profiling on they are stepped from the host instead, so
// that each kernel is timed.
static int sssp_run(la3g_graph* G, SsspScratch* ss, uint32_t root, la3g_stats* st)
{
  DevGraph& g = G->g;
  cudaStream_t s = G->stream;
  const uint32_t N = g.nslots;
  const uint32_t words = N / 32 + 1;
  k_sssp_init<<<grid_for(N, 256), 256, 0, s>>>(N, ss->dist, ss->msg, ss->fmsg);
  LA3G_LAUNCHED();
  LA3G_CUDA(cudaMemsetAsync(ss->fbits, 0, (size_t) words * 4, s));
  k_sssp_root<<<1, 1, 0, s>>>(root, N, g.pos_of_id, g.out_ptr, ss->reg_end, g.nreg, g.src_base(), g.iso_base(),
                              ss->dist, ss->msg, ss->fbits, ss->state);
  LA3G_LAUNCHED();
  tls_launches += 2;
  if (!profile_enabled())
  {
    if (!ss->loop)
    {
      ss->loop = new (std::nothrow) DeviceLoop();
      if (!ss->loop) return set_error(LA3G_ENOMEM, "out of host memory");
      const int rc = device_loop_build(
          ss->loop, 2,
          [&](cudaStream_t c, cudaGraphConditionalHandle cont, cudaGraphConditionalHandle mode) {
            return sssp_decide(G, ss, c, cont, mode);
          },
          [&](cudaStream_t c, int k) { return sssp_body(G, ss, c, (unsigned) k, 0.0, 0.0); });
      if (rc != LA3G_OK)
      {
        delete ss->loop;
        ss->loop = nullptr;
        return rc;
      }
    }
    LA3G_CUDA(cudaGraphLaunch(ss->loop->exec, s));
  }
  else
  {
    for (;;)
    {
      LA3G_TRY(sssp_decide(G, ss, s, 0, 0));
      LA3G_CUDA(cudaMemcpyAsync(ss->hctr, ss->state, kStSlots * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
      LA3G_CUDA(cudaStreamSynchronize(s));
      const unsigned m = (unsigned) ss->hctr[kStMode];
      if (m == kDone) break;
      LA3G_TRY(sssp_body(G, ss, s, m, (double) ss->hctr[kStFrontDeg], (double) ss->hctr[kStNlist]));
    }
  }
  if (g.nsink)
  {
    // the sink rows' in-edges only (index + weight, and the column's
    // distance), their offsets and the distance read and written
    const double sink_in = (double) (g.nent - ss->reg_in);
    ProfileScope p("sssp_sinks", s, 12.0 * sink_in + 12.0 * g.nsink);
    k_sssp_sinks<<<grid_for(g.nsink, 256), 256, 0, s>>>(g.in_ptr, g.in_col, g.in_w, g.nreg, g.nsink, ss->state,
                                                         ss->dist);
    LA3G_LAUNCHED();
  }
  LA3G_CUDA(cudaMemcpyAsync(ss->hctr, ss->state, kStSlots * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  LA3G_CUDA(cudaStreamSynchronize(s));
  if (ss->hctr[kStStatus]) return set_error(LA3G_ETIMEOUT, "sssp did not converge");
  if (ss->loop && !profile_enabled())
  {
    // the graph's launches: one decide per pass, each body's kernels per step
    const uint64_t passes = ss->hctr[kStPulls] + ss->hctr[kStPushes] + 1;
    tls_launches += (uint32_t) (passes + ss->hctr[kStPulls] * ss->loop->body_launches[kPull] +
                                ss->hctr[kStPushes] * ss->loop->body_launches[kPush]);
  }
  if (st)
  {
    st->iterations = (uint32_t) ss->hctr[kStIter];
    st->edges_examined = ss->hctr[kStExamined];
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
