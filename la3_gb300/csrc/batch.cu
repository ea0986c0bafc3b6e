// Batched multi-source BFS and SSSP.  The reference runs one root per
// VertexProgram (bfs.cpp:11-37, sssp.cpp:11-37); here a batch of roots runs
// together and every root's result equals what la3g_bfs / la3g_sssp return
// for it alone.
//
// BFS: 64 roots per uint64 word, W = ceil(R / 64) words per vertex (vertex-
// major, so the W words of a vertex are contiguous).  A level is a bit-
// parallel SpMM over the OR semiring:
//     next[v][w] = (OR over neighbours u of front[u][w]) & ~visited[v][w]
// run bottom-up (pull) when the frontier is dense and top-down (push, an
// atomicOr per edge and word) when it is sparse.  Per-word "alive" masks
// record which roots still discovered something; words whose roots are all
// finished are skipped (done-masks).  Levels run either as a CUDA graph of
// one level replayed from the host (the level number and buffer parity live
// in device memory, so one captured graph serves every level), or inside one
// persistent cooperative kernel with a grid barrier whose waits are bounded
// (a barrier that waits too long records an error and every block returns).
// BFS levels are order-free, so hops equal the single-root runs; a batch
// whose BFS would exceed 254 levels (where the reference's uint8 hops wrap)
// is rerun root by root with la3g_bfs.
//
// SSSP: per-root distances, vertex-major ([vertex][root]); a frontier bit
// per (vertex, root); an iteration relaxes the out-edges of every active
// (vertex, root) into regular rows with atomicMin, then the sink rows are
// computed once, as in the single-root run.  With every edge weight at most
// (2^31 - 1) / n no distance can reach INF and no sum can wrap, so the fixed
// point equals the single-root result whatever the relaxation order; batches
// on graphs that do not satisfy that bound are run root by root.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "la3g_internal.h"
#include "frontier.cuh"
#include "lanes.cuh"

namespace la3g {


struct BatchConfig
{
  int mode = 0;          // 0 = per-level CUDA graph, 1 = persistent cooperative kernel
  int block = 256;       // threads per block of the level kernels
  double push_frac = 0.05;  // push when frontier edges * words < push_frac * m * words
  bool tuned = false;
};

// Polls a block of the persistent kernel makes at a grid barrier before it
// gives up (sets the error word, every block leaves, the call returns
// LA3G_ETIMEOUT); la3g_batch_set_wait_limit changes it per graph.
static constexpr long long kDefaultWaitPolls = 1ll << 26;

struct BatchScratch
{
  long long wait_polls = kDefaultWaitPolls;  // grid-barrier poll limit of the persistent kernel
  uint32_t cap_r = 0;        // roots the buffers were sized for
  uint64_t* vis = nullptr;   // [N][W]
  uint64_t* buf[2] = {nullptr, nullptr};  // frontier / next, [N][W]
  uint64_t* alive[2] = {nullptr, nullptr};  // [W] per-word "discovered something" masks
  uint8_t* hops = nullptr;   // [N][W * 64] by position (vertex-major)
  uint32_t* rpos = nullptr;  // root positions
  uint32_t* active = nullptr;  // push: active (vertex, word) pairs of small vertices
  uint32_t* phub = nullptr;    // push: pairs of hub vertices, and their first task numbers
  uint32_t* phub_t0 = nullptr;
  unsigned long long* ctr = nullptr;  // [0] new bits, [1] small pairs, [2] frontier edges*words, [3] level,
                                      // [4] levels that found something, [5] hub slots / tasks (packed)
  unsigned long long* hctr = nullptr;
  unsigned int* bar = nullptr;        // grid barrier: count, generation
  int* err = nullptr;
  cudaGraphExec_t pull_exec = nullptr;
  uint32_t pull_exec_w = 0, pull_exec_block = 0;
  cudaStream_t pull_exec_stream = nullptr;
  BatchConfig cfg;                           // set by hand, or the default
  std::vector<std::pair<uint32_t, BatchConfig>> tuned;  // autotuned, by words per batch
  // SSSP
  uint32_t cap_sr = 0;
  uint32_t* sdist = nullptr;   // [N][R]
  uint64_t* sfront[2] = {nullptr, nullptr};  // [N][W]
  uint32_t* sact[2] = {nullptr, nullptr};    // active (vertex, word) pairs, N*W each
  uint32_t* shub[2] = {nullptr, nullptr};    // pairs of high-degree vertices, N*W each
  uint32_t* shub_t0[2] = {nullptr, nullptr}; // their first task numbers
  uint32_t* reg_end = nullptr;
  uint32_t max_w = 0;
  uint32_t max_reg_deg = 0;    // most regular out-edges of one vertex
  bool max_w_known = false;
  uint32_t sssp_delta = 0;     // distance window width; 0 = automatic, kNoWindow = none
};

static void batch_scratch_free(void* p)
{
  BatchScratch* b = (BatchScratch*) p;
  if (b->pull_exec) cudaGraphExecDestroy(b->pull_exec);
  if (b->hctr) cudaFreeHost(b->hctr);
  delete b;
}

// ------------------------------------------------------------------ BFS

__global__ void k_ms_init(uint32_t N, uint32_t W, uint32_t R, uint64_t* vis, uint64_t* front, uint64_t* next)
{
  const uint64_t NW = (uint64_t) N * W;
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < NW; i += (uint64_t) gridDim.x * blockDim.x)
  {
    const uint32_t w = (uint32_t) (i % W);
    // roots beyond R in the last word count as already visited
    const uint32_t lo = w * 64;
    uint64_t pad = 0;
    if (lo + 64 > R) pad = ~0ull << (R - lo);
    vis[i] = pad;
    front[i] = 0;
    next[i] = 0;
  }
}

__global__ void k_ms_roots(const uint32_t* __restrict__ rpos, uint32_t R, uint32_t N, uint32_t W, uint64_t* vis,
                           uint64_t* front, uint8_t* hops, uint64_t* alive)
{
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < R; r += gridDim.x * blockDim.x)
  {
    const uint32_t p = rpos[r];
    if (p >= N) continue;  // out-of-range root: nothing matches, all 255
    const uint32_t w = r / 64;
    const uint64_t bit = 1ull << (r % 64);
    atomicOr((unsigned long long*) &vis[(uint64_t) p * W + w], (unsigned long long) bit);
    atomicOr((unsigned long long*) &front[(uint64_t) p * W + w], (unsigned long long) bit);
    atomicOr((unsigned long long*) &alive[w], (unsigned long long) bit);
    hops[((uint64_t) p * W + w) * 64 + r % 64] = 0;
  }
}

// Bottom-up level over (vertex, word) pairs (pull_scan: a lane per pair,
// the warp for long in-edge lists).  Reads the level from ctr[3]; front /
// next alternate with its parity.  tid / nthreads count whole warps.
__device__ __forceinline__ void ms_pull_body(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col,
                                             uint32_t nrows, uint32_t N, uint32_t W, uint64_t* vis, uint64_t* const* buf,
                                             uint64_t* const* alive, uint8_t* hops, unsigned long long* ctr,
                                             uint64_t tid, uint64_t nthreads)
{
  const uint32_t level = (uint32_t) ctr[3];
  const uint64_t* __restrict__ front = buf[level & 1];
  uint64_t* next = buf[(level + 1) & 1];
  const uint64_t* alive_now = alive[level & 1];
  uint64_t* alive_next = alive[(level + 1) & 1];
  const uint8_t hop = (uint8_t) (level + 1);
  unsigned long long cnt = 0;
  const uint64_t NW = (uint64_t) nrows * W;
  // a warp takes 32 consecutive pairs at a time (pull_scan is warp-collective)
  const int lane = threadIdx.x & 31;
  for (uint64_t base = (tid >> 5) * 32; base < NW; base += (nthreads >> 5) * 32)
  {
    const uint64_t i = base + lane;
    const bool ok = i < NW;
    const uint32_t v = ok ? (uint32_t) (i / W) : 0, w = ok ? (uint32_t) (i % W) : 0;
    const uint64_t seen = ok ? vis[i] : ~0ull;
    const uint64_t want = ok ? ~seen & alive_now[w] : 0;
    const uint64_t nb = pull_scan(v, w, W, want, ptr, col, front, lane);
    if (!ok) continue;
    next[i] = nb;
    if (nb)
    {
      vis[i] = seen | nb;
      cnt += __popcll(nb);
      atomicOr((unsigned long long*) &alive_next[w], (unsigned long long) nb);
      hops_record(hops + i * 64, nb, hop);
    }
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&ctr[0], cnt);
}

struct BufPair
{
  uint64_t* p[2];
};

__global__ void k_ms_pull(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, uint32_t nrows, uint32_t N,
                          uint32_t W, uint64_t* vis, BufPair buf, BufPair alive, uint8_t* hops, unsigned long long* ctr)
{
  ms_pull_body(ptr, col, nrows, N, W, vis, buf.p, alive.p, hops, ctr, (uint64_t) blockIdx.x * blockDim.x + threadIdx.x,
               (uint64_t) gridDim.x * blockDim.x);
}

// End of a level: clear the alive mask two levels ahead, advance the level.
__global__ void k_ms_advance(uint32_t W, BufPair alive, unsigned long long* ctr)
{
  const uint32_t level = (uint32_t) ctr[3];
  uint64_t* stale = alive.p[level & 1];  // becomes the "next" mask of the next level
  for (uint32_t w = threadIdx.x; w < W; w += blockDim.x) stale[w] = 0;
  __syncthreads();
  if (threadIdx.x == 0) ctr[3] = level + 1;
}

// Top-down level: list the nonzero frontier words, push them to neighbours
// (masked by visited), then apply.
__global__ void k_ms_list(uint32_t nrows, uint32_t W, BufPair buf, const uint32_t* __restrict__ ptr, PairList out,
                          const unsigned long long* __restrict__ ctr)
{
  const uint32_t level = (uint32_t) ctr[3];
  const uint64_t* front = buf.p[level & 1];
  const uint64_t NW = (uint64_t) nrows * W;
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < NW; i += (uint64_t) gridDim.x * blockDim.x)
    if (front[i])
    {
      const uint32_t v = (uint32_t) (i / W);
      bs_list_pair((uint32_t) i, ptr[v + 1] - ptr[v], out);
    }
}

__global__ void k_ms_push(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, uint32_t W, BufPair buf,
                          const uint64_t* __restrict__ vis, PairList list, const unsigned long long* __restrict__ ctr)
{
  const uint32_t level = (uint32_t) ctr[3];
  ms_push_pairs(ptr, col, W, buf.p[level & 1], vis, buf.p[(level + 1) & 1], list);
}

__global__ void k_ms_apply(uint32_t nrows, uint32_t N, uint32_t W, uint64_t* vis, BufPair buf, BufPair alive,
                           uint8_t* hops, unsigned long long* ctr)
{
  const uint32_t level = (uint32_t) ctr[3];
  uint64_t* next = buf.p[(level + 1) & 1];
  uint64_t* alive_next = alive.p[(level + 1) & 1];
  const uint8_t hop = (uint8_t) (level + 1);
  unsigned long long cnt = 0;
  const uint64_t NW = (uint64_t) nrows * W;
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < NW; i += (uint64_t) gridDim.x * blockDim.x)
  {
    const uint64_t nb = next[i] & ~vis[i];
    next[i] = nb;
    if (nb)
    {
      vis[i] |= nb;
      cnt += __popcll(nb);
      atomicOr((unsigned long long*) &alive_next[i % W], (unsigned long long) nb);
      hops_record(hops + i * 64, nb, hop);
    }
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&ctr[0], cnt);
}

// The front buffer must be zero before it is reused as "next" two levels
// later; the pull kernel overwrites every word, the push path clears it.
__global__ void k_ms_clear(uint64_t n, BufPair buf, unsigned long long* ctr)
{
  const uint32_t level = (uint32_t) ctr[3];
  uint64_t* next = buf.p[(level + 1) & 1];
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
    next[i] = 0;
}

// Grid barrier for the persistent kernel: bounded spin (at most `limit`
// polls); on timeout the error word is set and every block leaves.
__device__ bool grid_barrier(unsigned int* bar, int* err, unsigned int nblocks, long long limit)
{
  __syncthreads();
  bool ok = true;
  if (threadIdx.x == 0)
  {
    volatile unsigned int* vgen = bar + 1;
    const unsigned int gen = *vgen;
    __threadfence();
    if (atomicAdd(bar, 1u) == nblocks - 1)
    {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    }
    else
    {
      long long spins = 0;
      while (*vgen == gen)
      {
        if (spins++ >= limit || *(volatile int*) err)
        {
          atomicExch(err, 1);
          ok = false;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __shared__ int s_ok;
  if (threadIdx.x == 0) s_ok = ok && !*(volatile int*) err;
  __syncthreads();
  return s_ok;
}

// All pull levels in one cooperative launch.
__global__ void k_ms_persistent(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, uint32_t nrows,
                                uint32_t N, uint32_t W, uint64_t* vis, BufPair buf, BufPair alive, uint8_t* hops,
                                unsigned long long* ctr, unsigned int* bar, int* err, uint32_t max_levels,
                                long long wait_limit)
{
  const uint64_t tid = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t nth = (uint64_t) gridDim.x * blockDim.x;
  for (uint32_t it = 0; it < max_levels; it++)
  {
    ms_pull_body(ptr, col, nrows, N, W, vis, buf.p, alive.p, hops, ctr, tid, nth);
    if (!grid_barrier(bar, err, gridDim.x, wait_limit)) return;
    const unsigned long long found = ctr[0];
    if (!grid_barrier(bar, err, gridDim.x, wait_limit)) return;
    if (blockIdx.x == 0)
    {
      const uint32_t level = (uint32_t) ctr[3];
      uint64_t* stale = alive.p[level & 1];
      for (uint32_t w = threadIdx.x; w < W; w += blockDim.x) stale[w] = 0;
      __syncthreads();
      if (threadIdx.x == 0)
      {
        ctr[3] = level + 1;
        ctr[4] += found ? 1 : 0;
        ctr[0] = 0;
      }
    }
    if (!grid_barrier(bar, err, gridDim.x, wait_limit)) return;
    if (!found) return;
  }
}

// Hops to out[root][id] in two passes, so that no pass gathers across the
// whole [N][W * 64] array: a tiled transpose by position (32 positions x 32
// roots per tile through shared memory; reads and writes move 32-byte runs)
// into tpos[root][position], then a gather by id inside one root's N-byte
// row, which stays in L2.
__global__ void __launch_bounds__(256) k_ms_out_pos(uint32_t N, uint32_t R, uint32_t W, const uint8_t* __restrict__ hops,
                                                    uint8_t* tpos)
{
  __shared__ uint8_t t[32][33];
  const uint32_t tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const uint32_t np = (N + 31) / 32, nr = (R + 31) / 32;
  const uint64_t RW = (uint64_t) W * 64;
  for (uint64_t tile = blockIdx.x; tile < (uint64_t) np * nr; tile += gridDim.x)
  {
    const uint32_t p0 = (uint32_t) (tile % np) * 32, r0 = (uint32_t) (tile / np) * 32;
    for (uint32_t k = ty; k < 32; k += 8)
    {
      const uint32_t p = p0 + k;
      t[k][tx] = p < N && r0 + tx < R ? hops[(uint64_t) p * RW + r0 + tx] : 255;
    }
    __syncthreads();
    for (uint32_t k = ty; k < 32; k += 8)
    {
      const uint32_t r = r0 + k, p = p0 + tx;
      if (r < R && p < N) tpos[(uint64_t) r * N + p] = t[tx][k];
    }
    __syncthreads();
  }
}

__global__ void k_ms_out_id(uint32_t N, uint32_t R, const uint32_t* __restrict__ pos_of_id, const uint8_t* __restrict__ tpos,
                            uint8_t* out)
{
  const uint64_t RN = (uint64_t) R * N;
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < RN; i += (uint64_t) gridDim.x * blockDim.x)
  {
    const uint64_t r = i / N;
    out[i] = tpos[r * N + pos_of_id[i - r * N]];
  }
}

static int batch_scratch(la3g_graph* G, BatchScratch** out)
{
  BatchScratch* b = (BatchScratch*) G->slot[kSlotBatch];
  if (!b)
  {
    b = new (std::nothrow) BatchScratch();
    if (!b) return set_error(LA3G_ENOMEM, "out of host memory");
    G->slot[kSlotBatch] = b;
    G->slot_free[kSlotBatch] = batch_scratch_free;
    LA3G_TRY(galloc(G, &b->ctr, 8));
    LA3G_TRY(galloc(G, &b->bar, 2));
    LA3G_TRY(galloc(G, &b->err, 1));
    LA3G_CUDA(cudaHostAlloc(&b->hctr, 8 * sizeof(unsigned long long), cudaHostAllocDefault));
  }
  *out = b;
  return LA3G_OK;
}

static int ms_bfs_alloc(la3g_graph* G, BatchScratch* b, uint32_t R)
{
  if (R <= b->cap_r) return LA3G_OK;
  const uint32_t N = G->g.nslots, W = (R + 63) / 64;
  // buffers sized for the new R; the old ones stay owned by the graph
  LA3G_TRY(galloc(G, &b->vis, (size_t) N * W));
  LA3G_TRY(galloc(G, &b->buf[0], (size_t) N * W));
  LA3G_TRY(galloc(G, &b->buf[1], (size_t) N * W));
  LA3G_TRY(galloc(G, &b->alive[0], W));
  LA3G_TRY(galloc(G, &b->alive[1], W));
  LA3G_TRY(galloc(G, &b->hops, (size_t) N * W * 64));
  LA3G_TRY(galloc(G, &b->rpos, R));
  LA3G_TRY(galloc(G, &b->active, (size_t) N * W));
  LA3G_TRY(galloc(G, &b->phub, (size_t) N * W));
  LA3G_TRY(galloc(G, &b->phub_t0, (size_t) N * W));
  b->cap_r = R;
  if (b->pull_exec)
  {
    cudaGraphExecDestroy(b->pull_exec);
    b->pull_exec = nullptr;
  }
  return LA3G_OK;
}

__global__ void k_root_pos(const uint32_t* __restrict__ ids, uint32_t R, uint32_t N, const uint32_t* __restrict__ pos_of_id,
                           uint32_t* out)
{
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < R; r += gridDim.x * blockDim.x)
    out[r] = ids[r] < N ? pos_of_id[ids[r]] : 0xFFFFFFFFu;
}

// Runs one batch; hops by position stay in b->hops.  Returns the level count
// in *levels; *wrap = true when some root would need more than 254 levels.
static int ms_bfs_run(la3g_graph* G, BatchScratch* b, const uint32_t* roots_host, uint32_t R, const BatchConfig& cfg,
                      uint32_t* levels, bool* wrap, uint64_t* edges_words)
{
  DevGraph& g = G->g;
  cudaStream_t s = G->stream;
  const uint32_t N = g.nslots, nrows = g.nrows(), W = (R + 63) / 64;
  LA3G_TRY(ms_bfs_alloc(G, b, R));
  BufPair buf{{b->buf[0], b->buf[1]}}, alive{{b->alive[0], b->alive[1]}};
  LA3G_CUDA(cudaMemcpyAsync(b->active, roots_host, (size_t) R * 4, cudaMemcpyHostToDevice, s));
  k_root_pos<<<grid_for(R, 256), 256, 0, s>>>(b->active, R, N, g.pos_of_id, b->rpos);
  LA3G_LAUNCHED();
  k_ms_init<<<num_sms() * 8, 256, 0, s>>>(N, W, R, b->vis, b->buf[0], b->buf[1]);
  LA3G_LAUNCHED();
  LA3G_CUDA(cudaMemsetAsync(b->hops, 0xFF, (size_t) N * W * 64, s));
  LA3G_CUDA(cudaMemsetAsync(b->alive[0], 0, (size_t) W * 8, s));
  LA3G_CUDA(cudaMemsetAsync(b->alive[1], 0, (size_t) W * 8, s));
  LA3G_CUDA(cudaMemsetAsync(b->ctr, 0, 8 * 8, s));
  k_ms_roots<<<grid_for(R, 256), 256, 0, s>>>(b->rpos, R, N, W, b->vis, b->buf[0], b->hops, b->alive[0]);
  LA3G_LAUNCHED();
  tls_launches += 4;
  *wrap = false;
  *edges_words = 0;
  const unsigned blocks = num_sms() * (2048 / cfg.block);
  if (cfg.mode == 1)
  {
    // persistent cooperative kernel (pull levels)
    int per_sm = 0;
    LA3G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ms_persistent, cfg.block, 0));
    int dev = 0, sms = num_sms();
    LA3G_CUDA(cudaGetDevice(&dev));
    LA3G_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    unsigned grid = (unsigned) std::max(1, per_sm) * (unsigned) sms;
    LA3G_CUDA(cudaMemsetAsync(b->bar, 0, 8, s));
    LA3G_CUDA(cudaMemsetAsync(b->err, 0, 4, s));
    const uint32_t* ptr = g.in_ptr;
    const uint32_t* col = g.in_col;
    uint64_t* vis = b->vis;
    uint8_t* hops = b->hops;
    unsigned long long* ctr = b->ctr;
    unsigned int* bar = b->bar;
    int* err = b->err;
    uint32_t maxl = 255;
    long long wait_limit = b->wait_polls;
    void* args[] = {(void*) &ptr, (void*) &col, (void*) &nrows, (void*) &N, (void*) &W, (void*) &vis, (void*) &buf,
                    (void*) &alive, (void*) &hops, (void*) &ctr, (void*) &bar, (void*) &err, (void*) &maxl,
                    (void*) &wait_limit};
    {
      ProfileScope p("msbfs_persistent", s, 0.0);
      LA3G_CUDA(cudaLaunchCooperativeKernel((void*) k_ms_persistent, grid, cfg.block, args, 0, s));
    }
    int herr = 0;
    LA3G_CUDA(cudaMemcpyAsync(&herr, b->err, 4, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaMemcpyAsync(b->hctr, b->ctr, 8 * 8, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    if (herr) return set_error(LA3G_ETIMEOUT, "batched BFS: a grid barrier wait ran out");
    *levels = (uint32_t) b->hctr[3];
    *wrap = b->hctr[3] >= 255;
    *edges_words = (uint64_t) *levels * g.nent * W;
    return LA3G_OK;
  }
  // per-level: the bottom-up level is one captured graph replayed each level
  if (!b->pull_exec || b->pull_exec_w != W || b->pull_exec_block != (uint32_t) cfg.block || b->pull_exec_stream != s)
  {
    if (b->pull_exec) cudaGraphExecDestroy(b->pull_exec);
    b->pull_exec = nullptr;
    cudaStream_t cap;
    LA3G_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t graph;
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess)
    {
      k_ms_pull<<<blocks, cfg.block, 0, cap>>>(g.in_ptr, g.in_col, nrows, N, W, b->vis, buf, alive, b->hops, b->ctr);
      k_ms_advance<<<1, 256, 0, cap>>>(W, alive, b->ctr);
      e = cudaStreamEndCapture(cap, &graph);
    }
    if (e == cudaSuccess)
    {
      e = cudaGraphInstantiate(&b->pull_exec, graph, 0);
      cudaGraphDestroy(graph);
    }
    cudaStreamDestroy(cap);
    if (e != cudaSuccess) return set_error(LA3G_ECUDA, "graph capture of the BFS level failed: %s", cudaGetErrorString(e));
    b->pull_exec_w = W;
    b->pull_exec_block = (uint32_t) cfg.block;
    b->pull_exec_stream = s;
  }
  uint64_t front_bits = 0;
  for (uint32_t level = 0; level < 255; level++)
  {
    // frontier popcount of level 0 = number of valid roots (approximate: R)
    const uint64_t fb = level == 0 ? R : front_bits;
    const bool push = (double) fb * ((double) g.nent / std::max<uint32_t>(1, nrows)) <
                      cfg.push_frac * (double) g.nent * 64.0 * W;
    LA3G_CUDA(cudaMemsetAsync(b->ctr, 0, 2 * 8, s));
    if (push)
    {
      ProfileScope p("msbfs_push", s, 0.0);
      const PairList pl{b->active, b->phub, b->phub_t0, b->ctr + 1, b->ctr + 5};
      LA3G_CUDA(cudaMemsetAsync(b->ctr + 5, 0, 8, s));
      k_ms_clear<<<blocks, cfg.block, 0, s>>>((uint64_t) N * W, buf, b->ctr);
      k_ms_list<<<blocks, cfg.block, 0, s>>>(nrows, W, buf, g.in_ptr, pl, b->ctr);
      k_ms_push<<<blocks, cfg.block, 0, s>>>(g.in_ptr, g.in_col, W, buf, b->vis, pl, b->ctr);
      k_ms_apply<<<blocks, cfg.block, 0, s>>>(nrows, N, W, b->vis, buf, alive, b->hops, b->ctr);
      k_ms_advance<<<1, 256, 0, s>>>(W, alive, b->ctr);
      LA3G_LAUNCHED();
      tls_launches += 4;
    }
    else
    {
      ProfileScope p("msbfs_pull", s, 0.0);
      LA3G_CUDA(cudaGraphLaunch(b->pull_exec, s));
      tls_launches += 1;
    }
    *edges_words += (uint64_t) g.nent * W;
    LA3G_CUDA(cudaMemcpyAsync(b->hctr, b->ctr, 4 * 8, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    front_bits = b->hctr[0];
    *levels = level + 1;
    if (front_bits == 0) return LA3G_OK;
  }
  *wrap = true;
  return LA3G_OK;
}

// ------------------------------------------------------------------ SSSP

__global__ void k_bs_init(uint64_t n, uint32_t* dist, uint64_t nw, uint64_t* f0, uint64_t* f1)
{
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
    dist[i] = kInfD;
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += (uint64_t) gridDim.x * blockDim.x)
  {
    f0[i] = 0;
    f1[i] = 0;
  }
}

__global__ void k_bs_roots(const uint32_t* __restrict__ rpos, uint32_t R, uint32_t N, uint32_t W, uint32_t nreg,
                           uint32_t src_base, uint32_t iso_base, uint32_t* dist, uint64_t* front)
{
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < R; r += gridDim.x * blockDim.x)
  {
    const uint32_t p = rpos[r];
    if (p >= N) continue;
    dist[(uint64_t) p * R + r] = 0;
    if (p < nreg || (p >= src_base && p < iso_base))
      atomicOr((unsigned long long*) &front[(uint64_t) p * W + r / 64], 1ull << (r % 64));
  }
}

// Sink rows once: min over regular in-neighbours' final distances and the
// root's message where the root is a source.
__global__ void k_bs_sinks(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, const uint32_t* __restrict__ wgt,
                           uint32_t nreg, uint32_t nsink, uint32_t R, const uint32_t* __restrict__ rpos,
                           uint32_t src_base, uint32_t iso_base, uint32_t* dist)
{
  const uint64_t n = (uint64_t) nsink * R;
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
  {
    const uint32_t v = nreg + (uint32_t) (i / R), r = (uint32_t) (i % R);
    const uint32_t rp = rpos[r];
    uint32_t y = kInfD;
    for (uint32_t e = ptr[v]; e < ptr[v + 1]; e++)
    {
      const uint32_t c = col[e];
      uint32_t cand;
      if (c < nreg) cand = dist[(uint64_t) c * R + r] + wgt[e];
      else if (c == rp && rp >= src_base && rp < iso_base) cand = wgt[e];
      else continue;
      y = min(y, cand);
    }
    uint32_t* d = &dist[(uint64_t) v * R + r];
    *d = min(*d, y);
  }
}

__global__ void k_bs_out(uint32_t N, uint32_t R, const uint32_t* __restrict__ id_of_pos, const uint32_t* __restrict__ dist,
                         uint32_t* out)
{
  const uint64_t n = (uint64_t) N * R;
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
  {
    const uint32_t p = (uint32_t) (i / R), r = (uint32_t) (i % R);
    out[(uint64_t) r * N + id_of_pos[p]] = dist[i];
  }
}

}  // namespace la3g

using namespace la3g;

extern "C" int la3g_bfs_batch(la3g_graph* G, const uint32_t* roots, uint32_t nroots, uint8_t* hops_out, la3g_stats* st)
{
  if (!G) return set_error(LA3G_EINVAL, "null graph");
  if (nroots == 0) return set_error(LA3G_EINVAL, "nroots must be > 0");
  if (!roots) return set_error(LA3G_EINVAL, "roots is null");
  DevGraph& g = G->g;
  if (g.directed()) return set_error(LA3G_EINVAL, "bfs needs an undirected graph");
  CallTimer T(G, st);
  BatchScratch* b = nullptr;
  LA3G_TRY(batch_scratch(G, &b));
  const uint32_t N = g.nslots;
  uint32_t levels = 0;
  bool wrap = false;
  uint64_t ew = 0;
  T.device_begin();
  // the configuration tuned for this many words if there is one (the nearest
  // tuned word count otherwise), else the hand-set / default one
  BatchConfig cfg = b->cfg;
  {
    const uint32_t W = (nroots + 63) / 64;
    uint32_t best = 0xFFFFFFFFu;
    for (const auto& t : b->tuned)
    {
      const uint32_t dist = t.first > W ? t.first - W : W - t.first;
      if (dist < best) { best = dist; cfg = t.second; }
    }
  }
  LA3G_TRY(ms_bfs_run(G, b, roots, nroots, cfg, &levels, &wrap, &ew));
  T.device_end();
  cudaStream_t s = G->stream;
  if (hops_out)
  {
    // the by-id rows go into the hop array itself (N x W x 64 >= nroots x N
    // bytes), which the next batch re-initialises
    DevBuf tpos;
    LA3G_TRY(tpos.alloc((size_t) nroots * N));
    k_ms_out_pos<<<num_sms() * 8, 256, 0, s>>>(N, nroots, (nroots + 63) / 64, b->hops, tpos.as<uint8_t>());
    LA3G_LAUNCHED();
    k_ms_out_id<<<num_sms() * 8, 256, 0, s>>>(N, nroots, g.pos_of_id, tpos.as<uint8_t>(), b->hops);
    LA3G_LAUNCHED();
    LA3G_CUDA(cudaMemcpyAsync(hops_out, b->hops, (size_t) nroots * N, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
  }
  LA3G_TRY(T.finish());
  if (wrap && hops_out)
  {
    // more than 254 levels: the reference's uint8 hops wrap; rerun the roots
    // one by one with the single-root path, which follows it exactly
    for (uint32_t r = 0; r < nroots; r++) LA3G_TRY(la3g_bfs(G, roots[r], hops_out + (size_t) r * N, nullptr, nullptr));
  }
  if (st)
  {
    st->iterations = levels;
    st->edges_examined = ew * 64;
  }
  return LA3G_OK;
}

static constexpr uint32_t kSsspChunk = 256;  // roots per device pass (bounds the [N][R] state)

// Default window width of the batched SSSP.  The window pays where degrees
// are even (ER 2^22 x16, weights 1-128, 256 roots: 248 ms with a window of
// 128 against 272 ms without; 64 and 256 give 257 / 282 ms) and costs where
// hubs already make the frontier converge in few iterations (R-MAT s22: 88
// against 75 ms), so it is on only when no vertex is a hub (more than kBigDeg
// regular out-edges), with the largest weight as its width.
static uint32_t sssp_auto_delta(uint32_t max_w, uint32_t max_reg_deg)
{
  return max_reg_deg <= kBigDeg ? std::max(max_w, 1u) : kNoWindow;
}

__global__ void k_max_reg_deg(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ reg_end, uint32_t N,
                              unsigned int* out)
{
  unsigned int m = 0;
  for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < N; u += gridDim.x * blockDim.x)
    m = max(m, reg_end[u] - ptr[u]);
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

static int sssp_batch_chunk(la3g_graph* G, BatchScratch* b, const uint32_t* roots, uint32_t R, uint32_t* dist_out,
                            uint32_t* iters_out);

extern "C" int la3g_sssp_batch(la3g_graph* G, const uint32_t* roots, uint32_t nroots, uint32_t* dist_out,
                               la3g_stats* st)
{
  if (!G) return set_error(LA3G_EINVAL, "null graph");
  if (nroots == 0) return set_error(LA3G_EINVAL, "nroots must be > 0");
  if (!roots) return set_error(LA3G_EINVAL, "roots is null");
  DevGraph& g = G->g;
  if (!g.directed() || !g.weighted() || (g.flags & (LA3G_REVERSE | LA3G_ACYCLIC | LA3G_BIPARTITE)))
    return set_error(LA3G_EINVAL, "sssp needs a graph loaded with LA3G_DIRECTED | LA3G_WEIGHTED");
  CallTimer T(G, st);
  LA3G_TRY(build_push_csr(G));
  BatchScratch* b = nullptr;
  LA3G_TRY(batch_scratch(G, &b));
  uint32_t iters = 0;
  T.device_begin();
  for (uint32_t r0 = 0; r0 < nroots; r0 += kSsspChunk)
  {
    const uint32_t R = std::min(kSsspChunk, nroots - r0);
    uint32_t it = 0;
    LA3G_TRY(sssp_batch_chunk(G, b, roots + r0, R, dist_out ? dist_out + (size_t) r0 * g.nslots : nullptr, &it));
    iters = std::max(iters, it);
  }
  T.device_end();
  LA3G_TRY(T.finish());
  if (st) st->iterations = iters;
  return LA3G_OK;
}

static int sssp_batch_chunk(la3g_graph* G, BatchScratch* b, const uint32_t* roots, uint32_t R, uint32_t* dist_out,
                            uint32_t* iters_out)
{
  DevGraph& g = G->g;
  cudaStream_t s = G->stream;
  const uint32_t N = g.nslots, W = (R + 63) / 64;
  if (!b->max_w_known)
  {
    DevBuf m;
    LA3G_TRY(m.alloc(8));
    LA3G_CUDA(cudaMemsetAsync(m.p, 0, 8, s));
    if (g.nent)
    {
      k_max_u32<<<grid_for(g.nent, 256), 256, 0, s>>>(g.out_w, g.nent, m.as<unsigned int>());
      LA3G_LAUNCHED();
    }
    LA3G_TRY(galloc(G, &b->reg_end, N));
    k_reg_end<<<grid_for(N, 256), 256, 0, s>>>(g.out_ptr, g.out_row, N, g.nreg, b->reg_end);
    LA3G_LAUNCHED();
    k_max_reg_deg<<<grid_for(N, 256), 256, 0, s>>>(g.out_ptr, b->reg_end, N, m.as<unsigned int>() + 1);
    LA3G_LAUNCHED();
    uint32_t hm[2] = {0, 0};
    LA3G_CUDA(cudaMemcpyAsync(hm, m.p, 8, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    b->max_w = hm[0];
    b->max_reg_deg = hm[1];
    b->max_w_known = true;
  }
  // Exact regardless of relaxation order only if no distance can reach INF.
  if ((uint64_t) b->max_w * (uint64_t) N >= (uint64_t) kInfD)
  {
    for (uint32_t r = 0; r < R; r++)
      LA3G_TRY(la3g_sssp(G, roots[r], dist_out ? dist_out + (size_t) r * N : nullptr, nullptr));
    *iters_out = 0;
    return LA3G_OK;
  }
  if (R > b->cap_sr)
  {
    LA3G_TRY(galloc(G, &b->sdist, (size_t) N * R));
    LA3G_TRY(galloc(G, &b->sfront[0], (size_t) N * W));
    LA3G_TRY(galloc(G, &b->sfront[1], (size_t) N * W));
    LA3G_TRY(galloc(G, &b->sact[0], (size_t) N * W));
    LA3G_TRY(galloc(G, &b->sact[1], (size_t) N * W));
    LA3G_TRY(galloc(G, &b->shub[0], (size_t) N * W));
    LA3G_TRY(galloc(G, &b->shub[1], (size_t) N * W));
    LA3G_TRY(galloc(G, &b->shub_t0[0], (size_t) N * W));
    LA3G_TRY(galloc(G, &b->shub_t0[1], (size_t) N * W));
    b->cap_sr = R;
  }
  if (R > b->cap_r) LA3G_TRY(ms_bfs_alloc(G, b, R));
  LA3G_CUDA(cudaMemcpyAsync(b->active, roots, (size_t) R * 4, cudaMemcpyHostToDevice, s));
  k_root_pos<<<grid_for(R, 256), 256, 0, s>>>(b->active, R, N, g.pos_of_id, b->rpos);
  LA3G_LAUNCHED();
  k_bs_init<<<num_sms() * 8, 256, 0, s>>>((uint64_t) N * R, b->sdist, (uint64_t) N * W, b->sfront[0], b->sfront[1]);
  LA3G_LAUNCHED();
  k_bs_roots<<<grid_for(R, 256), 256, 0, s>>>(b->rpos, R, N, W, g.nreg, g.src_base(), g.iso_base(), b->sdist,
                                              b->sfront[0]);
  LA3G_LAUNCHED();
  tls_launches += 3;
  int cur = 0;
  uint32_t iters = 0;
  // the distance window: roots at distance <= limit relax, the rest wait;
  // after each iteration limit = (smallest distance left in the frontier) +
  // delta, which ctr[6] collects (atomicMin over the relax kernel's warps)
  const uint32_t delta = b->sssp_delta ? b->sssp_delta : sssp_auto_delta(b->max_w, b->max_reg_deg);
  uint32_t limit = delta;
  unsigned int* pend = (unsigned int*) (b->ctr + 6);
  // two alternating pair lists; ctr[c] / ctr[2 + c] count list c's small
  // pairs and its packed hub slots / tasks
  PairList L[2];
  for (int c = 0; c < 2; c++) L[c] = PairList{b->sact[c], b->shub[c], b->shub_t0[c], b->ctr + c, b->ctr + 2 + c};
  LA3G_CUDA(cudaMemsetAsync(b->ctr, 0, 4 * 8, s));
  k_bs_list<<<num_sms() * 8, 256, 0, s>>>((uint64_t) N * W, W, g.out_ptr, b->reg_end, b->sfront[0], L[0]);
  LA3G_LAUNCHED();
  tls_launches++;
  for (;;)
  {
    if (iters > 1000000) return set_error(LA3G_ETIMEOUT, "batched sssp did not converge");
    iters++;
    if (delta != kNoWindow) LA3G_CUDA(cudaMemsetAsync(pend, 0xFF, 4, s));
    {
      ProfileScope p("sssp_batch_relax", s, 0.0);
      k_bs_relax<<<num_sms() * 16, 256, 0, s>>>(g.out_ptr, b->reg_end, g.out_row, g.out_w, R, W, b->sfront[cur], L[cur],
                                           b->sfront[cur ^ 1], b->sdist, delta == kNoWindow ? kNoWindow : limit,
                                           delta == kNoWindow ? nullptr : pend);
      LA3G_LAUNCHED();
    }
    LA3G_CUDA(cudaMemsetAsync(b->ctr + (cur ^ 1), 0, 8, s));
    LA3G_CUDA(cudaMemsetAsync(b->ctr + 2 + (cur ^ 1), 0, 8, s));
    k_bs_apply<<<num_sms() * 8, 256, 0, s>>>(N, W, g.out_ptr, b->reg_end, b->sfront[cur ^ 1], L[cur ^ 1], b->sfront[cur],
                                        L[cur]);
    LA3G_LAUNCHED();
    tls_launches += 2;
    unsigned long long act[7] = {0, 0, 0, 0, 0, 0, 0};
    LA3G_CUDA(cudaMemcpyAsync(act, b->ctr, 7 * 8, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    cur ^= 1;
    if (!act[cur] && !act[2 + cur]) break;
    if (delta != kNoWindow)
    {
      uint32_t lo;
      std::memcpy(&lo, &act[6], 4);
      limit = lo > kNoWindow - 1 - delta ? kNoWindow - 1 : lo + delta;
    }
  }
  if (g.nsink)
  {
    k_bs_sinks<<<num_sms() * 8, 256, 0, s>>>(g.in_ptr, g.in_col, g.in_w, g.nreg, g.nsink, R, b->rpos, g.src_base(),
                                        g.iso_base(), b->sdist);
    LA3G_LAUNCHED();
    tls_launches++;
  }
  if (dist_out)
  {
    DevBuf tmp;
    LA3G_TRY(tmp.alloc((size_t) N * R * 4));
    k_bs_out<<<num_sms() * 8, 256, 0, s>>>(N, R, g.id_of_pos, b->sdist, tmp.as<uint32_t>());
    LA3G_LAUNCHED();
    LA3G_CUDA(cudaMemcpyAsync(dist_out, tmp.p, (size_t) N * R * 4, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
  }
  *iters_out = iters;
  return LA3G_OK;
}

// Project autotuner for the batched BFS: times every combination of level
// mode (per-level CUDA graph / persistent kernel), block size and push
// threshold on the caller's roots and keeps the fastest for this graph.
extern "C" int la3g_batch_autotune(la3g_graph* G, const uint32_t* roots, uint32_t nroots, char* report, size_t cap)
{
  if (!G || !roots || nroots == 0) return set_error(LA3G_EINVAL, "graph and roots are required");
  if (G->g.directed()) return set_error(LA3G_EINVAL, "the batched BFS tunes on an undirected graph");
  BatchScratch* b = nullptr;
  LA3G_TRY(batch_scratch(G, &b));
  std::string rep = "[";
  BatchConfig best;
  double best_ms = 1e300;
  const int modes[] = {0, 1};
  const int blocks[] = {128, 256, 512};
  const double fracs[] = {0.0, 0.001, 0.003, 0.01, 0.02, 0.05, 0.1, 0.2, 0.4};
  for (int mode : modes)
    for (int block : blocks)
      for (double frac : fracs)
      {
        if (mode == 1 && frac != 0.0) continue;  // the persistent kernel runs pull levels only
        BatchConfig c;
        c.mode = mode;
        c.block = block;
        c.push_frac = frac;
        uint32_t lv = 0;
        bool wrap = false;
        uint64_t ew = 0;
        LA3G_TRY(ms_bfs_run(G, b, roots, nroots, c, &lv, &wrap, &ew));  // warm
        LA3G_CUDA(cudaStreamSynchronize(G->stream));
        double ms = 1e300;
        for (int rep = 0; rep < 2; rep++)  // best of two
        {
          const double t0 = now_ms();
          LA3G_TRY(ms_bfs_run(G, b, roots, nroots, c, &lv, &wrap, &ew));
          LA3G_CUDA(cudaStreamSynchronize(G->stream));
          ms = std::min(ms, now_ms() - t0);
        }
        char buf[160];
        std::snprintf(buf, sizeof buf, "%s{\"mode\": %d, \"block\": %d, \"push_frac\": %.3f, \"ms\": %.4f}",
                      rep.size() > 1 ? ", " : "", mode, block, frac, ms);
        rep += buf;
        if (ms < best_ms) { best_ms = ms; best = c; }
      }
  best.tuned = true;
  const uint32_t W = (nroots + 63) / 64;
  bool found = false;
  for (auto& t : b->tuned)
    if (t.first == W)
    {
      t.second = best;
      found = true;
    }
  if (!found) b->tuned.emplace_back(W, best);
  rep += "]";
  if (report && cap)
  {
    size_t n = std::min(rep.size(), cap - 1);
    std::memcpy(report, rep.data(), n);
    report[n] = 0;
  }
  return LA3G_OK;
}

extern "C" int la3g_batch_set_wait_limit(la3g_graph* G, long long polls)
{
  if (!G) return set_error(LA3G_EINVAL, "null graph");
  BatchScratch* b = nullptr;
  LA3G_TRY(batch_scratch(G, &b));
  b->wait_polls = polls < 0 ? kDefaultWaitPolls : polls;
  return LA3G_OK;
}

extern "C" int la3g_batch_sssp_window(la3g_graph* G, uint32_t delta)
{
  if (!G) return set_error(LA3G_EINVAL, "null graph");
  BatchScratch* b = nullptr;
  LA3G_TRY(batch_scratch(G, &b));
  b->sssp_delta = delta;
  return LA3G_OK;
}

extern "C" int la3g_batch_config(la3g_graph* G, int mode, int block, double push_frac)
{
  if (!G) return set_error(LA3G_EINVAL, "null graph");
  if ((mode != 0 && mode != 1) || (block != 128 && block != 256 && block != 512) || push_frac < 0 || push_frac > 1)
    return set_error(LA3G_EINVAL, "mode must be 0 or 1, block 128/256/512, push_frac in [0, 1]");
  BatchScratch* b = nullptr;
  LA3G_TRY(batch_scratch(G, &b));
  b->cfg.mode = mode;
  b->cfg.block = block;
  b->cfg.push_frac = push_frac;
  b->cfg.tuned = true;
  b->tuned.clear();  // a hand-set configuration replaces the tuned ones
  return LA3G_OK;
}
