// Serving loop: BFS / SSSP / BM25 / LM queries against several device-resident
// graphs, admitted as they arrive.
//
// The reference answers one query per VertexProgram run (bfs.cpp:11-37,
// sssp.cpp:11-37, bm25.cpp:8-114); here every resident graph gets an engine
// with its own worker thread and CUDA stream, so work on different graphs
// overlaps on the device:
//
//  * BFS and SSSP engines run "lanes": a query occupies one bit of a 64-bit
//    frontier word per vertex (the batched layout), and one engine iteration
//    advances every occupied lane by one BSP step.  Between iterations the
//    worker retires lanes whose frontier emptied (their results are copied
//    out and the lane's state reset) and admits queued queries into free
//    lanes.  Continuous batching: a query never waits for a batch to drain.
//    SSSP queries take any free lane.  BFS queries are admitted a word (64
//    lanes) at a time: the queries queued when a word frees up start
//    together, so each word runs a level-synchronous multi-source BFS whose
//    direction (push or pull) is chosen per word and per level, while the
//    engine's words sit at different levels.
//    Each lane's arithmetic is that of the single-root call, and lanes never
//    read one another's bits, so a result does not depend on the mix.
//    Adaptive batching: an engine with no lanes in flight and only a few
//    queries waiting answers them one at a time through the single-root
//    entry point (faster per query at low load); lanes take over when the
//    queue is deeper.
//  * BM25 engines run their queries (BM25 and LM) one after another on their
//    corpus.
//
// Admission by HBM budget: a graph joins only if its device bytes plus the
// engine's lane state fit in what is left of the budget (the lane count is
// halved down to 64 before LA3G_EBUDGET is returned); queries then wait for a
// free lane of their graph's engine.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "la3g_internal.h"
#include "lanes.cuh"

namespace la3g {
namespace {

constexpr uint32_t kOutChunk = 64;   // BFS lanes retired per output pass (staging rows)

double wall_ms()
{
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Ticket
{
  la3g_query q{};
  std::vector<uint32_t> terms;
  int status = -1;  // -1 pending
  double submit_ms = 0, start_ms = 0, done_ms = 0;
  uint32_t in_flight = 0;
  uint32_t nout = 0;
};

// ------------------------------------------------------------------ BFS lanes

// BFS engine words: the 64 lanes of a word are admitted together and share
// the word's level, so every word runs a level-synchronous multi-source BFS
// (direction chosen per word) while different words sit at different
// levels.  Words are bit w of the `words` masks below (W <= 64).
struct WordHops
{
  uint8_t h[64];  // hop value written at this level, per word
};

__global__ void k_lb_admit(const uint32_t* __restrict__ adm, uint32_t n, uint32_t N, uint32_t W,
                           const uint32_t* __restrict__ ptr, uint64_t* vis, uint64_t* front, uint8_t* hops,
                           uint64_t* alive, unsigned long long* fdeg)
{
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
  {
    const uint32_t l = adm[2 * j], p = adm[2 * j + 1];
    const uint32_t w = l / 64;
    const unsigned long long bit = 1ull << (l % 64);
    atomicOr((unsigned long long*) &vis[(uint64_t) p * W + w], bit);
    atomicOr((unsigned long long*) &front[(uint64_t) p * W + w], bit);
    atomicOr((unsigned long long*) &alive[w], bit);
    hops[((uint64_t) p * W + w) * 64 + l % 64] = 0;
    atomicAdd(&fdeg[w], (unsigned long long) (ptr[p + 1] - ptr[p]));
  }
}

// Per-word frontier degree sums, gathered per block in shared memory.
__device__ __forceinline__ void lb_deg_flush(unsigned long long* sdeg, uint32_t W, unsigned long long* fdeg)
{
  __syncthreads();
  for (uint32_t w = threadIdx.x; w < W; w += blockDim.x)
    if (sdeg[w]) atomicAdd(&fdeg[w], sdeg[w]);
}

// Bottom-up step over (vertex, word) pairs of the pull words.
__global__ void __launch_bounds__(256)
k_lb_pull(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, uint32_t nrows, uint32_t N, uint32_t W,
          uint64_t* vis, const uint64_t* __restrict__ front, uint64_t* next, const uint64_t* __restrict__ alive_cur,
          uint64_t* alive_next, uint8_t* hops, WordHops hop, uint64_t words, unsigned long long* fdeg)
{
  __shared__ unsigned long long sdeg[64];
  for (uint32_t w = threadIdx.x; w < W; w += blockDim.x) sdeg[w] = 0;
  __syncthreads();
  const uint64_t NW = (uint64_t) nrows * W;
  const int lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t) gridDim.x * blockDim.x) >> 5;
  for (uint64_t base = warp * 32; base < NW; base += nwarps * 32)
  {
    const uint64_t i = base + lane;
    const uint32_t w = i < NW ? (uint32_t) (i % W) : 0;
    const bool ok = i < NW && ((words >> w) & 1ull);
    const uint32_t v = ok ? (uint32_t) (i / W) : 0;
    const uint64_t seen = ok ? vis[i] : ~0ull;
    const uint64_t want = ok ? ~seen & alive_cur[w] : 0;
    const uint64_t nb = pull_scan(v, w, W, want, ptr, col, front, lane);
    if (!ok) continue;
    next[i] = nb;
    if (nb)
    {
      vis[i] = seen | nb;
      atomicAdd(&sdeg[w], (unsigned long long) (ptr[v + 1] - ptr[v]));
      atomicOr((unsigned long long*) &alive_next[w], (unsigned long long) nb);
      hops_record(hops + i * 64, nb, hop.h[w]);
    }
  }
  lb_deg_flush(sdeg, W, fdeg);
}

// Clears the frontier words of the given words (after a pull consumed them).
__global__ void k_lb_clear(uint64_t NW, uint32_t W, uint64_t* buf, uint64_t words)
{
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < NW; i += (uint64_t) gridDim.x * blockDim.x)
    if ((words >> (i % W)) & 1ull) buf[i] = 0;
}

__global__ void k_lb_list(uint64_t NW, uint32_t W, const uint32_t* __restrict__ ptr, const uint64_t* __restrict__ front,
                          uint64_t words, PairList out)
{
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < NW; i += (uint64_t) gridDim.x * blockDim.x)
    if (((words >> (i % W)) & 1ull) && front[i])
    {
      const uint32_t v = (uint32_t) (i / W);
      bs_list_pair((uint32_t) i, ptr[v + 1] - ptr[v], out);
    }
}

// Top-down step over the listed frontier words (ms_push_pairs: small pairs a
// warp each, hub edges as tasks), ORing them into the neighbours' next words
// (masked by visited).
__global__ void k_lb_push(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, uint32_t W,
                          const uint64_t* __restrict__ front, const uint64_t* __restrict__ vis, uint64_t* next, PairList list)
{
  ms_push_pairs(ptr, col, W, front, vis, next, list);
}

// After a push: new bits = next & ~visited; the old frontier words of the
// push words are cleared so that the buffer can serve as the next "next".
__global__ void __launch_bounds__(256)
k_lb_apply(const uint32_t* __restrict__ ptr, uint32_t nrows, uint32_t N, uint32_t W, uint64_t* vis, uint64_t* front,
           uint64_t* next, uint64_t* alive_next, uint8_t* hops, WordHops hop, uint64_t words, unsigned long long* fdeg)
{
  __shared__ unsigned long long sdeg[64];
  for (uint32_t w = threadIdx.x; w < W; w += blockDim.x) sdeg[w] = 0;
  __syncthreads();
  const uint64_t NW = (uint64_t) nrows * W;
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < NW; i += (uint64_t) gridDim.x * blockDim.x)
  {
    const uint32_t w = (uint32_t) (i % W);
    if (!((words >> w) & 1ull)) continue;
    front[i] = 0;
    const uint64_t x = next[i];
    if (!x) continue;
    const uint64_t nb = x & ~vis[i];
    next[i] = nb;
    if (nb)
    {
      const uint32_t v = (uint32_t) (i / W);
      vis[i] |= nb;
      atomicAdd(&sdeg[w], (unsigned long long) (ptr[v + 1] - ptr[v]));
      atomicOr((unsigned long long*) &alive_next[w], (unsigned long long) nb);
      hops_record(hops + i * 64, nb, hop.h[w]);
    }
  }
  lb_deg_flush(sdeg, W, fdeg);
}

// Retiring lanes, in two passes so that no pass gathers across the whole
// [N][L] hop array: first by position (hop rows read in order) into tmp[j][p],
// resetting the bytes to 255; then by id, staging[j][id] = tmp[j][pos(id)],
// a gather inside one lane's N-byte row, which stays in L2.  The retiring
// lanes of a pass are given per word (wmask[w]; wbase[w] = index j of the
// word's first one); a thread loads the 8-byte groups of a (position, word)
// block that hold them at once and writes the 255s back with masked words.
__global__ void k_lb_out_pos(const uint64_t* __restrict__ wmask, const uint32_t* __restrict__ wbase, uint32_t N, uint32_t W,
                             uint8_t* hops, uint8_t* tmp)
{
  for (uint64_t p = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (uint64_t) gridDim.x * blockDim.x)
    for (uint32_t w = 0; w < W; w++)
    {
      const uint64_t mw = wmask[w];
      if (!mw) continue;
      uint64_t* blk = reinterpret_cast<uint64_t*>(hops + (p * W + w) * 64);
      uint64_t q[8];
#pragma unroll
      for (int g = 0; g < 8; g++) q[g] = ((mw >> (8 * g)) & 0xFFu) ? blk[g] : 0;
      uint32_t j = wbase[w];
#pragma unroll
      for (int g = 0; g < 8; g++)
      {
        const uint32_t m8 = (uint32_t) (mw >> (8 * g)) & 0xFFu;
        if (!m8) continue;
        for (uint32_t m = m8; m; m &= m - 1)
          tmp[(uint64_t) j++ * N + p] = (uint8_t) (q[g] >> (8 * (__ffs(m) - 1)));
        blk[g] = q[g] | spread_bits_to_bytes(m8);
      }
    }
}

__global__ void k_lb_out_id(uint32_t nl, uint32_t N, const uint32_t* __restrict__ pos_of_id, const uint8_t* __restrict__ tmp,
                            uint8_t* staging)
{
  for (uint64_t id = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; id < N; id += (uint64_t) gridDim.x * blockDim.x)
  {
    const uint32_t p = pos_of_id[id];
    for (uint32_t j = 0; j < nl; j++) staging[(uint64_t) j * N + id] = tmp[(uint64_t) j * N + p];
  }
}

// Clears the retired lanes' bits (mask: W words) from the bitmaps.
__global__ void k_lb_unset(uint64_t NW, uint32_t W, const uint64_t* __restrict__ mask, uint64_t* a, uint64_t* b)
{
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < NW; i += (uint64_t) gridDim.x * blockDim.x)
  {
    const uint64_t m = mask[i % W];
    if (a[i] & m) a[i] &= ~m;
    if (b && (b[i] & m)) b[i] &= ~m;
  }
}

__global__ void k_lb_fill_u8(uint64_t n, uint8_t* p, uint8_t v)
{
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
    p[i] = v;
}

// ------------------------------------------------------------------ SSSP lanes

__global__ void k_ls_fill_u32(uint64_t n, uint32_t* p, uint32_t v)
{
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
    p[i] = v;
}

__global__ void k_ls_admit(const uint32_t* __restrict__ adm, uint32_t n, uint32_t L, uint32_t W,
                           const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ reg_end, uint32_t nreg,
                           uint32_t src_base, uint32_t iso_base, uint32_t* dist, uint64_t* front,
                           uint32_t* rpos, PairList list)
{
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
  {
    const uint32_t l = adm[2 * j], p = adm[2 * j + 1];
    dist[(uint64_t) p * L + l] = 0;
    rpos[l] = p;
    if (p < nreg || (p >= src_base && p < iso_base))
    {
      const uint64_t i = (uint64_t) p * W + l / 64;
      const unsigned long long old = atomicOr((unsigned long long*) &front[i], 1ull << (l % 64));
      if (!old) bs_list_pair((uint32_t) i, reg_end[p] - ptr[p], list);
    }
  }
}

// Sink rows of the retiring lanes, once, from their final regular
// distances (vertex_program_execute.hpp:131-148), then distances by id into
// the staging rows and the lanes' columns reset to INF.
__global__ void k_ls_sinks(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col,
                           const uint32_t* __restrict__ wgt, uint32_t nreg, uint32_t nsink, uint32_t L,
                           const uint32_t* __restrict__ lanes, uint32_t nl, const uint32_t* __restrict__ rpos,
                           uint32_t src_base, uint32_t iso_base, uint32_t* dist)
{
  const uint64_t n = (uint64_t) nsink * nl;
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
  {
    const uint32_t v = nreg + (uint32_t) (i / nl), l = lanes[i % nl];
    const uint32_t rp = rpos[l];
    uint32_t y = kInfD;
    for (uint32_t e = ptr[v]; e < ptr[v + 1]; e++)
    {
      const uint32_t c = col[e];
      uint32_t cand;
      if (c < nreg) cand = dist[(uint64_t) c * L + l] + wgt[e];
      else if (c == rp && rp >= src_base && rp < iso_base) cand = wgt[e];
      else continue;
      y = min(y, cand);
    }
    uint32_t* d = &dist[(uint64_t) v * L + l];
    *d = min(*d, y);
  }
}

// Retiring SSSP lanes in two passes: by position, a thread per vertex loads
// the retiring lanes' distances of its row (all in flight together), writes
// them to tmp[j][p] (coalesced per lane) and resets them to INF; then by id,
// staging[j][id] = tmp[j][pos(id)], a gather inside one lane's N-entry row,
// which stays in L2 (a scatter by id straight from the rows would spread
// partial-sector writes over all nl rows at once).
static constexpr uint32_t kOutChunkS = 16;  // SSSP lanes retired per output pass (staging rows)

__global__ void k_ls_out_pos(const uint32_t* __restrict__ lanes, uint32_t nl, uint32_t N, uint32_t L, uint32_t* dist,
                             uint32_t* __restrict__ tmp)
{
  uint32_t ln[kOutChunkS];
#pragma unroll
  for (uint32_t j = 0; j < kOutChunkS; j++) ln[j] = j < nl ? lanes[j] : 0;
  for (uint64_t p = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (uint64_t) gridDim.x * blockDim.x)
  {
    uint32_t* row = dist + p * L;
    uint32_t x[kOutChunkS];
#pragma unroll
    for (uint32_t j = 0; j < kOutChunkS; j++) x[j] = j < nl ? __ldcg(&row[ln[j]]) : 0;
#pragma unroll
    for (uint32_t j = 0; j < kOutChunkS; j++)
      if (j < nl)
      {
        tmp[(uint64_t) j * N + p] = x[j];
        row[ln[j]] = kInfD;
      }
  }
}

__global__ void k_ls_out_id(uint32_t nl, uint32_t N, const uint32_t* __restrict__ pos_of_id, const uint32_t* __restrict__ tmp,
                            uint32_t* __restrict__ staging)
{
  const uint64_t n = (uint64_t) nl * N;
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
  {
    const uint64_t j = i / N;
    staging[i] = tmp[j * N + pos_of_id[i - j * N]];
  }
}

}  // namespace
}  // namespace la3g

using namespace la3g;

// ------------------------------------------------------------------ engines

struct la3g_server;

namespace {

enum EngineKind
{
  kEngBfs = 1,
  kEngSssp = 2,
  kEngBm25 = 3
};

struct Engine
{
  la3g_server* S = nullptr;
  la3g_graph* G = nullptr;
  int kind = 0;
  uint32_t id = 0;
  std::deque<Ticket*> queue;  // guarded by the server mutex
  std::condition_variable cv;
  std::thread th;
  bool stop = false;
  uint64_t bytes = 0;         // engine state bytes (the graph's own are counted apart)
  int error = LA3G_OK;        // sticky CUDA error of the worker
  std::string error_msg;
  // lanes
  uint32_t L = 0, W = 0, N = 0;
  std::vector<Ticket*> lane;
  std::vector<uint32_t> wlevel;     // BFS: levels each word has run since its admission
  std::vector<uint32_t> wbusy;      // BFS: occupied lanes per word
  std::vector<uint32_t> pos_of_id;  // host copy
  bool exact_lanes = true;          // SSSP: max weight * N < INF
  DevBuf vis, buf[2], hops, alive[2], active, ctr, adm, ret, mask, staging, outpos, fdeg;
  // SSSP
  DevBuf dist, sfront[2], small[2], hub[2], hub_t0[2], reg_end, rpos;
  unsigned long long* hctr = nullptr;  // pinned: counters + alive words
  // BM25 / LM: a stream of the device's greatest priority, so that a query's
  // few small kernels get SMs ahead of the waiting blocks of the BFS / SSSP
  // lane kernels on the other engines' streams
  cudaStream_t prio = nullptr;
};

}  // namespace

struct la3g_server
{
  uint64_t budget = 0, used = 0;
  uint32_t bfs_lanes = 256, sssp_lanes = 256;
  uint32_t solo_bfs = 16, solo_sssp = 4;  // adaptive batching depths
  std::mutex mu;
  std::condition_variable done_cv;
  std::unordered_map<uint64_t, Ticket*> tickets;
  uint64_t next_ticket = 1;
  std::vector<Engine*> engines;
  std::atomic<uint64_t> completed{0};
};

namespace {

uint32_t solo_depth(const Engine* E)
{
  return E->kind == kEngBfs ? E->S->solo_bfs : E->S->solo_sssp;
}

uint64_t bfs_lane_bytes(uint32_t N, uint32_t L)
{
  const uint64_t W = L / 64;
  return (uint64_t) N * W * 8 * 3 + (uint64_t) N * L + (uint64_t) N * W * 4 * 3 + (uint64_t) kOutChunk * N * 2 + 4096 +
         L * 16;
}

uint64_t sssp_lane_bytes(uint32_t N, uint32_t L)
{
  const uint64_t W = L / 64;
  return (uint64_t) N * L * 4 + (uint64_t) N * W * 8 * 2 + (uint64_t) N * W * 4 * 6 + (uint64_t) N * 4 +
         (uint64_t) kOutChunkS * N * 4 * 2 + 4096 + L * 16;
}

void finish_ticket(la3g_server* S, Ticket* t, int status)
{
  std::lock_guard<std::mutex> lk(S->mu);
  t->status = status;
  t->done_ms = wall_ms();
  S->completed++;
  S->done_cv.notify_all();
}

void engine_fail(Engine* E, int st)
{
  // a CUDA error leaves the engine unusable: fail everything it holds
  E->error = st;
  E->error_msg = la3g_last_error_string();
  std::vector<Ticket*> all;
  {
    std::lock_guard<std::mutex> lk(E->S->mu);
    for (Ticket* t : E->queue) all.push_back(t);
    E->queue.clear();
  }
  for (Ticket*& t : E->lane)
    if (t)
    {
      all.push_back(t);
      t = nullptr;
    }
  for (Ticket* t : all) finish_ticket(E->S, t, st);
}

// Pops up to `free_lanes` queued tickets (waits while there is no work).
// Returns false when the engine stops.
// Adaptive batching: an engine with no lanes in flight and at most
// solo_depth queries waiting answers them one at a time through the
// single-root path, which is faster per query at low load; lanes take over
// above it (la3g_server_set_solo sets the depths; 0 = lanes only).
uint32_t solo_depth(const Engine* E);

// Waits for work.  With no lanes in flight and a short queue, pops one
// ticket into *solo; otherwise pops up to `free_lanes` into got.  Returns
// false when the engine stops.
bool take_work(Engine* E, uint32_t busy, uint32_t free_lanes, std::vector<Ticket*>& got, Ticket** solo = nullptr)
{
  std::unique_lock<std::mutex> lk(E->S->mu);
  while (!E->stop && busy == 0 && E->queue.empty()) E->cv.wait(lk);
  if (E->stop) return false;
  if (solo && busy == 0 && E->queue.size() <= solo_depth(E))
  {
    *solo = E->queue.front();
    E->queue.pop_front();
    return true;
  }
  while (free_lanes && !E->queue.empty())
  {
    got.push_back(E->queue.front());
    E->queue.pop_front();
    free_lanes--;
  }
  return true;
}

int run_single(Engine* E, Ticket* t);
void finish_out_of_range(Engine* E, Ticket* t);

// A query answered alone (adaptive batching): the single-root entry point.
void run_solo(Engine* E, Ticket* t)
{
  t->start_ms = wall_ms();
  t->in_flight = 1;
  if (t->q.root >= E->N) finish_out_of_range(E, t);
  else finish_ticket(E->S, t, run_single(E, t));
}

int bfs_engine_init(Engine* E)
{
  DevGraph& g = E->G->g;
  cudaStream_t s = E->G->stream;
  const uint32_t N = E->N, W = E->W, L = E->L;
  const uint64_t NW = (uint64_t) N * W;
  LA3G_TRY(E->vis.alloc(NW * 8));
  LA3G_TRY(E->buf[0].alloc(NW * 8));
  LA3G_TRY(E->buf[1].alloc(NW * 8));
  LA3G_TRY(E->hops.alloc((uint64_t) L * N));
  LA3G_TRY(E->alive[0].alloc(W * 8));
  LA3G_TRY(E->alive[1].alloc(W * 8));
  LA3G_TRY(E->active.alloc(NW * 4));
  LA3G_TRY(E->hub[0].alloc(NW * 4));
  LA3G_TRY(E->hub_t0[0].alloc(NW * 4));
  LA3G_TRY(E->ctr.alloc(8 * 8));
  LA3G_TRY(E->adm.alloc((uint64_t) L * 8));
  LA3G_TRY(E->ret.alloc((uint64_t) L * 4));
  LA3G_TRY(E->mask.alloc(W * 8));
  LA3G_TRY(E->fdeg.alloc(W * 8));
  LA3G_TRY(E->staging.alloc((uint64_t) kOutChunk * N));
  LA3G_TRY(E->outpos.alloc((uint64_t) kOutChunk * N));
  LA3G_CUDA(cudaMemsetAsync(E->fdeg.p, 0, W * 8, s));
  LA3G_CUDA(cudaMemsetAsync(E->vis.p, 0, NW * 8, s));
  LA3G_CUDA(cudaMemsetAsync(E->buf[0].p, 0, NW * 8, s));
  LA3G_CUDA(cudaMemsetAsync(E->buf[1].p, 0, NW * 8, s));
  LA3G_CUDA(cudaMemsetAsync(E->alive[0].p, 0, W * 8, s));
  LA3G_CUDA(cudaMemsetAsync(E->alive[1].p, 0, W * 8, s));
  k_lb_fill_u8<<<num_sms() * 8, 256, 0, s>>>((uint64_t) L * N, E->hops.as<uint8_t>(), 255);
  LA3G_LAUNCHED();
  (void) g;
  return LA3G_OK;
}

int sssp_engine_init(Engine* E)
{
  DevGraph& g = E->G->g;
  cudaStream_t s = E->G->stream;
  const uint32_t N = E->N, W = E->W, L = E->L;
  const uint64_t NW = (uint64_t) N * W;
  LA3G_TRY(E->dist.alloc((uint64_t) N * L * 4));
  for (int c = 0; c < 2; c++)
  {
    LA3G_TRY(E->sfront[c].alloc(NW * 8));
    LA3G_TRY(E->small[c].alloc(NW * 4));
    LA3G_TRY(E->hub[c].alloc(NW * 4));
    LA3G_TRY(E->hub_t0[c].alloc(NW * 4));
    LA3G_CUDA(cudaMemsetAsync(E->sfront[c].p, 0, NW * 8, s));
  }
  LA3G_TRY(E->reg_end.alloc((uint64_t) N * 4));
  LA3G_TRY(E->rpos.alloc((uint64_t) L * 4));
  LA3G_TRY(E->alive[0].alloc(W * 8));
  LA3G_TRY(E->ctr.alloc(8 * 8));
  LA3G_TRY(E->adm.alloc((uint64_t) L * 8));
  LA3G_TRY(E->ret.alloc((uint64_t) L * 4));
  LA3G_TRY(E->staging.alloc((uint64_t) kOutChunkS * N * 4));
  LA3G_TRY(E->outpos.alloc((uint64_t) kOutChunkS * N * 4));
  LA3G_CUDA(cudaMemsetAsync(E->ctr.p, 0, 64, s));
  k_ls_fill_u32<<<num_sms() * 8, 256, 0, s>>>((uint64_t) N * L, E->dist.as<uint32_t>(), kInfD);
  LA3G_LAUNCHED();
  k_reg_end<<<grid_for(N, 256), 256, 0, s>>>(g.out_ptr, g.out_row, N, g.nreg, E->reg_end.as<uint32_t>());
  LA3G_LAUNCHED();
  // lanes are exact regardless of relaxation order only if no distance can
  // reach INF; otherwise every query runs the single-root path
  DevBuf m;
  LA3G_TRY(m.alloc(4));
  LA3G_CUDA(cudaMemsetAsync(m.p, 0, 4, s));
  if (g.nent)
  {
    k_max_u32<<<grid_for(g.nent, 256), 256, 0, s>>>(g.out_w, g.nent, m.as<unsigned int>());
    LA3G_LAUNCHED();
  }
  unsigned int maxw = 0;
  LA3G_CUDA(cudaMemcpyAsync(&maxw, m.p, 4, cudaMemcpyDeviceToHost, s));
  LA3G_CUDA(cudaStreamSynchronize(s));
  E->exact_lanes = (uint64_t) maxw * (uint64_t) N < (uint64_t) kInfD;
  return LA3G_OK;
}

// Copies each retiring lane's result into its ticket's output (when
// `deliver`) and frees the lane: its bits leave the visited bitmap and, for
// lanes leaving early, the current frontier and alive mask as well.
int bfs_retire(Engine* E, const std::vector<uint32_t>& lanes_in, bool deliver, uint64_t* front, uint64_t* alive)
{
  DevGraph& g = E->G->g;
  cudaStream_t s = E->G->stream;
  const uint32_t N = E->N, W = E->W;
  std::vector<uint32_t> lanes(lanes_in);
  std::sort(lanes.begin(), lanes.end());  // staging row j = j-th retiring lane in lane order
  for (size_t j0 = 0; j0 < lanes.size(); j0 += kOutChunk)
  {
    const uint32_t nl = (uint32_t) std::min<size_t>(kOutChunk, lanes.size() - j0);
    // per-word masks of this pass's lanes (ascending, so lane order = j order)
    std::vector<uint64_t> wm(W, 0);
    std::vector<uint32_t> wb(W, 0);
    for (uint32_t j = nl; j-- > 0;)
    {
      const uint32_t l = lanes[j0 + j];
      wm[l / 64] |= 1ull << (l % 64);
      wb[l / 64] = j;
    }
    LA3G_CUDA(cudaMemcpyAsync(E->ret.p, wm.data(), W * 8, cudaMemcpyHostToDevice, s));
    LA3G_CUDA(cudaMemcpyAsync(E->ret.as<uint8_t>() + W * 8, wb.data(), W * 4, cudaMemcpyHostToDevice, s));
    ProfileScope prof("serve_bfs_out", s, 0.0);
    k_lb_out_pos<<<num_sms() * 8, 256, 0, s>>>(E->ret.as<uint64_t>(), (const uint32_t*) (E->ret.as<uint8_t>() + W * 8), N, W,
                                          E->hops.as<uint8_t>(), E->outpos.as<uint8_t>());
    LA3G_LAUNCHED();
    k_lb_out_id<<<num_sms() * 8, 256, 0, s>>>(nl, N, g.pos_of_id, E->outpos.as<uint8_t>(), E->staging.as<uint8_t>());
    LA3G_LAUNCHED();
    tls_launches += 2;
    for (uint32_t j = 0; deliver && j < nl; j++)
    {
      Ticket* t = E->lane[lanes[j0 + j]];
      if (t->q.out)
        LA3G_CUDA(cudaMemcpyAsync(t->q.out, E->staging.as<uint8_t>() + (size_t) j * N, N, cudaMemcpyDeviceToHost, s));
    }
    LA3G_CUDA(cudaStreamSynchronize(s));
  }
  std::vector<uint64_t> m(W, 0);
  for (uint32_t l : lanes) m[l / 64] |= 1ull << (l % 64);
  LA3G_CUDA(cudaMemcpyAsync(E->mask.p, m.data(), W * 8, cudaMemcpyHostToDevice, s));
  k_lb_unset<<<num_sms() * 8, 256, 0, s>>>((uint64_t) N * W, W, E->mask.as<uint64_t>(), E->vis.as<uint64_t>(), front);
  LA3G_LAUNCHED();
  tls_launches++;
  if (alive)
  {
    k_lb_unset<<<1, 64, 0, s>>>(W, W, E->mask.as<uint64_t>(), alive, nullptr);
    LA3G_LAUNCHED();
  }
  LA3G_CUDA(cudaStreamSynchronize(s));
  return LA3G_OK;
}

// Runs one query alone through the single-root entry point (used for BFS
// lanes that would pass 254 levels and for SSSP graphs whose weights could
// reach INF).
int run_single(Engine* E, Ticket* t)
{
  if (E->kind == kEngBfs) return la3g_bfs(E->G, t->q.root, (uint8_t*) t->q.out, nullptr, nullptr);
  return la3g_sssp(E->G, t->q.root, (uint32_t*) t->q.out, nullptr);
}

// Completes a ticket whose root has no vertex: nothing is reached
// (la3g_bfs / la3g_sssp give the same).
void finish_out_of_range(Engine* E, Ticket* t)
{
  if (t->q.out)
  {
    if (E->kind == kEngBfs) std::memset(t->q.out, 255, E->N);
    else
      for (uint32_t i = 0; i < E->N; i++) ((uint32_t*) t->q.out)[i] = kInfD;
  }
  finish_ticket(E->S, t, LA3G_OK);
}

// SSSP admission: queued tickets take any free lane; tickets that need no
// lane (root out of range) or must run alone are completed here.  Returns
// the (lane, position) pairs to initialise on the device.
int admit(Engine* E, std::vector<Ticket*>& got, uint32_t& busy, std::vector<uint32_t>& adm)
{
  adm.clear();
  const double now = wall_ms();
  for (Ticket* t : got)
  {
    t->start_ms = now;
    const uint32_t root = t->q.root;
    if (root >= E->N)
    {
      finish_out_of_range(E, t);
      continue;
    }
    if (E->kind == kEngSssp && !E->exact_lanes)
    {
      finish_ticket(E->S, t, run_single(E, t));
      continue;
    }
    uint32_t l = 0;
    while (E->lane[l]) l++;
    E->lane[l] = t;
    busy++;
    t->in_flight = busy;
    adm.push_back(l);
    adm.push_back(E->pos_of_id[root]);
  }
  return LA3G_OK;
}

int bfs_loop(Engine* E)
{
  DevGraph& g = E->G->g;
  cudaStream_t s = E->G->stream;
  const uint32_t N = E->N, W = E->W, nrows = g.nrows();
  const uint64_t NW = (uint64_t) nrows * W;
  unsigned long long* ctr = E->ctr.as<unsigned long long>();
  unsigned long long* fdeg = E->fdeg.as<unsigned long long>();
  uint32_t busy = 0;
  uint64_t words_busy = 0;  // words with lanes in flight
  int cur = 0;
  std::vector<Ticket*> got;
  std::vector<uint32_t> adm, fin;
  std::vector<unsigned long long> hdeg(W);
  LA3G_CUDA(cudaMemsetAsync(ctr, 0, 64, s));
  for (;;)
  {
    // a free word takes up to 64 queued queries at once
    const uint32_t free_words = W - (uint32_t) __builtin_popcountll(words_busy);
    got.clear();
    Ticket* solo = nullptr;
    if (!take_work(E, busy, free_words * 64, got, &solo)) return LA3G_OK;
    if (solo)
    {
      run_solo(E, solo);
      continue;
    }
    adm.clear();
    const double now = wall_ms();
    size_t k = 0;
    for (uint32_t w = 0; w < W && k < got.size(); w++)
    {
      if ((words_busy >> w) & 1ull) continue;
      uint32_t j = 0;
      for (; k < got.size() && j < 64; k++)
      {
        Ticket* t = got[k];
        t->start_ms = now;
        if (t->q.root >= N)
        {
          finish_out_of_range(E, t);
          continue;
        }
        const uint32_t l = w * 64 + j++;
        E->lane[l] = t;
        busy++;
        t->in_flight = busy;
        adm.push_back(l);
        adm.push_back(E->pos_of_id[t->q.root]);
      }
      if (j)
      {
        words_busy |= 1ull << w;
        E->wbusy[w] = j;
        E->wlevel[w] = 0;
      }
    }
    for (; k < got.size(); k++) finish_out_of_range(E, got[k]);  // only out-of-range ones can be left
    if (!adm.empty())
    {
      const uint32_t n = (uint32_t) adm.size() / 2;
      LA3G_CUDA(cudaMemcpyAsync(E->adm.p, adm.data(), adm.size() * 4, cudaMemcpyHostToDevice, s));
      k_lb_admit<<<grid_for(n, 128), 128, 0, s>>>(E->adm.as<uint32_t>(), n, N, W, g.in_ptr, E->vis.as<uint64_t>(),
                                                 E->buf[cur].as<uint64_t>(), E->hops.as<uint8_t>(),
                                                 E->alive[cur].as<uint64_t>(), fdeg);
      LA3G_LAUNCHED();
      tls_launches++;
    }
    if (busy == 0) continue;
    uint64_t* front = E->buf[cur].as<uint64_t>();
    uint64_t* next = E->buf[cur ^ 1].as<uint64_t>();
    // words whose next hop would be 255 hand their lanes to the single-root
    // path, which follows the reference's uint8 wrap exactly
    fin.clear();
    for (uint32_t w = 0; w < W; w++)
      if (((words_busy >> w) & 1ull) && E->wlevel[w] + 1 >= 255)
        for (uint32_t l = w * 64; l < w * 64 + 64; l++)
          if (E->lane[l]) fin.push_back(l);
    if (!fin.empty())
    {
      LA3G_TRY(bfs_retire(E, fin, false, front, E->alive[cur].as<uint64_t>()));
      for (uint32_t l : fin)
      {
        Ticket* t = E->lane[l];
        E->lane[l] = nullptr;
        busy--;
        if (--E->wbusy[l / 64] == 0) words_busy &= ~(1ull << (l / 64));
        finish_ticket(E->S, t, run_single(E, t));
      }
      if (busy == 0) continue;
    }
    // one level for every busy word: push while its frontier's edges are
    // few, pull otherwise (per word, Beamer-style)
    LA3G_CUDA(cudaMemcpyAsync(hdeg.data(), fdeg, W * 8, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    LA3G_CUDA(cudaMemsetAsync(fdeg, 0, W * 8, s));
    LA3G_CUDA(cudaMemsetAsync(ctr + 2, 0, 8, s));
    LA3G_CUDA(cudaMemsetAsync(E->alive[cur ^ 1].p, 0, W * 8, s));
    uint64_t pull_words = 0, push_words = 0;
    WordHops hop{};
    for (uint32_t w = 0; w < W; w++)
    {
      if (!((words_busy >> w) & 1ull)) continue;
      hop.h[w] = (uint8_t) (E->wlevel[w] + 1);
      if ((double) hdeg[w] * 20.0 >= (double) g.nent) pull_words |= 1ull << w;
      else push_words |= 1ull << w;
    }
    if (pull_words)
    {
      ProfileScope prof("serve_bfs_pull", s, 0.0);
      k_lb_pull<<<num_sms() * 8, 256, 0, s>>>(g.in_ptr, g.in_col, nrows, N, W, E->vis.as<uint64_t>(), front, next,
                                         E->alive[cur].as<uint64_t>(), E->alive[cur ^ 1].as<uint64_t>(),
                                         E->hops.as<uint8_t>(), hop, pull_words, fdeg);
      LA3G_LAUNCHED();
      k_lb_clear<<<num_sms() * 8, 256, 0, s>>>(NW, W, front, pull_words);
      LA3G_LAUNCHED();
      tls_launches += 2;
    }
    if (push_words)
    {
      ProfileScope prof("serve_bfs_push", s, 0.0);
      const PairList pl{E->active.as<uint32_t>(), E->hub[0].as<uint32_t>(), E->hub_t0[0].as<uint32_t>(), ctr + 2, ctr + 4};
      LA3G_CUDA(cudaMemsetAsync(ctr + 4, 0, 8, s));
      k_lb_list<<<num_sms() * 8, 256, 0, s>>>(NW, W, g.in_ptr, front, push_words, pl);
      LA3G_LAUNCHED();
      k_lb_push<<<num_sms() * 8, 256, 0, s>>>(g.in_ptr, g.in_col, W, front, E->vis.as<uint64_t>(), next, pl);
      LA3G_LAUNCHED();
      k_lb_apply<<<num_sms() * 8, 256, 0, s>>>(g.in_ptr, nrows, N, W, E->vis.as<uint64_t>(), front, next,
                                          E->alive[cur ^ 1].as<uint64_t>(), E->hops.as<uint8_t>(), hop, push_words,
                                          fdeg);
      LA3G_LAUNCHED();
      tls_launches += 3;
    }
    LA3G_CUDA(cudaMemcpyAsync(E->hctr, E->alive[cur ^ 1].p, W * 8, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    cur ^= 1;
    for (uint32_t w = 0; w < W; w++)
      if ((words_busy >> w) & 1ull) E->wlevel[w]++;
    // a lane that found no new vertex is finished; a word is free again
    // when all its lanes are
    fin.clear();
    for (uint32_t l = 0; l < E->L; l++)
      if (E->lane[l] && !((E->hctr[l / 64] >> (l % 64)) & 1ull)) fin.push_back(l);
    if (!fin.empty())
    {
      LA3G_TRY(bfs_retire(E, fin, true, nullptr, nullptr));
      for (uint32_t l : fin)
      {
        Ticket* t = E->lane[l];
        E->lane[l] = nullptr;
        busy--;
        if (--E->wbusy[l / 64] == 0) words_busy &= ~(1ull << (l / 64));
        finish_ticket(E->S, t, LA3G_OK);
      }
    }
  }
}

int sssp_retire(Engine* E, const std::vector<uint32_t>& lanes)
{
  DevGraph& g = E->G->g;
  cudaStream_t s = E->G->stream;
  const uint32_t N = E->N, L = E->L;
  for (size_t j0 = 0; j0 < lanes.size(); j0 += kOutChunkS)
  {
    const uint32_t nl = (uint32_t) std::min<size_t>(kOutChunkS, lanes.size() - j0);
    LA3G_CUDA(cudaMemcpyAsync(E->ret.p, lanes.data() + j0, nl * 4, cudaMemcpyHostToDevice, s));
    ProfileScope prof("serve_sssp_out", s, 0.0);
    if (g.nsink)
    {
      k_ls_sinks<<<num_sms() * 8, 256, 0, s>>>(g.in_ptr, g.in_col, g.in_w, g.nreg, g.nsink, L, E->ret.as<uint32_t>(), nl,
                                          E->rpos.as<uint32_t>(), g.src_base(), g.iso_base(), E->dist.as<uint32_t>());
      LA3G_LAUNCHED();
      tls_launches++;
    }
    k_ls_out_pos<<<num_sms() * 8, 256, 0, s>>>(E->ret.as<uint32_t>(), nl, N, L, E->dist.as<uint32_t>(),
                                          E->outpos.as<uint32_t>());
    LA3G_LAUNCHED();
    k_ls_out_id<<<num_sms() * 8, 256, 0, s>>>(nl, N, g.pos_of_id, E->outpos.as<uint32_t>(), E->staging.as<uint32_t>());
    LA3G_LAUNCHED();
    tls_launches += 2;
    for (uint32_t j = 0; j < nl; j++)
    {
      Ticket* t = E->lane[lanes[j0 + j]];
      if (t->q.out)
        LA3G_CUDA(cudaMemcpyAsync(t->q.out, E->staging.as<uint32_t>() + (size_t) j * N, (size_t) N * 4,
                                  cudaMemcpyDeviceToHost, s));
    }
    LA3G_CUDA(cudaStreamSynchronize(s));
  }
  return LA3G_OK;
}

int sssp_loop(Engine* E)
{
  DevGraph& g = E->G->g;
  cudaStream_t s = E->G->stream;
  const uint32_t N = E->N, W = E->W, L = E->L;
  unsigned long long* ctr = E->ctr.as<unsigned long long>();
  PairList PL[2];
  for (int c = 0; c < 2; c++)
    PL[c] = PairList{E->small[c].as<uint32_t>(), E->hub[c].as<uint32_t>(), E->hub_t0[c].as<uint32_t>(), ctr + c,
                     ctr + 2 + c};
  uint32_t busy = 0;
  int cur = 0;
  std::vector<Ticket*> got;
  std::vector<uint32_t> adm, fin;
  for (;;)
  {
    got.clear();
    Ticket* solo = nullptr;
    if (!take_work(E, busy, L - busy, got, E->exact_lanes ? &solo : nullptr)) return LA3G_OK;
    if (solo)
    {
      run_solo(E, solo);
      continue;
    }
    LA3G_TRY(admit(E, got, busy, adm));
    if (!adm.empty())
    {
      const uint32_t n = (uint32_t) adm.size() / 2;
      LA3G_CUDA(cudaMemcpyAsync(E->adm.p, adm.data(), adm.size() * 4, cudaMemcpyHostToDevice, s));
      k_ls_admit<<<grid_for(n, 128), 128, 0, s>>>(E->adm.as<uint32_t>(), n, L, W, g.out_ptr,
                                                 E->reg_end.as<uint32_t>(), g.nreg, g.src_base(), g.iso_base(),
                                                 E->dist.as<uint32_t>(),
                                                 E->sfront[cur].as<uint64_t>(), E->rpos.as<uint32_t>(), PL[cur]);
      LA3G_LAUNCHED();
      tls_launches++;
    }
    if (busy == 0) continue;
    // one relaxation step for every occupied lane
    LA3G_CUDA(cudaMemsetAsync(E->alive[0].p, 0, W * 8, s));
    {
      ProfileScope p("serve_sssp_relax", s, 0.0);
      k_bs_relax<<<num_sms() * 16, 256, 0, s>>>(g.out_ptr, E->reg_end.as<uint32_t>(), g.out_row, g.out_w, L, W,
                                           E->sfront[cur].as<uint64_t>(), PL[cur], E->sfront[cur ^ 1].as<uint64_t>(),
                                           E->dist.as<uint32_t>());
      LA3G_LAUNCHED();
    }
    LA3G_CUDA(cudaMemsetAsync(ctr + (cur ^ 1), 0, 8, s));
    LA3G_CUDA(cudaMemsetAsync(ctr + 2 + (cur ^ 1), 0, 8, s));
    k_bs_apply<<<num_sms() * 8, 256, 0, s>>>(N, W, g.out_ptr, E->reg_end.as<uint32_t>(), E->sfront[cur ^ 1].as<uint64_t>(),
                                        PL[cur ^ 1], E->sfront[cur].as<uint64_t>(), PL[cur],
                                        E->alive[0].as<uint64_t>());
    LA3G_LAUNCHED();
    tls_launches += 2;
    LA3G_CUDA(cudaMemcpyAsync(E->hctr, E->alive[0].p, W * 8, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    cur ^= 1;
    fin.clear();
    for (uint32_t l = 0; l < L; l++)
      if (E->lane[l] && !((E->hctr[l / 64] >> (l % 64)) & 1ull)) fin.push_back(l);
    if (!fin.empty())
    {
      LA3G_TRY(sssp_retire(E, fin));
      for (uint32_t l : fin)
      {
        Ticket* t = E->lane[l];
        E->lane[l] = nullptr;
        busy--;
        finish_ticket(E->S, t, LA3G_OK);
      }
    }
  }
}

int bm25_loop(Engine* E)
{
  std::vector<Ticket*> got;
  for (;;)
  {
    got.clear();
    if (!take_work(E, 0, 1, got)) return LA3G_OK;
    for (Ticket* t : got)
    {
      t->start_ms = wall_ms();
      t->in_flight = 1;
      uint32_t nout = 0;
      // the engine's priority stream for this call (only this worker uses the graph while it is served)
      const cudaStream_t saved = E->G->stream;
      if (E->prio) E->G->stream = E->prio;
      const int st = t->q.kind == LA3G_QUERY_LM
                         ? la3g_lm_query(E->G, t->terms.data(), (uint32_t) t->terms.size(), t->q.k,
                                         (uint32_t*) t->q.out, t->q.scores_out, &nout, nullptr, nullptr, nullptr)
                         : la3g_bm25_query(E->G, t->terms.data(), (uint32_t) t->terms.size(), t->q.k,
                                           (uint32_t*) t->q.out, t->q.scores_out, &nout, nullptr, nullptr, nullptr);
      E->G->stream = saved;
      t->nout = nout;
      finish_ticket(E->S, t, st);
    }
  }
}

void worker(Engine* E)
{
  int st = LA3G_OK;
  if (E->kind == kEngBfs) st = bfs_loop(E);
  else if (E->kind == kEngSssp) st = sssp_loop(E);
  else st = bm25_loop(E);
  if (st != LA3G_OK) engine_fail(E, st);
}

}  // namespace

// ------------------------------------------------------------------ ABI

extern "C" int la3g_server_create(uint64_t budget_bytes, uint32_t bfs_lanes, uint32_t sssp_lanes, la3g_server** out)
{
  if (!out) return set_error(LA3G_EINVAL, "out is null");
  *out = nullptr;
  if (bfs_lanes == 0) bfs_lanes = 256;
  if (sssp_lanes == 0) sssp_lanes = 256;
  if (bfs_lanes % 64 || sssp_lanes % 64 || bfs_lanes > 4096 || sssp_lanes > 4096)
    return set_error(LA3G_EINVAL, "lane counts must be multiples of 64, at most 4096");
  la3g_server* S = new (std::nothrow) la3g_server();
  if (!S) return set_error(LA3G_ENOMEM, "out of host memory");
  S->budget = budget_bytes;
  S->bfs_lanes = bfs_lanes;
  S->sssp_lanes = sssp_lanes;
  *out = S;
  return LA3G_OK;
}

extern "C" int la3g_server_add_graph(la3g_server* S, la3g_graph* G, uint32_t* graph_id)
{
  if (!S || !G) return set_error(LA3G_EINVAL, "null server or graph");
  DevGraph& g = G->g;
  int kind = 0;
  if (g.flags & LA3G_BIPARTITE) kind = kEngBm25;
  else if (!g.directed()) kind = kEngBfs;
  else if (g.weighted() && !(g.flags & (LA3G_REVERSE | LA3G_ACYCLIC))) kind = kEngSssp;
  else return set_error(LA3G_EINVAL, "serve graphs loaded undirected (BFS), DIRECTED|WEIGHTED (SSSP) or BIPARTITE (BM25)");
  {
    std::lock_guard<std::mutex> lk(S->mu);
    for (Engine* e : S->engines)
      if (e->G == G) return set_error(LA3G_EINVAL, "graph already served");
  }
  if (kind == kEngSssp) LA3G_TRY(build_push_csr(G));
  if (kind == kEngBm25 && !G->slot[kSlotBm25]) LA3G_TRY(la3g_bm25_prepare(G, nullptr, nullptr, nullptr));
  if (kind == kEngBm25)
  {
    // LM too; one empty query takes the first query's leftover term activity
    // (lm.cpp:46-86), so every served LM query sees the steady state
    if (!G->slot[kSlotLm]) LA3G_TRY(la3g_lm_prepare(G, nullptr, nullptr));
    LA3G_TRY(la3g_lm_query(G, nullptr, 0, 0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr));
  }
  const uint32_t N = g.nslots;
  uint32_t L = kind == kEngBfs ? S->bfs_lanes : (kind == kEngSssp ? S->sssp_lanes : 0);
  auto need = [&](uint32_t lanes) -> uint64_t {
    if (kind == kEngBfs) return bfs_lane_bytes(N, lanes);
    if (kind == kEngSssp) return sssp_lane_bytes(N, lanes);
    return 0;
  };
  uint64_t eng_bytes = 0;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    const uint64_t left = S->budget > S->used ? S->budget - S->used : 0;
    while (L > 64 && G->device_bytes + need(L) > left) L /= 2;
    eng_bytes = need(L);
    if (G->device_bytes + eng_bytes > left)
      return set_error(LA3G_EBUDGET, "graph and its lane state exceed the server's HBM budget");
    S->used += G->device_bytes + eng_bytes;  // reserved before allocation
  }
  Engine* E = new (std::nothrow) Engine();
  if (!E)
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->used -= G->device_bytes + eng_bytes;
    return set_error(LA3G_ENOMEM, "out of host memory");
  }
  E->S = S;
  E->G = G;
  E->kind = kind;
  E->N = N;
  E->L = L;
  E->W = L / 64;
  E->bytes = eng_bytes;
  E->lane.assign(L, nullptr);
  E->wlevel.assign(E->W, 0);
  E->wbusy.assign(E->W, 0);
  int st = LA3G_OK;
  if (kind == kEngBm25)
  {
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess ||
        cudaStreamCreateWithPriority(&E->prio, cudaStreamNonBlocking, greatest) != cudaSuccess)
    {
      cudaGetLastError();
      E->prio = nullptr;  // served on the graph's own stream
    }
  }
  if (kind != kEngBm25)
  {
    E->pos_of_id.resize(N);
    st = la3g_graph_positions(G, E->pos_of_id.data(), nullptr);
    if (st == LA3G_OK && cudaHostAlloc(&E->hctr, 64 * 8 + E->W * 8, cudaHostAllocDefault) != cudaSuccess)
      st = set_error(LA3G_ECUDA, "pinned counter allocation failed");
    if (st == LA3G_OK) st = kind == kEngBfs ? bfs_engine_init(E) : sssp_engine_init(E);
    if (st == LA3G_OK && cudaStreamSynchronize(G->stream) != cudaSuccess)
      st = set_error(LA3G_ECUDA, "engine initialisation failed");
  }
  if (st != LA3G_OK)
  {
    if (E->hctr) cudaFreeHost(E->hctr);
    if (E->prio) cudaStreamDestroy(E->prio);
    delete E;
    std::lock_guard<std::mutex> lk(S->mu);
    S->used -= G->device_bytes + eng_bytes;
    return st;
  }
  {
    std::lock_guard<std::mutex> lk(S->mu);
    E->id = (uint32_t) S->engines.size();
    S->engines.push_back(E);
  }
  E->th = std::thread(worker, E);
  if (graph_id) *graph_id = E->id;
  return LA3G_OK;
}

extern "C" int la3g_server_submit(la3g_server* S, const la3g_query* q, uint64_t* ticket)
{
  if (!S || !q || !ticket) return set_error(LA3G_EINVAL, "null argument");
  Ticket* t = new (std::nothrow) Ticket();
  if (!t) return set_error(LA3G_ENOMEM, "out of host memory");
  t->q = *q;
  t->submit_ms = wall_ms();
  std::lock_guard<std::mutex> lk(S->mu);
  if (q->graph >= S->engines.size())
  {
    delete t;
    return set_error(LA3G_EINVAL, "no such graph id");
  }
  Engine* E = S->engines[q->graph];
  const int want = q->kind == LA3G_QUERY_BFS ? kEngBfs : q->kind == LA3G_QUERY_SSSP ? kEngSssp
                                                    : (q->kind == LA3G_QUERY_BM25 || q->kind == LA3G_QUERY_LM) ? kEngBm25 : -1;
  if (want != E->kind)
  {
    delete t;
    return set_error(LA3G_EINVAL, "query kind does not match the graph");
  }
  if (E->error != LA3G_OK)
  {
    delete t;
    return set_error(E->error, "the graph's engine failed: %s", E->error_msg.c_str());
  }
  if (want == kEngBm25)
  {
    if (!q->terms || q->nterms == 0 || q->k == 0)
    {
      delete t;
      return set_error(LA3G_EINVAL, "bm25 / lm queries need terms and k > 0");
    }
    t->terms.assign(q->terms, q->terms + q->nterms);
    t->q.terms = nullptr;
  }
  const uint64_t id = S->next_ticket++;
  S->tickets[id] = t;
  E->queue.push_back(t);
  E->cv.notify_one();
  *ticket = id;
  return LA3G_OK;
}

extern "C" int la3g_server_poll(la3g_server* S, uint64_t ticket, int timeout_ms, la3g_query_result* res)
{
  if (!S) return set_error(LA3G_EINVAL, "null server");
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->tickets.find(ticket);
  if (it == S->tickets.end()) return set_error(LA3G_EINVAL, "unknown ticket");
  Ticket* t = it->second;
  if (t->status < 0 && timeout_ms != 0)
  {
    auto pred = [&] { return t->status >= 0; };
    if (timeout_ms < 0) S->done_cv.wait(lk, pred);
    else S->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred);
  }
  if (t->status < 0) return LA3G_EBUSY;
  if (res)
  {
    res->status = t->status;
    res->kind = t->q.kind;
    res->queue_ms = t->start_ms - t->submit_ms;
    res->latency_ms = t->done_ms - t->submit_ms;
    res->in_flight = t->in_flight;
    res->nout = t->nout;
  }
  S->tickets.erase(it);
  delete t;
  return LA3G_OK;
}

extern "C" int la3g_server_info(la3g_server* S, la3g_server_stats* out)
{
  if (!S || !out) return set_error(LA3G_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  std::memset(out, 0, sizeof(*out));
  out->budget_bytes = S->budget;
  out->used_bytes = S->used;
  out->ngraphs = (uint32_t) S->engines.size();
  out->completed = S->completed.load();
  uint64_t pend = 0;
  for (Engine* e : S->engines) pend += e->queue.size();
  out->queued = pend;
  out->pending = S->tickets.size();
  return LA3G_OK;
}

extern "C" int la3g_server_set_solo(la3g_server* S, uint32_t bfs_depth, uint32_t sssp_depth)
{
  if (!S) return set_error(LA3G_EINVAL, "null server");
  std::lock_guard<std::mutex> lk(S->mu);
  S->solo_bfs = bfs_depth;
  S->solo_sssp = sssp_depth;
  return LA3G_OK;
}

extern "C" int la3g_server_lanes(la3g_server* S, uint32_t graph_id, uint32_t* lanes)
{
  if (!S || !lanes) return set_error(LA3G_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  if (graph_id >= S->engines.size()) return set_error(LA3G_EINVAL, "no such graph id");
  *lanes = S->engines[graph_id]->L;
  return LA3G_OK;
}

extern "C" void la3g_server_free(la3g_server* S)
{
  if (!S) return;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    for (Engine* e : S->engines)
    {
      e->stop = true;
      e->cv.notify_all();
    }
  }
  for (Engine* e : S->engines)
    if (e->th.joinable()) e->th.join();
  // every worker synchronises its stream before it waits for work, so once
  // the threads are joined no engine work is in flight (the graphs are not
  // touched here: they may already be gone)
  for (Engine* e : S->engines)
  {
    if (e->hctr) cudaFreeHost(e->hctr);
    if (e->prio) cudaStreamDestroy(e->prio);
    delete e;
  }
  for (auto& kv : S->tickets) delete kv.second;
  delete S;
}
