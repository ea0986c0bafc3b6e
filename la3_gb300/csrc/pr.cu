// PageRank: the reference pr app (src/apps/graph_analytics/pr.cpp:11-55,
// pr.h:12-46) on the device.
//
// Reference semantics kept exactly:
//   * degree = number of distinct out-neighbours (DegVertex on the reversed
//     graph, pr.cpp:14-21, degree.h:24-35);
//   * rank starts at alpha = 0.15; x = rank / degree (pr.h:37);
//   * every iteration (the app is stationary) each regular row sums the
//     messages of its in-neighbours, source columns first, then regular
//     columns, each ascending (vertex_program_execute.hpp:479-482,
//     564-603), in FP64, one addition at a time in that order; then
//     rank = alpha + (1 - alpha) * y (pr.h:40-45);
//   * sinks are computed once after the iterations from the final regular
//     ranks (vertex_program_execute.hpp:131-148); sources and isolated
//     vertices keep alpha.
// Every floating-point operation is an explicit round-to-nearest intrinsic,
// so nothing is contracted into an FMA and the result is bit-identical to
// the reference built without contraction.
//
// Kernel layout (pr_pull): one warp owns 32 consecutive rows; it streams the
// rows' in-edges in chunks of 32 x 8 entries through shared memory (coalesced
// index loads, gathered x values) and each lane adds its own row's values in
// order.  Rows longer than kLongRow are skipped there and summed by a single
// lane that walks the row sequentially with its warp prefetching the values;
// those warps are the first blocks of the same launch, so the long chains
// start first.
#include <algorithm>
#include <cstring>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "la3g_internal.h"

namespace la3g {

static constexpr double kAlpha = 0.15;
static constexpr double kTol = 1e-5;
static constexpr uint32_t kLongRow = 1024;
static constexpr int kChunk = 256;  // edges staged per warp per step
static constexpr int kWarpsPerBlock = 8;

struct PrScratch
{
  uint32_t* deg = nullptr;      // [nslots] out-degree
  double* rank = nullptr;       // [nslots]
  double* x[2] = {nullptr, nullptr};  // [nslots] messages (scatter values)
  uint32_t* long_rows = nullptr;      // rows with degree > kLongRow, descending
  uint32_t nlong = 0;
  int* flag = nullptr;          // any-activated flag
  float* xf[2] = {nullptr, nullptr};  // FP32 study
  float* rankf = nullptr;
  double* resid = nullptr;
  bool ready = false;
  // tiled layout of the regular rows (la3g_pr_f32_tiled), built on first use
  uint32_t tile_rows = 0, ntiles = 0;
  uint64_t tile_ncols = 0, tile_nent = 0;
  uint32_t* tile_col = nullptr;  // [ntiles + 1] first non-empty-column slot of each tile
  uint32_t* tcol = nullptr;      // [ncols] column positions, ascending within a tile
  uint32_t* tptr = nullptr;      // [ncols + 1] first entry of each non-empty column
  uint16_t* trow = nullptr;      // [nent] row of each entry, local to its tile
  uint32_t* tecol = nullptr;     // [nent] column of each entry (the hypersparse tiles' form)
  int tile_blocks = 0;           // resident blocks per SM of the tiled kernel
};

static void pr_scratch_free(void* p) { delete (PrScratch*) p; }

__global__ void k_outdeg(const uint32_t* __restrict__ col, uint64_t m, uint32_t* __restrict__ deg)
{
  for (uint64_t e = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (uint64_t) gridDim.x * blockDim.x)
    atomicAdd(&deg[col[e]], 1u);
}

__global__ void k_pr_init(uint32_t N, uint32_t nreg, uint32_t src_base, uint32_t iso_base,
                          const uint32_t* __restrict__ deg, double* rank, double* x0, double* x1)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x)
  {
    rank[p] = kAlpha;
    // init(vid, other, s) returns true for everyone, so regular and source
    // vertices scatter rank / degree (pr.h:34-37); sinks and isolated
    // vertices have no out-edges and are never read as columns.
    double xv = 0.0;
    if (p < nreg || (p >= src_base && p < iso_base)) xv = __ddiv_rn(kAlpha, (double) deg[p]);
    x0[p] = xv;
    x1[p] = xv;
  }
}

__global__ void k_mark_long(const uint32_t* __restrict__ ptr, uint32_t nrows, uint32_t* keys, uint32_t* vals,
                            uint32_t* count)
{
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x)
  {
    uint32_t d = ptr[r + 1] - ptr[r];
    if (d > kLongRow)
    {
      uint32_t i = atomicAdd(count, 1u);
      keys[i] = ~d;  // ascending sort of ~d = descending degree
      vals[i] = r;
    }
  }
}

// rank = alpha + (1 - alpha) * y with y = 0.0 + partial (combine into A()).
__device__ __forceinline__ double pr_apply(double partial)
{
  double y = __dadd_rn(0.0, partial);
  return __dadd_rn(kAlpha, __dmul_rn(1.0 - kAlpha, y));
}

__device__ __forceinline__ void pr_finish_row(uint32_t r, double acc, const uint32_t* __restrict__ deg, double* rank,
                                              double* xnext, int* flag, bool write_x)
{
  double old = rank[r];
  double nr = pr_apply(acc);
  rank[r] = nr;
  if (write_x) xnext[r] = __ddiv_rn(nr, (double) deg[r]);
  if (flag && fabs(__dsub_rn(nr, old)) > kTol) *flag = 1;
}

// Rows [row_lo, row_hi).  Blocks [0, long_blocks) take the long rows (one
// warp per row, descending length); the rest take 32-row tiles.
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
k_pr_pull(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, const double* __restrict__ x,
          double* __restrict__ xnext, double* __restrict__ rank, const uint32_t* __restrict__ deg,
          const uint32_t* __restrict__ long_rows, uint32_t nlong, uint32_t long_blocks, uint32_t row_lo,
          uint32_t row_hi, int* flag, int write_x)
{
  __shared__ double sx[kWarpsPerBlock][kChunk];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  if (blockIdx.x < long_blocks)
  {
    for (uint32_t li = blockIdx.x * kWarpsPerBlock + wib; li < nlong; li += long_blocks * kWarpsPerBlock)
    {
      uint32_t r = long_rows[li];
      if (r < row_lo || r >= row_hi) continue;
      uint32_t b = ptr[r], e = ptr[r + 1];
      double acc = 0.0;
      // prefetch one chunk ahead; lane 0 adds sequentially
      double v[kChunk / 32];
#pragma unroll
      for (int k = 0; k < kChunk / 32; k++)
      {
        uint32_t i = b + k * 32 + lane;
        v[k] = i < e ? x[col[i]] : 0.0;
      }
      for (uint32_t base = b; base < e; base += kChunk)
      {
#pragma unroll
        for (int k = 0; k < kChunk / 32; k++) sx[wib][k * 32 + lane] = v[k];
        __syncwarp();
        uint32_t nb = base + kChunk;
#pragma unroll
        for (int k = 0; k < kChunk / 32; k++)
        {
          uint32_t i = nb + k * 32 + lane;
          v[k] = i < e ? x[col[i]] : 0.0;
        }
        if (lane == 0)
        {
          uint32_t n = min((uint32_t) kChunk, e - base);
          if (n == kChunk)
          {
#pragma unroll 32
            for (uint32_t j = 0; j < kChunk; j++) acc = __dadd_rn(acc, sx[wib][j]);
          }
          else
          {
            for (uint32_t j = 0; j < n; j++) acc = __dadd_rn(acc, sx[wib][j]);
          }
        }
        __syncwarp();
      }
      if (lane == 0) pr_finish_row(r, acc, deg, rank, xnext, flag, write_x);
    }
    return;
  }
  const uint32_t ntiles = (row_hi - row_lo + 31) / 32;
  const uint32_t nwarps = (gridDim.x - long_blocks) * kWarpsPerBlock;
  for (uint32_t t = (blockIdx.x - long_blocks) * kWarpsPerBlock + wib; t < ntiles; t += nwarps)
  {
    const uint32_t r0 = row_lo + t * 32;
    const uint32_t r = r0 + lane;
    const bool valid = r < row_hi;
    uint32_t rb = valid ? ptr[r] : 0, re = valid ? ptr[r + 1] : 0;
    const bool mine = valid && (re - rb) <= kLongRow;
    if (!mine) { rb = 0; re = 0; }
    // Walk the short rows' edges in chunks; each chunk starts at the lowest
    // edge any lane still needs, which skips over the long rows' edges.
    const uint32_t te = ptr[min(r0 + 32, row_hi)];
    double acc = 0.0;
    uint32_t cur = rb;  // next edge of my row to add
    for (;;)
    {
      const uint32_t base = __reduce_min_sync(0xffffffffu, cur < re ? cur : 0xffffffffu);
      if (base == 0xffffffffu) break;
      const uint32_t lim = min(base + kChunk, te);
#pragma unroll
      for (int k = 0; k < kChunk / 32; k++)
      {
        uint32_t i = base + k * 32 + lane;
        if (i < lim) sx[wib][k * 32 + lane] = x[col[i]];
      }
      __syncwarp();
      const uint32_t stop = min(re, lim);
      for (; cur < stop; cur++) acc = __dadd_rn(acc, sx[wib][cur - base]);
      __syncwarp();
    }
    if (mine) pr_finish_row(r, acc, deg, rank, xnext, flag, write_x);
  }
}

__global__ void k_scatter_pos(uint32_t N, const uint32_t* __restrict__ id_of_pos, const double* __restrict__ val,
                              double* __restrict__ out)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) out[id_of_pos[p]] = val[p];
}

__global__ void k_scatter_pos_u32(uint32_t N, const uint32_t* __restrict__ id_of_pos, const uint32_t* __restrict__ val,
                                  uint32_t* __restrict__ out)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) out[id_of_pos[p]] = val[p];
}

static int pr_prepare(la3g_graph* G, PrScratch** out)
{
  DevGraph& g = G->g;
  cudaStream_t s = G->stream;
  PrScratch* ps = (PrScratch*) G->slot[kSlotPr];
  if (ps && ps->ready) { *out = ps; return LA3G_OK; }
  if (!ps)
  {
    ps = new (std::nothrow) PrScratch();
    if (!ps) return set_error(LA3G_ENOMEM, "out of host memory");
    G->slot[kSlotPr] = ps;
    G->slot_free[kSlotPr] = pr_scratch_free;
  }
  const uint32_t N = g.nslots;
  LA3G_TRY(galloc(G, &ps->deg, N));
  LA3G_TRY(galloc(G, &ps->rank, N));
  LA3G_TRY(galloc(G, &ps->x[0], N));
  LA3G_TRY(galloc(G, &ps->x[1], N));
  LA3G_TRY(galloc(G, &ps->flag, 4));
  LA3G_CUDA(cudaMemsetAsync(ps->deg, 0, (size_t) N * 4, s));
  if (g.nent)
  {
    ProfileScope ps_("pr_outdeg", s, (double) g.nent * 4);
    k_outdeg<<<grid_for(g.nent, 256), 256, 0, s>>>(g.in_col, g.nent, ps->deg);
    LA3G_LAUNCHED();
  }
  // long rows, sorted by descending degree
  DevBuf keys, vals, keys2, vals2, cnt;
  LA3G_TRY(keys.alloc((size_t) g.nrows() * 4 + 4));
  LA3G_TRY(vals.alloc((size_t) g.nrows() * 4 + 4));
  LA3G_TRY(cnt.alloc(4));
  LA3G_CUDA(cudaMemsetAsync(cnt.p, 0, 4, s));
  if (g.nrows())
  {
    k_mark_long<<<grid_for(g.nrows(), 256), 256, 0, s>>>(g.in_ptr, g.nrows(), keys.as<uint32_t>(), vals.as<uint32_t>(),
                                                         cnt.as<uint32_t>());
    LA3G_LAUNCHED();
  }
  uint32_t nlong = 0;
  LA3G_CUDA(cudaMemcpyAsync(&nlong, cnt.p, 4, cudaMemcpyDeviceToHost, s));
  LA3G_CUDA(cudaStreamSynchronize(s));
  ps->nlong = nlong;
  LA3G_TRY(galloc(G, &ps->long_rows, nlong + 1));
  if (nlong)
  {
    LA3G_TRY(keys2.alloc((size_t) nlong * 4 + 4));
    size_t tb = 0;
    LA3G_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, keys.as<uint32_t>(), keys2.as<uint32_t>(), vals.as<uint32_t>(),
                                              ps->long_rows, nlong, 0, 32, s));
    DevBuf tmp;
    LA3G_TRY(tmp.alloc(tb));
    LA3G_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tb, keys.as<uint32_t>(), keys2.as<uint32_t>(), vals.as<uint32_t>(),
                                              ps->long_rows, nlong, 0, 32, s));
  }
  LA3G_CUDA(cudaStreamSynchronize(s));
  ps->ready = true;
  *out = ps;
  return LA3G_OK;
}

static int pr_launch(la3g_graph* G, PrScratch* ps, const double* x, double* xnext, uint32_t row_lo, uint32_t row_hi,
                     int* flag, bool write_x)
{
  DevGraph& g = G->g;
  if (row_hi <= row_lo) return LA3G_OK;
  const uint32_t long_blocks = ps->nlong ? std::min<uint32_t>((ps->nlong + kWarpsPerBlock - 1) / kWarpsPerBlock, num_sms()) : 0;
  const uint32_t ntiles = (row_hi - row_lo + 31) / 32;
  const uint32_t tile_blocks = std::min<uint32_t>((ntiles + kWarpsPerBlock - 1) / kWarpsPerBlock, num_sms() * 8);
  uint64_t edges = 0;  // algorithmic bytes: 4 B index per edge + per-row ptr, x, rank, xnext
  (void) edges;
  double bytes = 4.0 * (double) g.nent + 4.0 * (row_hi - row_lo + 1) + 8.0 * (double) g.nslots +
                 (write_x ? 16.0 : 8.0) * (row_hi - row_lo) + 4.0 * (row_hi - row_lo);
  ProfileScope p("pr_pull_f64", G->stream, bytes);
  k_pr_pull<<<long_blocks + std::max<uint32_t>(tile_blocks, 1), kWarpsPerBlock * 32, 0, G->stream>>>(
      g.in_ptr, g.in_col, x, xnext, ps->rank, ps->deg, ps->long_rows, ps->nlong, long_blocks, row_lo, row_hi, flag,
      write_x ? 1 : 0);
  LA3G_LAUNCHED();
  return LA3G_OK;
}

// ------------------------------------------------------------------ FP32 study

__global__ void k_prf_init(uint32_t N, uint32_t nrows_reg, uint32_t src_base, uint32_t iso_base,
                           const uint32_t* __restrict__ deg, float* rankf, double* rank, float* x0, float* x1)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x)
  {
    rankf[p] = (float) kAlpha;
    rank[p] = kAlpha;
    float xv = 0.0f;
    bool scat = (p < nrows_reg) || (p >= src_base && p < iso_base);
    if (scat && deg[p]) xv = (float) kAlpha / (float) deg[p];
    x0[p] = xv;
    x1[p] = xv;
  }
}

__device__ __forceinline__ double prf_finish(uint32_t r, float acc, float* __restrict__ xnext, float* __restrict__ rankf,
                                             double* __restrict__ rank, const uint32_t* __restrict__ deg, int write_x)
{
  const float nr = (float) kAlpha + (float) (1.0 - kAlpha) * acc;
  const double d = fabs((double) nr - (double) rankf[r]);
  rankf[r] = nr;
  rank[r] = (double) nr;
  if (write_x) xnext[r] = nr / (float) deg[r];
  return d;
}

// FP32 SpMV with FP32 accumulation (any order inside a row is allowed
// here).  The first `long_blocks` blocks take the rows longer than
// kLongRow, one block per row with a shared-memory reduction; the others
// give each row of at most kLongRow edges a group of 4 lanes (eight rows
// per warp), so average-degree rows keep the lanes busy.  The L1 residual
// is reduced in FP64.
__global__ void __launch_bounds__(256)
k_prf_pull(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col, const float* __restrict__ x,
           float* __restrict__ xnext, float* __restrict__ rankf, double* __restrict__ rank,
           const uint32_t* __restrict__ deg, const uint32_t* __restrict__ long_rows, uint32_t nlong,
           uint32_t long_blocks, uint32_t row_lo, uint32_t row_hi, double* resid, int write_x)
{
  const int lane = threadIdx.x & 31;
  double local = 0.0;
  if (blockIdx.x < long_blocks)
  {
    __shared__ float part[8];
    for (uint32_t k = blockIdx.x; k < nlong; k += long_blocks)
    {
      const uint32_t r = long_rows[k];
      if (r < row_lo || r >= row_hi) continue;  // uniform per block
      float acc = 0.0f;
      for (uint32_t i = ptr[r] + threadIdx.x; i < ptr[r + 1]; i += blockDim.x) acc += x[col[i]];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) part[threadIdx.x >> 5] = acc;
      __syncthreads();
      if (threadIdx.x == 0)
      {
        float t = 0.0f;
        for (int w = 0; w < (int) (blockDim.x >> 5); w++) t += part[w];
        local += prf_finish(r, t, xnext, rankf, rank, deg, write_x);
      }
      __syncthreads();
    }
    if (threadIdx.x == 0 && local != 0.0) atomicAdd(resid, local);
    return;
  }
  // short rows: 4 lanes per row, each keeping four independent loads in
  // flight per step (the step is bound by memory latency)
  constexpr uint32_t G = 4;
  const uint32_t sub = lane & (G - 1);
  const uint32_t group = ((blockIdx.x - long_blocks) * blockDim.x + threadIdx.x) / G;
  const uint32_t ngroups = ((gridDim.x - long_blocks) * blockDim.x) / G;
  const uint32_t nrows = row_hi - row_lo;
  // all groups of a warp run the same number of rounds
  const uint32_t rounds = (nrows + ngroups - 1) / ngroups;
  for (uint32_t k = 0; k < rounds; k++)
  {
    const uint32_t r = row_lo + group + k * ngroups;
    float acc = 0.0f;
    bool mine = false;
    if (r < row_hi)
    {
      const uint32_t b = ptr[r], e = ptr[r + 1];
      mine = (e - b) <= kLongRow;
      if (mine)
        for (uint32_t i = b + sub; i < e; i += 4 * G)
        {
          uint32_t c[4];
#pragma unroll
          for (int u = 0; u < 4; u++) c[u] = i + u * G < e ? col[i + u * G] : 0xFFFFFFFFu;
          float v[4];
#pragma unroll
          for (int u = 0; u < 4; u++) v[u] = c[u] != 0xFFFFFFFFu ? x[c[u]] : 0.0f;
#pragma unroll
          for (int u = 0; u < 4; u++) acc += v[u];
        }
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (mine && sub == 0) local += prf_finish(r, acc, xnext, rankf, rank, deg, write_x);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  // one FP64 atomic per block (per-warp atomics on one word serialise)
  __shared__ double wsum[8];
  if (lane == 0) wsum[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x == 0)
  {
    double t = 0.0;
    for (int w = 0; w < (int) (blockDim.x >> 5); w++) t += wsum[w];
    if (t != 0.0) atomicAdd(resid, t);
  }
}

// ------------------------------------------------------------- tiled layout
//
// The regular rows are cut into tiles of kTileRows consecutive rows.  Each
// tile keeps its entries doubly compressed by column (the reference's
// per-tile DCSC, src/utils/csc.h:60-130: only the non-empty columns are
// listed, with their offsets): tcol / tptr over the tile's non-empty columns
// in ascending position, and a 16-bit row inside the tile per entry.  One
// CTA takes a tile at a time with its rows' accumulators in shared memory,
// walks the tile's columns (one thread per column, four columns' messages
// loaded at once; columns with many entries in the tile go to whole warps)
// and adds each column's message into its rows with shared-memory atomics,
// so every message is read once per tile and no row needs a reduction across
// lanes.  Rows with more than kLongRow in-edges stay out of the tiles (their
// thousands of additions would serialise on one shared-memory word) and are
// summed a block each by the first blocks of the same launch.
// Addition order inside a row is free in the FP32 study (the FP64 path keeps
// the reference's order on the flat CSR).
static constexpr uint32_t kTileRows = 2048;    // rows per tile: 8 KB of FP32 accumulators
static constexpr uint32_t kTileThreads = 512;
static constexpr uint32_t kTileBig = 32;       // columns with more entries in a tile go to a warp
static constexpr uint32_t kTileBigCap = 1024;  // such columns queued per tile (the rest run serially)
static constexpr uint32_t kTileDense = 2;      // entries per non-empty column at which a tile walks its DCSC columns

__global__ void k_tile_colof(const uint32_t* __restrict__ ptr, uint32_t ncol, uint32_t* colof)
{
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < ncol; c += gridDim.x * blockDim.x)
    for (uint32_t i = ptr[c]; i < ptr[c + 1]; i++) colof[i] = c;
}

// Tile of each push entry; entries of sink rows and of long regular rows
// (more than kLongRow in-edges: summed by the flat kernel's block-per-row
// path, since thousands of additions into one shared-memory word would
// serialise) sort last and are dropped.
__global__ void k_tile_keys(const uint32_t* __restrict__ row, uint64_t m, uint32_t nreg,
                            const uint32_t* __restrict__ in_ptr, uint32_t* key, uint32_t* idx,
                            unsigned long long* kept)
{
  unsigned long long c = 0;
  for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < m; i += (uint64_t) gridDim.x * blockDim.x)
  {
    const uint32_t r = row[i];
    const bool keep = r < nreg && in_ptr[r + 1] - in_ptr[r] <= kLongRow;
    key[i] = keep ? r / kTileRows : 0xFFFFFFFFu;
    idx[i] = (uint32_t) i;
    c += keep;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(kept, c);
}

// Entries in (tile, column, row) order: local rows, and a flag where a new
// (tile, column) pair starts.
__global__ void k_tile_flags(const uint32_t* __restrict__ order, uint64_t n, const uint32_t* __restrict__ colof,
                             const uint32_t* __restrict__ row, uint16_t* trow, uint32_t* tecol, uint32_t* flag)
{
  for (uint64_t e = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; e < n; e += (uint64_t) gridDim.x * blockDim.x)
  {
    const uint32_t i = order[e];
    const uint32_t r = row[i], t = r / kTileRows;
    trow[e] = (uint16_t) (r - t * kTileRows);
    tecol[e] = colof[i];
    bool start = e == 0;
    if (!start)
    {
      const uint32_t j = order[e - 1];
      start = colof[j] != colof[i] || row[j] / kTileRows != t;
    }
    flag[e] = start ? 1u : 0u;
  }
}

__global__ void k_tile_cols(const uint32_t* __restrict__ order, uint64_t n, const uint32_t* __restrict__ colof,
                            const uint32_t* __restrict__ row, const uint32_t* __restrict__ flag,
                            const uint32_t* __restrict__ slot, uint32_t* tcol, uint32_t* tptr, uint32_t* tile_col)
{
  for (uint64_t e = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; e < n; e += (uint64_t) gridDim.x * blockDim.x)
  {
    if (!flag[e]) continue;
    const uint32_t i = order[e], k = slot[e];
    tcol[k] = colof[i];
    tptr[k] = (uint32_t) e;
    const uint32_t t = row[i] / kTileRows;
    if (e == 0 || row[order[e - 1]] / kTileRows != t) tile_col[t] = k;
  }
}

static int pr_build_tiles(la3g_graph* G, PrScratch* ps)
{
  if (ps->tile_col) return LA3G_OK;
  DevGraph& g = G->g;
  cudaStream_t s = G->stream;
  LA3G_TRY(build_push_csr(G));
  const uint64_t m = g.nent;
  const uint32_t ntiles = (g.nreg + kTileRows - 1) / kTileRows;
  DevBuf colof, key, key2, idx, idx2, flag, slot, tmp, kept;
  LA3G_TRY(kept.alloc(8));
  LA3G_CUDA(cudaMemsetAsync(kept.p, 0, 8, s));
  LA3G_TRY(colof.alloc(m * 4 + 4));
  LA3G_TRY(key.alloc(m * 4 + 4));
  LA3G_TRY(key2.alloc(m * 4 + 4));
  LA3G_TRY(idx.alloc(m * 4 + 4));
  LA3G_TRY(idx2.alloc(m * 4 + 4));
  if (m)
  {
    k_tile_colof<<<grid_for(g.nslots, 256), 256, 0, s>>>(g.out_ptr, g.nslots, colof.as<uint32_t>());
    LA3G_LAUNCHED();
    k_tile_keys<<<grid_for(m, 256), 256, 0, s>>>(g.out_row, m, g.nreg, g.in_ptr, key.as<uint32_t>(), idx.as<uint32_t>(),
                                                 kept.as<unsigned long long>());
    LA3G_LAUNCHED();
    // stable by tile: the push CSR's (column, row) order is kept inside each tile
    size_t tb = 0;
    LA3G_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, key.as<uint32_t>(), key2.as<uint32_t>(), idx.as<uint32_t>(),
                                              idx2.as<uint32_t>(), (int64_t) m, 0, 32, s));
    LA3G_TRY(tmp.alloc(tb));
    LA3G_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tb, key.as<uint32_t>(), key2.as<uint32_t>(), idx.as<uint32_t>(),
                                              idx2.as<uint32_t>(), (int64_t) m, 0, 32, s));
  }
  // the kept entries sort first
  unsigned long long nkept = 0;
  LA3G_CUDA(cudaMemcpyAsync(&nkept, kept.p, 8, cudaMemcpyDeviceToHost, s));
  LA3G_CUDA(cudaStreamSynchronize(s));
  const uint64_t n = nkept;
  LA3G_TRY(flag.alloc(n * 4 + 4));
  LA3G_TRY(slot.alloc(n * 4 + 4));
  LA3G_TRY(galloc(G, &ps->trow, n + 8));
  LA3G_TRY(galloc(G, &ps->tecol, n + 8));
  uint32_t ncols = 0;
  if (n)
  {
    k_tile_flags<<<grid_for(n, 256), 256, 0, s>>>(idx2.as<uint32_t>(), n, colof.as<uint32_t>(), g.out_row, ps->trow,
                                                  ps->tecol, flag.as<uint32_t>());
    LA3G_LAUNCHED();
    size_t tb = 0;
    LA3G_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, flag.as<uint32_t>(), slot.as<uint32_t>(), (int64_t) n, s));
    LA3G_TRY(tmp.alloc(tb));
    LA3G_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, tb, flag.as<uint32_t>(), slot.as<uint32_t>(), (int64_t) n, s));
    uint32_t last[2];
    LA3G_CUDA(cudaMemcpyAsync(&last[0], slot.as<uint32_t>() + n - 1, 4, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaMemcpyAsync(&last[1], flag.as<uint32_t>() + n - 1, 4, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    ncols = last[0] + last[1];
  }
  LA3G_TRY(galloc(G, &ps->tcol, (size_t) ncols + 1));
  LA3G_TRY(galloc(G, &ps->tptr, (size_t) ncols + 1));
  LA3G_TRY(galloc(G, &ps->tile_col, (size_t) ntiles + 1));
  std::vector<uint32_t> tc(ntiles + 1, ncols);
  LA3G_CUDA(cudaMemcpyAsync(ps->tile_col, tc.data(), tc.size() * 4, cudaMemcpyHostToDevice, s));
  if (n)
  {
    k_tile_cols<<<grid_for(n, 256), 256, 0, s>>>(idx2.as<uint32_t>(), n, colof.as<uint32_t>(), g.out_row,
                                                 flag.as<uint32_t>(), slot.as<uint32_t>(), ps->tcol, ps->tptr,
                                                 ps->tile_col);
    LA3G_LAUNCHED();
  }
  const uint32_t end = (uint32_t) n;
  LA3G_CUDA(cudaMemcpyAsync(ps->tptr + ncols, &end, 4, cudaMemcpyHostToDevice, s));
  // empty tiles start where the next tile starts
  LA3G_CUDA(cudaMemcpyAsync(tc.data(), ps->tile_col, tc.size() * 4, cudaMemcpyDeviceToHost, s));
  LA3G_CUDA(cudaStreamSynchronize(s));
  for (int64_t t = (int64_t) ntiles - 1; t >= 0; t--) tc[t] = std::min(tc[t], tc[t + 1]);
  LA3G_CUDA(cudaMemcpyAsync(ps->tile_col, tc.data(), tc.size() * 4, cudaMemcpyHostToDevice, s));
  LA3G_CUDA(cudaStreamSynchronize(s));
  ps->tile_rows = kTileRows;
  ps->ntiles = ntiles;
  ps->tile_ncols = ncols;
  ps->tile_nent = n;
  return LA3G_OK;
}

__global__ void __launch_bounds__(kTileThreads)
k_prf_tiles(const uint32_t* __restrict__ tile_col, const uint32_t* __restrict__ tcol,
            const uint32_t* __restrict__ tptr, const uint16_t* __restrict__ trow,
            const uint32_t* __restrict__ tecol, uint32_t ntiles, uint32_t nreg,
            const uint32_t* __restrict__ in_ptr, const uint32_t* __restrict__ in_col,
            const uint32_t* __restrict__ long_rows, uint32_t nlong, uint32_t long_blocks,
            const float* __restrict__ x, float* __restrict__ xnext, float* __restrict__ rankf,
            double* __restrict__ rank, const uint32_t* __restrict__ deg, double* resid)
{
  extern __shared__ float ys[];  // kTileRows accumulators
  __shared__ uint32_t s_big[kTileBigCap];
  __shared__ uint32_t s_nbig;
  __shared__ double s_part[kTileThreads / 32];
  __shared__ float s_lpart[kTileThreads / 32];
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double local = 0.0;
  // the first long_blocks blocks: the long rows, a block each, from the flat CSR
  for (uint32_t k = blockIdx.x; blockIdx.x < long_blocks && k < nlong; k += long_blocks)
  {
    const uint32_t r = long_rows[k];
    if (r >= nreg) continue;  // a sink row (uniform per block)
    float acc = 0.0f;
    for (uint32_t i = in_ptr[r] + tid; i < in_ptr[r + 1]; i += kTileThreads) acc += x[in_col[i]];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) s_lpart[warp] = acc;
    __syncthreads();
    if (tid == 0)
    {
      float t = 0.0f;
      for (uint32_t w = 0; w < kTileThreads / 32; w++) t += s_lpart[w];
      local += prf_finish(r, t, xnext, rankf, rank, deg, 1);
    }
    __syncthreads();
  }
  const uint32_t tblocks = gridDim.x - long_blocks;
  for (uint32_t t = blockIdx.x - long_blocks; blockIdx.x >= long_blocks && t < ntiles; t += tblocks)
  {
    const uint32_t r0 = t * kTileRows, nr = min(kTileRows, nreg - r0);
    for (uint32_t i = tid; i < nr; i += kTileThreads) ys[i] = 0.0f;
    if (tid == 0) s_nbig = 0;
    __syncthreads();
    const uint32_t k0 = tile_col[t], k1 = tile_col[t + 1];
    const uint32_t e0 = tptr[k0], e1 = tptr[k1];
    // hypersparse tile (fewer than kTileDense entries per non-empty column):
    // a thread per entry, its column from the per-entry form, four entries in
    // flight; denser tiles walk their DCSC columns, each message read once
    const bool by_entry = (uint64_t) (e1 - e0) < (uint64_t) kTileDense * (k1 - k0);
    for (uint32_t eb = e0; by_entry && eb < e1; eb += 4 * kTileThreads)
    {
      float xv[4];
      uint32_t rr[4];
#pragma unroll
      for (int u = 0; u < 4; u++)
      {
        const uint32_t e = eb + u * kTileThreads + tid;
        rr[u] = e < e1 ? trow[e] : 0xFFFFFFFFu;
        xv[u] = e < e1 ? x[tecol[e]] : 0.0f;
      }
#pragma unroll
      for (int u = 0; u < 4; u++)
        if (rr[u] != 0xFFFFFFFFu) atomicAdd(&ys[rr[u]], xv[u]);
    }
    // a thread per column, four columns' messages in flight
    for (uint32_t kb = k0; !by_entry && kb < k1; kb += 4 * kTileThreads)
    {
      uint32_t b[4], e[4];
      float xv[4];
#pragma unroll
      for (int u = 0; u < 4; u++)
      {
        const uint32_t k = kb + u * kTileThreads + tid;
        b[u] = e[u] = 0;
        if (k < k1)
        {
          b[u] = tptr[k];
          e[u] = tptr[k + 1];
        }
      }
#pragma unroll
      for (int u = 0; u < 4; u++)
      {
        const uint32_t k = kb + u * kTileThreads + tid;
        xv[u] = (k < k1 && e[u] - b[u] <= kTileBig) ? x[tcol[k]] : 0.0f;
      }
#pragma unroll
      for (int u = 0; u < 4; u++)
      {
        const uint32_t k = kb + u * kTileThreads + tid;
        if (k >= k1) continue;
        if (e[u] - b[u] > kTileBig)
        {
          const uint32_t q = atomicAdd(&s_nbig, 1u);
          if (q < kTileBigCap)
          {
            s_big[q] = k;
            continue;
          }
          xv[u] = x[tcol[k]];  // queue full: this thread adds the column itself
        }
        for (uint32_t j = b[u]; j < e[u]; j++) atomicAdd(&ys[trow[j]], xv[u]);
      }
    }
    __syncthreads();
    const uint32_t nb = min(s_nbig, kTileBigCap);
    for (uint32_t q = warp; q < nb; q += kTileThreads / 32)
    {
      const uint32_t k = s_big[q];
      const float v = x[tcol[k]];
      for (uint32_t j = tptr[k] + lane; j < tptr[k + 1]; j += 32) atomicAdd(&ys[trow[j]], v);
    }
    __syncthreads();
    for (uint32_t i = tid; i < nr; i += kTileThreads)
      if (in_ptr[r0 + i + 1] - in_ptr[r0 + i] <= kLongRow)  // long rows are finished by the flat kernel
        local += prf_finish(r0 + i, ys[i], xnext, rankf, rank, deg, 1);
    __syncthreads();
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  if (lane == 0) s_part[warp] = local;
  __syncthreads();
  if (tid == 0)
  {
    double sum = 0.0;
    for (uint32_t w = 0; w < kTileThreads / 32; w++) sum += s_part[w];
    if (sum != 0.0) atomicAdd(resid, sum);
  }
}

}  // namespace la3g

using namespace la3g;

extern "C" int la3g_pr(la3g_graph* G, uint32_t iters, double* rank_out, uint32_t* degree_out, la3g_stats* st)
{
  if (!G) return set_error(LA3G_EINVAL, "null graph");
  DevGraph& g = G->g;
  if (!g.directed() || (g.flags & (LA3G_REVERSE | LA3G_ACYCLIC | LA3G_BIPARTITE)))
    return set_error(LA3G_EINVAL, "pagerank needs a graph loaded with LA3G_DIRECTED only");
  CallTimer T(G, st);
  PrScratch* ps = nullptr;
  LA3G_TRY(pr_prepare(G, &ps));
  cudaStream_t s = G->stream;
  const uint32_t N = g.nslots;
  T.device_begin();
  k_pr_init<<<grid_for(N, 256), 256, 0, s>>>(N, g.nreg, g.src_base(), g.iso_base(), ps->deg, ps->rank, ps->x[0], ps->x[1]);
  LA3G_LAUNCHED();
  tls_launches++;
  // k_pr_init gives regular and source vertices a message; sinks and
  // isolated vertices never scatter (their x stays 0 and is never read).
  uint32_t it = 0;
  int cur = 0;
  const bool until = iters == 0;
  for (;;)
  {
    if (!until && it >= iters) break;
    if (until) LA3G_CUDA(cudaMemsetAsync(ps->flag, 0, 4, s));
    LA3G_TRY(pr_launch(G, ps, ps->x[cur], ps->x[cur ^ 1], 0, g.nreg, until ? ps->flag : nullptr, true));
    cur ^= 1;
    it++;
    if (until)
    {
      int f = 0;
      LA3G_CUDA(cudaMemcpyAsync(&f, ps->flag, 4, cudaMemcpyDeviceToHost, s));
      LA3G_CUDA(cudaStreamSynchronize(s));
      if (!f) break;
    }
  }
  // sink pass from the final messages (vertex_program_execute.hpp:131-148)
  LA3G_TRY(pr_launch(G, ps, ps->x[cur], ps->x[cur ^ 1], g.nreg, g.nreg + g.nsink, nullptr, false));
  T.device_end();
  if (st)
  {
    st->iterations = it;
    st->teps_edges = (uint64_t) it * g.nent;
    st->edges_examined = (uint64_t) it * g.nent + g.nent;
    st->algo_bytes = (uint64_t) ((4.0 * g.nent + 28.0 * N) * it);
  }
  if (rank_out || degree_out)
  {
    DevBuf tmp;
    LA3G_TRY(tmp.alloc((size_t) N * 8));
    if (rank_out)
    {
      k_scatter_pos<<<grid_for(N, 256), 256, 0, s>>>(N, g.id_of_pos, ps->rank, tmp.as<double>());
      LA3G_LAUNCHED();
      LA3G_CUDA(cudaMemcpyAsync(rank_out, tmp.p, (size_t) N * 8, cudaMemcpyDeviceToHost, s));
      LA3G_CUDA(cudaStreamSynchronize(s));
    }
    if (degree_out)
    {
      k_scatter_pos_u32<<<grid_for(N, 256), 256, 0, s>>>(N, g.id_of_pos, ps->deg, tmp.as<uint32_t>());
      LA3G_LAUNCHED();
      LA3G_CUDA(cudaMemcpyAsync(degree_out, tmp.p, (size_t) N * 4, cudaMemcpyDeviceToHost, s));
      LA3G_CUDA(cudaStreamSynchronize(s));
    }
  }
  return T.finish();
}

static int pr_f32_run(la3g_graph* G, uint32_t iters, double tol, double* rank_out, double* residual_out,
                      la3g_stats* st, bool tiled)
{
  if (!G) return set_error(LA3G_EINVAL, "null graph");
  DevGraph& g = G->g;
  if (!g.directed() || (g.flags & (LA3G_REVERSE | LA3G_ACYCLIC | LA3G_BIPARTITE)))
    return set_error(LA3G_EINVAL, "pagerank needs a graph loaded with LA3G_DIRECTED only");
  if (iters == 0) return set_error(LA3G_EINVAL, "iters must be > 0");
  CallTimer T(G, st);
  PrScratch* ps = nullptr;
  LA3G_TRY(pr_prepare(G, &ps));
  cudaStream_t s = G->stream;
  const uint32_t N = g.nslots;
  if (!ps->rankf)
  {
    LA3G_TRY(galloc(G, &ps->rankf, N));
    LA3G_TRY(galloc(G, &ps->xf[0], N));
    LA3G_TRY(galloc(G, &ps->xf[1], N));
    LA3G_TRY(galloc(G, &ps->resid, 1));
  }
  if (tiled && !ps->tile_col)
  {
    LA3G_TRY(pr_build_tiles(G, ps));
    LA3G_CUDA(cudaFuncSetAttribute(k_prf_tiles, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) (kTileRows * 4)));
    LA3G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ps->tile_blocks, k_prf_tiles, kTileThreads,
                                                            kTileRows * 4));
  }
  T.device_begin();
  k_prf_init<<<grid_for(N, 256), 256, 0, s>>>(N, g.nreg, g.src_base(), g.iso_base(), ps->deg, ps->rankf, ps->rank,
                                              ps->xf[0], ps->xf[1]);
  LA3G_LAUNCHED();
  tls_launches++;
  int cur = 0;
  uint32_t it = 0;
  double res = 0.0;
  const uint32_t long_blocks = ps->nlong ? std::min<uint32_t>(ps->nlong, num_sms() * 2) : 0;
  const unsigned blocks = long_blocks + std::max<uint32_t>(grid_for((uint64_t) g.nreg * 4, 256, num_sms() * 8), 1);
  // algorithmic bytes per iteration (FP32 form of the FP64 count): column
  // index per edge, row offsets, x read, rank read + write, next x write
  const double it_bytes = 4.0 * g.nent + 4.0 * (g.nreg + 1) + 4.0 * N + 8.0 * g.nreg + 8.0 * g.nreg + 4.0 * g.nreg;
  for (; it < iters;)
  {
    LA3G_CUDA(cudaMemsetAsync(ps->resid, 0, 8, s));
    if (tiled)
    {
      // per tile: its non-empty columns (index, offset, message) and 2 B per
      // entry, then the rows' rank read + write and next message write
      ProfileScope p("pr_tiles_f32", s, 12.0 * ps->tile_ncols + 2.0 * ps->tile_nent + 4.0 * (g.nreg + 1) + 8.0 * g.nreg +
                                            8.0 * g.nreg + 4.0 * g.nreg);
      // long rows first (a block each), then the tiles
      const uint32_t lblocks = ps->nlong ? std::min<uint32_t>(ps->nlong, num_sms()) : 0;
      const unsigned tgrid = std::min<unsigned>(std::max<uint32_t>(ps->ntiles, 1), num_sms() * std::max(ps->tile_blocks, 1));
      k_prf_tiles<<<lblocks + tgrid, kTileThreads, kTileRows * 4, s>>>(
          ps->tile_col, ps->tcol, ps->tptr, ps->trow, ps->tecol, ps->ntiles, g.nreg, g.in_ptr, g.in_col, ps->long_rows,
          ps->nlong,
          lblocks, ps->xf[cur], ps->xf[cur ^ 1], ps->rankf, ps->rank, ps->deg, ps->resid);
      LA3G_LAUNCHED();
    }
    else
    {
      ProfileScope p("pr_pull_f32", s, it_bytes);
      k_prf_pull<<<blocks, 256, 0, s>>>(g.in_ptr, g.in_col, ps->xf[cur], ps->xf[cur ^ 1], ps->rankf, ps->rank, ps->deg,
                                        ps->long_rows, ps->nlong, long_blocks, 0, g.nreg, ps->resid, 1);
      LA3G_LAUNCHED();
    }
    cur ^= 1;
    it++;
    if (tol > 0)
    {
      LA3G_CUDA(cudaMemcpyAsync(&res, ps->resid, 8, cudaMemcpyDeviceToHost, s));
      LA3G_CUDA(cudaStreamSynchronize(s));
      if (res < tol) break;
    }
  }
  // the residual of the last iteration (the sink pass below reuses the counter)
  if (tol <= 0) LA3G_CUDA(cudaMemcpyAsync(&res, ps->resid, 8, cudaMemcpyDeviceToHost, s));
  if (g.nsink)
  {
    const unsigned sb = long_blocks + std::max<uint32_t>(grid_for((uint64_t) g.nsink * 4, 256, num_sms() * 8), 1);
    LA3G_CUDA(cudaMemsetAsync(ps->resid, 0, 8, s));
    k_prf_pull<<<sb, 256, 0, s>>>(g.in_ptr, g.in_col, ps->xf[cur], ps->xf[cur ^ 1], ps->rankf, ps->rank, ps->deg,
                                  ps->long_rows, ps->nlong, long_blocks, g.nreg, g.nreg + g.nsink, ps->resid, 0);
    LA3G_LAUNCHED();
  }
  T.device_end();
  if (st)
  {
    st->iterations = it;
    st->teps_edges = (uint64_t) it * g.nent;
    st->edges_examined = (uint64_t) it * g.nent;
    st->algo_bytes = (uint64_t) ((4.0 * g.nent + 20.0 * N) * it);
  }
  if (rank_out)
  {
    DevBuf tmp;
    LA3G_TRY(tmp.alloc((size_t) N * 8));
    k_scatter_pos<<<grid_for(N, 256), 256, 0, s>>>(N, g.id_of_pos, ps->rank, tmp.as<double>());
    LA3G_LAUNCHED();
    LA3G_CUDA(cudaMemcpyAsync(rank_out, tmp.p, (size_t) N * 8, cudaMemcpyDeviceToHost, s));
  }
  LA3G_TRY(T.finish());
  if (residual_out) *residual_out = res;
  return LA3G_OK;
}

extern "C" int la3g_pr_f32(la3g_graph* G, uint32_t iters, double tol, double* rank_out, double* residual_out,
                           la3g_stats* st)
{
  return pr_f32_run(G, iters, tol, rank_out, residual_out, st, false);
}

extern "C" int la3g_pr_f32_tiled(la3g_graph* G, uint32_t iters, double tol, double* rank_out, double* residual_out,
                                 la3g_stats* st)
{
  return pr_f32_run(G, iters, tol, rank_out, residual_out, st, true);
}
