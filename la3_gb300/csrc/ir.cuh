// Top-k over 64-bit keys (value in the high half, ~id in the low half, so
// that ties go to the smaller id), used by BM25, LM and the degree app, and
// the kernels the two information-retrieval apps share, BM25 (bm25.cu) and
// LM (lm.cu), over a bipartite corpus: docs 1..D then terms D+1..D+T,
// identity hash, so positions ascend with ids and a term's pull row lists
// its docs ascending.  The kernels are defined in bm25.cu.
#ifndef LA3G_IR_CUH
#define LA3G_IR_CUH

#include <cstdint>

namespace la3g {

constexpr int kTopKMax = 64;       // largest k of a top-k query
constexpr int kTopThreads = 128;   // threads of the top-k blocks
constexpr int kTopBlocks = 2 * 152;  // partial top-k blocks (two per SM of a GB300)

// Block-level top-k of a key stream: each thread keeps its k best keys, the
// block then extracts the k largest by repeated block-wide max.
static __device__ void block_topk(unsigned long long* mine, int k, unsigned long long* out)
{
  __shared__ unsigned long long s_best[kTopThreads];
  __shared__ int s_who[kTopThreads];
  for (int r = 0; r < k; r++)
  {
    unsigned long long m = 0;
    int mi = -1;
    for (int i = 0; i < k; i++)
      if (mine[i] > m) { m = mine[i]; mi = i; }
    s_best[threadIdx.x] = m;
    s_who[threadIdx.x] = threadIdx.x;
    __syncthreads();
    for (int o = kTopThreads / 2; o > 0; o >>= 1)
    {
      if ((int) threadIdx.x < o && s_best[threadIdx.x + o] > s_best[threadIdx.x])
      {
        s_best[threadIdx.x] = s_best[threadIdx.x + o];
        s_who[threadIdx.x] = s_who[threadIdx.x + o];
      }
      __syncthreads();
    }
    unsigned long long top = s_best[0];
    int who = s_who[0];
    __syncthreads();
    if (threadIdx.x == 0) out[r] = top;
    if ((int) threadIdx.x == who && mi >= 0 && top != 0) mine[mi] = 0;
    __syncthreads();
  }
}

static __device__ __forceinline__ void keep_best(unsigned long long* mine, int k, unsigned long long key)
{
  int mi = 0;
  unsigned long long mv = mine[0];
  for (int i = 1; i < k; i++)
    if (mine[i] < mv) { mv = mine[i]; mi = i; }
  if (key > mv) mine[mi] = key;
}

// Sum of (float) tf over rows [row_lo, row_hi), ascending entry order, then
// length = sum (avg == 0) or BM25's K(d) (avg > 0).
__global__ void k_bm25_dl(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ w, uint32_t row_lo,
                          uint32_t row_hi, float avg, float* length);
// Sum over positions of (uint64) length (values <= -1 count as 0).
__global__ void k_bm25_tokens(const float* __restrict__ length, uint32_t n, unsigned long long* out);
// StreamingArray push emulation of a query's term list: (position, value)
// pairs ascending by position in out[1..], count in out[0].
__global__ void k_bm25_pair(const uint32_t* __restrict__ q, uint32_t nq, uint32_t nslots, uint32_t nreg,
                            const uint32_t* __restrict__ pos_of_id, const float* __restrict__ length, uint32_t* out);
// Top k (score desc, id asc) of the touched rows: per-block candidates, then
// one block over them.
__global__ void __launch_bounds__(kTopThreads) k_bm25_top_partial(const uint32_t* __restrict__ touched, const unsigned long long* __restrict__ ctr,
                                                               const float* __restrict__ score,
                                                               const uint32_t* __restrict__ id_of_pos, int k,
                                                               unsigned long long* cand);
__global__ void __launch_bounds__(kTopThreads) k_bm25_top_final(const unsigned long long* __restrict__ cand, int ncand, int k,
                                 unsigned long long* best);
// Scores and activity of the touched rows, by id.
__global__ void k_bm25_dump(const uint32_t* __restrict__ touched, const unsigned long long* __restrict__ ctr,
                            const float* __restrict__ score, const uint32_t* __restrict__ id_of_pos, float* all,
                            uint8_t* act);
__global__ void k_f32_by_id(uint32_t N, const uint32_t* __restrict__ id_of_pos, const float* __restrict__ v, float* out);

}  // namespace la3g

#endif
