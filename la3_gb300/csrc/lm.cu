// LM: the reference lm app (src/apps/information_retrieval/lm.cpp:8-144,
// lm.h:16-75) on the device: query likelihood with Dirichlet smoothing
// (mu = 2000) over the same bipartite corpus as BM25.
//
// prepare (lm.cpp:16-46):
//   DL:  length(d) = sum over d's terms, ascending, of (float) tf (float adds);
//   tokens = sum over every vertex of (uint64) its float length (terms hold 0);
//   TL:  length(t) = (sum over t's docs, ascending, of (float) tf) / (float)
//        tokens — the sums of frequent terms pass 2^24, where float addition
//        rounds, so each term row is summed in the reference's order (a warp
//        loads 32 entries at a time, lanes' values are added one after
//        another);
//   the per-vertex factor log10f(mu / (length + mu)) of the score
//        (lm.h:74): that log10 takes a float, so the reference calls the float
//        overload of the platform's libm, which is not correctly rounded; the
//        factor depends only on the vertex's length and is evaluated once per
//        vertex here, with the same libm function, and kept on the device.
// query (lm.cpp:57-87): the listed term vertices push their length through a
//   StreamingArray (k_bm25_pair); term by term, ascending, every doc of the
//   term adds (float) log10(1.0 + (double) (tf / (mu * length(t)))) — a
//   double log10, rounded to float — to its score, from 0.0f; the touched
//   vertices then take score = y + (float) nterms * factor.  The top k of the
//   active vertices are returned (score desc, id asc).  The TFIDF program
//   reads no state in gather, so the reference takes no mirrors at its first
//   initialize and the activity the TL pass left (every term row) is still
//   set in the first query after prepare: those terms join that query's pool
//   with score 0, as in the reference.
// All float operations are explicit _rn intrinsics (no contraction).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "la3g_internal.h"
#include "ir.cuh"

namespace la3g {

static constexpr float kMu = 2000.0f;

struct LmScratch
{
  float* length = nullptr;      // [nslots] DtState.length by position
  float* factor = nullptr;      // [nslots] log10f(mu / (length + mu)) by position
  float* score = nullptr;       // [nslots]
  uint32_t* stamp = nullptr;    // [nslots] query id that last touched the vertex
  uint32_t* touched = nullptr;  // [nslots] active vertices of the current query
  unsigned long long* ctr = nullptr;  // [0] touched count, [1] tokens, [2] postings
  uint32_t* qin = nullptr;
  uint32_t* qpos = nullptr;
  unsigned long long* cand = nullptr;
  unsigned long long* best = nullptr;
  uint32_t qcap = 0;
  uint32_t term_row0 = 0;
  uint32_t query_id = 0;
  uint64_t tokens = 0;
  bool prepared = false;
  bool leftover = false;        // the TL pass's activity is still set (first query)
};

static void lm_scratch_free(void* p) { delete (LmScratch*) p; }

// TL on term rows [row_lo, row_hi): a warp per row, lanes load 32 entries at
// a time and the sum runs through them in entry (ascending doc) order.
__global__ void k_lm_tl(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ w, uint32_t row_lo,
                        uint32_t row_hi, float ntok, float* length)
{
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t r = row_lo + warp; r < row_hi; r += nwarps)
  {
    const uint32_t b = ptr[r], e = ptr[r + 1];
    float y = 0.0f;
    for (uint32_t c0 = b; c0 < e; c0 += 32)
    {
      const uint32_t n = min(32u, e - c0);
      const float v = (uint32_t) lane < n ? (float) w[c0 + lane] : 0.0f;
      for (uint32_t j = 0; j < n; j++) y = __fadd_rn(y, __shfl_sync(0xffffffffu, v, j));
    }
    y = __fadd_rn(0.0f, y);  // combine(partial, A())
    if (lane == 0) length[r] = __fdiv_rn(y, ntok);
  }
}

// One term: every doc of the term adds log10(1 + tf / (mu * msg)); a doc
// appears once per term, so there are no races inside a launch.
__global__ void k_lm_term(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col,
                          const uint32_t* __restrict__ w, const uint32_t* __restrict__ qpos, uint32_t nq, uint32_t j,
                          float* score, uint32_t* stamp, uint32_t qid, uint32_t* touched, unsigned long long* ctr)
{
  const uint32_t cnt = qpos[0];
  if (j >= cnt) return;
  const uint32_t t = qpos[1 + j];
  const float msg = __uint_as_float(qpos[1 + nq + j]);
  const uint32_t b = ptr[t], e = ptr[t + 1];
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ctr[2], (unsigned long long) (e - b));
  const float den = __fmul_rn(kMu, msg);
  for (uint32_t i = b + blockIdx.x * blockDim.x + threadIdx.x; i < e; i += gridDim.x * blockDim.x)
  {
    const uint32_t d = col[i];
    const float q = __fdiv_rn((float) w[i], den);
    const float c = (float) log10(__dadd_rn(1.0, (double) q));
    if (stamp[d] != qid)
    {
      stamp[d] = qid;
      score[d] = __fadd_rn(0.0f, c);
      touched[atomicAdd(&ctr[0], 1ull)] = d;
    }
    else
    {
      score[d] = __fadd_rn(score[d], c);
    }
  }
}

// apply on the touched vertices: score = y + (float) nterms * factor.
__global__ void k_lm_apply(const uint32_t* __restrict__ touched, const unsigned long long* __restrict__ ctr,
                           const float* __restrict__ factor, float nterms, float* score)
{
  const uint64_t n = ctr[0];
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
  {
    const uint32_t d = touched[i];
    score[d] = __fadd_rn(score[d], __fmul_rn(nterms, factor[d]));
  }
}

// The first query after prepare: the term rows the TL pass left active and
// this query did not reach join its pool with score 0.
__global__ void k_lm_leftover(uint32_t row_lo, uint32_t row_hi, uint32_t* stamp, uint32_t qid, float* score,
                              uint32_t* touched, unsigned long long* ctr)
{
  for (uint32_t r = row_lo + blockIdx.x * blockDim.x + threadIdx.x; r < row_hi; r += gridDim.x * blockDim.x)
    if (stamp[r] != qid)
    {
      stamp[r] = qid;
      score[r] = 0.0f;
      touched[atomicAdd(&ctr[0], 1ull)] = r;
    }
}

static int lm_scratch(la3g_graph* G, LmScratch** out)
{
  LmScratch* b = (LmScratch*) G->slot[kSlotLm];
  if (b) { *out = b; return LA3G_OK; }
  b = new (std::nothrow) LmScratch();
  if (!b) return set_error(LA3G_ENOMEM, "out of host memory");
  G->slot[kSlotLm] = b;
  G->slot_free[kSlotLm] = lm_scratch_free;
  const uint32_t N = G->g.nslots;
  LA3G_TRY(galloc(G, &b->length, N));
  LA3G_TRY(galloc(G, &b->factor, N));
  LA3G_TRY(galloc(G, &b->score, N));
  LA3G_TRY(galloc(G, &b->stamp, N));
  LA3G_TRY(galloc(G, &b->touched, N));
  LA3G_TRY(galloc(G, &b->ctr, 4));
  LA3G_TRY(galloc(G, &b->cand, (size_t) kTopBlocks * kTopKMax));
  LA3G_TRY(galloc(G, &b->best, kTopKMax));
  LA3G_CUDA(cudaMemsetAsync(b->stamp, 0, (size_t) N * 4, G->stream));
  *out = b;
  return LA3G_OK;
}

}  // namespace la3g

using namespace la3g;

extern "C" int la3g_lm_prepare(la3g_graph* G, uint64_t* ntokens_out, float* length_out)
{
  if (!G) return set_error(LA3G_EINVAL, "null graph");
  DevGraph& g = G->g;
  if (!(g.flags & LA3G_BIPARTITE) || g.directed() || !g.weighted())
    return set_error(LA3G_EINVAL, "lm needs a graph loaded with LA3G_BIPARTITE | LA3G_WEIGHTED (undirected)");
  LmScratch* b = nullptr;
  LA3G_TRY(lm_scratch(G, &b));
  cudaStream_t s = G->stream;
  const uint32_t N = g.nslots;
  LA3G_CUDA(cudaStreamSynchronize(s));
  uint32_t tb = 0;
  LA3G_TRY(bipartite_first_term_row(G, &tb));
  b->term_row0 = tb;
  LA3G_CUDA(cudaMemsetAsync(b->length, 0, (size_t) N * 4, s));
  LA3G_CUDA(cudaMemsetAsync(b->ctr, 0, 4 * 8, s));
  {
    ProfileScope p("lm_dl", s, 8.0 * g.nent / 2);
    k_bm25_dl<<<grid_for(tb, 256), 256, 0, s>>>(g.in_ptr, g.in_w, 0, tb, 0.0f, b->length);
    LA3G_LAUNCHED();
  }
  k_bm25_tokens<<<grid_for(N, 256), 256, 0, s>>>(b->length, N, b->ctr + 1);
  LA3G_LAUNCHED();
  unsigned long long tok = 0;
  LA3G_CUDA(cudaMemcpyAsync(&tok, b->ctr + 1, 8, cudaMemcpyDeviceToHost, s));
  LA3G_CUDA(cudaStreamSynchronize(s));
  if (g.nreg > tb)
  {
    ProfileScope p("lm_tl", s, 8.0 * g.nent / 2);
    // length = y / collection_ntokens (lm.h:55): the uint64 count as float
    k_lm_tl<<<grid_for((uint64_t) (g.nreg - tb) * 32, 256), 256, 0, s>>>(g.in_ptr, g.in_w, tb, g.nreg, (float) tok,
                                                                         b->length);
    LA3G_LAUNCHED();
  }
  // the score's per-vertex factor with the platform's log10f (see the top)
  std::vector<float> len(g.nreg), fac(g.nreg);
  if (g.nreg)
  {
    LA3G_CUDA(cudaMemcpyAsync(len.data(), b->length, (size_t) g.nreg * 4, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    for (uint32_t i = 0; i < g.nreg; i++) fac[i] = log10f(kMu / (len[i] + kMu));
    LA3G_CUDA(cudaMemcpyAsync(b->factor, fac.data(), (size_t) g.nreg * 4, cudaMemcpyHostToDevice, s));
  }
  b->tokens = tok;
  b->prepared = true;
  b->leftover = true;
  if (ntokens_out) *ntokens_out = tok;
  if (length_out)
  {
    DevBuf tmp;
    LA3G_TRY(tmp.alloc((size_t) N * 4));
    k_f32_by_id<<<grid_for(N, 256), 256, 0, s>>>(N, g.id_of_pos, b->length, tmp.as<float>());
    LA3G_LAUNCHED();
    LA3G_CUDA(cudaMemcpyAsync(length_out, tmp.p, (size_t) N * 4, cudaMemcpyDeviceToHost, s));
  }
  LA3G_CUDA(cudaStreamSynchronize(s));
  return LA3G_OK;
}

extern "C" int la3g_lm_query(la3g_graph* G, const uint32_t* term_vids, uint32_t nterms, uint32_t k, uint32_t* ids_out,
                             float* scores_out, uint32_t* nout, float* all_scores_out, uint8_t* active_out,
                             la3g_stats* st)
{
  if (!G) return set_error(LA3G_EINVAL, "null graph");
  if (nterms && !term_vids) return set_error(LA3G_EINVAL, "term_vids is null");
  if (k > kTopKMax) return set_error(LA3G_EINVAL, "k = %u exceeds the maximum of %d", k, kTopKMax);
  LmScratch* b = (LmScratch*) G->slot[kSlotLm];
  if (!b || !b->prepared) return set_error(LA3G_EINVAL, "call la3g_lm_prepare first");
  DevGraph& g = G->g;
  cudaStream_t s = G->stream;
  const uint32_t N = g.nslots;
  CallTimer T(G, st);
  if (nterms > b->qcap || !b->qpos)
  {
    uint32_t cap = std::max<uint32_t>(64, nterms);
    LA3G_TRY(galloc(G, &b->qin, cap));
    LA3G_TRY(galloc(G, &b->qpos, 1 + 2 * (size_t) cap));
    b->qcap = cap;
  }
  if (++b->query_id == 0)
  {
    LA3G_CUDA(cudaMemsetAsync(b->stamp, 0, (size_t) N * 4, s));
    b->query_id = 1;
  }
  T.device_begin();
  if (nterms) LA3G_CUDA(cudaMemcpyAsync(b->qin, term_vids, (size_t) nterms * 4, cudaMemcpyHostToDevice, s));
  LA3G_CUDA(cudaMemsetAsync(b->ctr, 0, 8, s));
  LA3G_CUDA(cudaMemsetAsync(b->ctr + 2, 0, 8, s));
  LA3G_CUDA(cudaMemsetAsync(b->qpos, 0, 4, s));
  if (nterms)
  {
    k_bm25_pair<<<1, 1, 0, s>>>(b->qin, nterms, N, g.nreg, g.pos_of_id, b->length, b->qpos);
    LA3G_LAUNCHED();
    tls_launches++;
  }
  for (uint32_t j = 0; j < nterms; j++)
  {
    ProfileScope p("lm_term", s, 0.0);
    k_lm_term<<<num_sms() * 4, 256, 0, s>>>(g.in_ptr, g.in_col, g.in_w, b->qpos, nterms, j, b->score, b->stamp,
                                      b->query_id, b->touched, b->ctr);
    LA3G_LAUNCHED();
  }
  // query_nterms = queries[q].size() (lm.cpp:66), as float in the apply
  k_lm_apply<<<num_sms() * 4, 256, 0, s>>>(b->touched, b->ctr, b->factor, (float) nterms, b->score);
  LA3G_LAUNCHED();
  tls_launches++;
  if (b->leftover)
  {
    if (g.nreg > b->term_row0)
    {
      k_lm_leftover<<<grid_for(g.nreg - b->term_row0, 256), 256, 0, s>>>(b->term_row0, g.nreg, b->stamp, b->query_id,
                                                                         b->score, b->touched, b->ctr);
      LA3G_LAUNCHED();
      tls_launches++;
    }
    b->leftover = false;  // tfidf.reset_activity() after the query (lm.cpp:86)
  }
  const int kk = (int) k;
  if (kk > 0)
  {
    k_bm25_top_partial<<<kTopBlocks, kTopThreads, 0, s>>>(b->touched, b->ctr, b->score, g.id_of_pos, kk, b->cand);
    LA3G_LAUNCHED();
    k_bm25_top_final<<<1, kTopThreads, 0, s>>>(b->cand, kTopBlocks * kk, kk, b->best);
    LA3G_LAUNCHED();
    tls_launches += 2;
  }
  T.device_end();
  unsigned long long ntouched = 0, postings = 0;
  LA3G_CUDA(cudaMemcpyAsync(&ntouched, b->ctr, 8, cudaMemcpyDeviceToHost, s));
  LA3G_CUDA(cudaMemcpyAsync(&postings, b->ctr + 2, 8, cudaMemcpyDeviceToHost, s));
  unsigned long long best[kTopKMax];
  if (kk > 0) LA3G_CUDA(cudaMemcpyAsync(best, b->best, (size_t) kk * 8, cudaMemcpyDeviceToHost, s));
  if (all_scores_out || active_out)
  {
    DevBuf a, c;
    if (all_scores_out) { LA3G_TRY(a.alloc((size_t) N * 4)); LA3G_CUDA(cudaMemsetAsync(a.p, 0, (size_t) N * 4, s)); }
    if (active_out) { LA3G_TRY(c.alloc(N)); LA3G_CUDA(cudaMemsetAsync(c.p, 0, N, s)); }
    k_bm25_dump<<<num_sms() * 4, 256, 0, s>>>(b->touched, b->ctr, b->score, g.id_of_pos, a.as<float>(), c.as<uint8_t>());
    LA3G_LAUNCHED();
    if (all_scores_out) LA3G_CUDA(cudaMemcpyAsync(all_scores_out, a.p, (size_t) N * 4, cudaMemcpyDeviceToHost, s));
    if (active_out) LA3G_CUDA(cudaMemcpyAsync(active_out, c.p, N, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
  }
  LA3G_TRY(T.finish());
  uint32_t n = (uint32_t) std::min<unsigned long long>(ntouched, (unsigned long long) k);
  for (uint32_t i = 0; i < n; i++)
  {
    uint32_t u = (uint32_t) (best[i] >> 32);
    u = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
    float sc;
    std::memcpy(&sc, &u, 4);
    if (ids_out) ids_out[i] = 0xFFFFFFFFu - (uint32_t) best[i];
    if (scores_out) scores_out[i] = sc;
  }
  if (nout) *nout = n;
  // algorithmic bytes: doc id + tf per posting walked, factor read and score
  // written per touched vertex, the top-k pass over them
  const double bytes = 8.0 * (double) postings + 12.0 * (double) ntouched;
  profile_add_bytes("lm_term", bytes);
  if (st)
  {
    st->iterations = 1;
    st->teps_edges = ntouched;
    st->edges_examined = postings;
    st->algo_bytes = (uint64_t) bytes;
  }
  return LA3G_OK;
}
