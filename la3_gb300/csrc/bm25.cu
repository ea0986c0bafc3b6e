// BM25: the reference bm25 app (src/apps/information_retrieval/bm25.cpp:8-114,
// bm25.h:11-92, helpers.hpp:76-123) on the device.
//
// The graph is bipartite and undirected (docs 1..D, terms D+1..D+T, identity
// hash), so every vertex with postings is regular and positions ascend with
// ids: docs first, then terms.  A term's row of the pull CSR lists its docs
// ascending, a doc's row lists its terms ascending — the order in which the
// reference's single-iteration SpMV visits them.
//
// prepare (bm25.cpp:16-47):
//   IDF:  y(t) = sum of 1.0f over t's docs (exactly min(df, 2^24) in float);
//         idf = (float) log10((double)((float) D - y) + 0.5) / ((double) y + 0.5));
//   DL 1: len(d) = sum over d's terms, ascending, of (float) tf (float adds);
//   tokens = sum over every vertex of (uint64) its float length (terms
//         contribute their truncated idf; values <= -1 count as 0);
//   avg = (float) tokens / (float) D;
//   DL 2: K(d) = 1.2f * ((1 - 0.75f) + 0.75f * (len / avg)).
// query (bm25.cpp:57-108): the listed term vertices push their idf through
//   a StreamingArray (values in push order, indices ascending — a list that
//   is not ascending pairs them the way the reference does, reproduced by
//   k_bm25_pair); then, term by term in ascending order, every doc of the
//   term gets score += (tf * 2.2f) / (tf + K(d)) * idf in float, starting
//   from 0.0f; the top k of the touched docs are returned in the order
//   score desc, id asc.
// All float operations are explicit _rn intrinsics (no contraction).
#include <algorithm>
#include <cstring>
#include <vector>

#include "la3g_internal.h"
#include "ir.cuh"

namespace la3g {

static constexpr float kK1 = 1.2f;
static constexpr float kB = 0.75f;

struct Bm25Scratch
{
  float* length = nullptr;      // [nslots] DtState.length by position
  float* score = nullptr;       // [nslots]
  uint32_t* stamp = nullptr;    // [nslots] query id that last touched the doc
  uint32_t* touched = nullptr;  // [nslots] touched docs of the current query
  unsigned long long* ctr = nullptr;  // [0] touched count, [1] tokens, [2] postings
  uint32_t* qin = nullptr;      // query vertex ids (device copy)
  uint32_t* qpos = nullptr;     // paired (position, idf bits) after the push emulation
  unsigned long long* cand = nullptr;  // kTopBlocks * kTopKMax candidates
  unsigned long long* best = nullptr;  // kTopKMax
  uint32_t qcap = 0;
  uint32_t term_row0 = 0;       // first regular position of a term (docs come first)
  uint32_t query_id = 0;
  uint64_t tokens = 0;
  float avg = 0.0f;
  bool prepared = false;
};

static void bm25_scratch_free(void* p) { delete (Bm25Scratch*) p; }

// IDF on term rows [row_lo, row_hi).
__global__ void k_bm25_idf(const uint32_t* __restrict__ ptr, uint32_t row_lo, uint32_t row_hi, uint32_t ndocs,
                           float* length)
{
  for (uint32_t r = row_lo + blockIdx.x * blockDim.x + threadIdx.x; r < row_hi; r += gridDim.x * blockDim.x)
  {
    uint32_t df = ptr[r + 1] - ptr[r];
    float y = df > (1u << 24) ? 16777216.0f : (float) df;  // sequential 1.0f adds saturate at 2^24
    float t = __fsub_rn((float) ndocs, y);
    double num = __dadd_rn((double) t, 0.5);
    double den = __dadd_rn((double) y, 0.5);
    length[r] = (float) log10(__ddiv_rn(num, den));
  }
}

// DL on doc rows [row_lo, row_hi): sum of tf in float, ascending term order.
__global__ void k_bm25_dl(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ w, uint32_t row_lo,
                          uint32_t row_hi, float avg, float* length)
{
  for (uint32_t r = row_lo + blockIdx.x * blockDim.x + threadIdx.x; r < row_hi; r += gridDim.x * blockDim.x)
  {
    float y = 0.0f;
    for (uint32_t e = ptr[r]; e < ptr[r + 1]; e++) y = __fadd_rn(y, (float) w[e]);
    y = __fadd_rn(0.0f, y);  // combine(partial, A())
    if (avg == 0.0f) length[r] = y;
    else length[r] = __fmul_rn(kK1, __fadd_rn(__fsub_rn(1.0f, kB), __fmul_rn(kB, __fdiv_rn(y, avg))));
  }
}

__global__ void k_bm25_tokens(const float* __restrict__ length, uint32_t n, unsigned long long* out)
{
  unsigned long long s = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
  {
    float f = length[i];
    s += f > 0.0f ? (unsigned long long) f : 0ull;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, s);
}

// StreamingArray push emulation (streaming_array.h:92-96) for one query:
// push(i, v) stores v at slot count and sets bit i; the j-th smallest set
// index is then read with the value of slot j.  Output: (position, idf)
// pairs ascending by position, count in qpos[0].
__global__ void k_bm25_pair(const uint32_t* __restrict__ q, uint32_t nq, uint32_t nslots, uint32_t nreg,
                            const uint32_t* __restrict__ pos_of_id, const float* __restrict__ length, uint32_t* out)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  uint32_t* idx = out + 1;        // set indices (insertion order)
  uint32_t* val = out + 1 + nq;   // slot values
  uint32_t cnt = 0;
  for (uint32_t i = 0; i < nq; i++)
  {
    uint32_t v = q[i];
    if (v >= nslots) continue;        // not a local vertex (vertex_program.hpp:199)
    uint32_t p = pos_of_id[v];
    if (p >= nreg) continue;          // isolated: init only, no scatter
    val[cnt] = __float_as_uint(length[p]);
    bool seen = false;
    for (uint32_t j = 0; j < cnt; j++) seen |= idx[j] == p;
    if (!seen) idx[cnt++] = p;
  }
  // sort the indices ascending (insertion sort; queries are short)
  for (uint32_t a = 1; a < cnt; a++)
  {
    uint32_t x = idx[a];
    int b = (int) a - 1;
    while (b >= 0 && idx[b] > x) { idx[b + 1] = idx[b]; b--; }
    idx[b + 1] = x;
  }
  out[0] = cnt;
}

// One term: every doc of the term adds its contribution; a doc appears once
// per term, so there are no races inside a launch.
// gather reads the row's mirror state, taken when the TFIDF program was
// first initialised: docs hold K(d); terms (not active then) hold zero.  A
// term row is reached only by a query that names a document vertex.
__global__ void k_bm25_term(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ col,
                            const uint32_t* __restrict__ w, const uint32_t* __restrict__ qpos, uint32_t nq,
                            uint32_t j, const float* __restrict__ length, uint32_t term_row0, float* score,
                            uint32_t* stamp, uint32_t qid, uint32_t* touched, unsigned long long* ctr)
{
  const uint32_t cnt = qpos[0];
  if (j >= cnt) return;
  const uint32_t t = qpos[1 + j];                          // j-th smallest pushed index
  const float idf = __uint_as_float(qpos[1 + nq + j]);     // value of slot j
  const uint32_t b = ptr[t], e = ptr[t + 1];
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ctr[2], (unsigned long long) (e - b));  // postings walked
  const float k1p1 = __fadd_rn(kK1, 1.0f);
  for (uint32_t i = b + blockIdx.x * blockDim.x + threadIdx.x; i < e; i += gridDim.x * blockDim.x)
  {
    const uint32_t d = col[i];
    const float wf = (float) w[i];
    const float kd = d < term_row0 ? length[d] : 0.0f;
    const float c = __fmul_rn(__fdiv_rn(__fmul_rn(wf, k1p1), __fadd_rn(wf, kd)), idf);
    if (stamp[d] != qid)
    {
      stamp[d] = qid;
      score[d] = __fadd_rn(0.0f, c);
      unsigned long long slot = atomicAdd(&ctr[0], 1ull);
      touched[slot] = d;
    }
    else
    {
      score[d] = __fadd_rn(score[d], c);
    }
  }
}

__device__ __forceinline__ unsigned long long bm25_key(float s, uint32_t id)
{
  // order-preserving map of the score (with -0 == +0), then smaller id first
  uint32_t u = __float_as_uint(s);
  if ((u & 0x7FFFFFFFu) == 0) u = 0;
  u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
  return ((unsigned long long) u << 32) | (0xFFFFFFFFu - id);
}

__global__ void __launch_bounds__(kTopThreads)
k_bm25_top_partial(const uint32_t* __restrict__ touched, const unsigned long long* __restrict__ ctr,
                   const float* __restrict__ score, const uint32_t* __restrict__ id_of_pos, int k,
                   unsigned long long* cand)
{
  unsigned long long mine[kTopKMax];
  for (int i = 0; i < k; i++) mine[i] = 0;
  const uint64_t n = ctr[0];
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
  {
    uint32_t d = touched[i];
    keep_best(mine, k, bm25_key(score[d], id_of_pos[d]));
  }
  block_topk(mine, k, cand + (size_t) blockIdx.x * k);
}

__global__ void __launch_bounds__(kTopThreads)
k_bm25_top_final(const unsigned long long* __restrict__ cand, int ncand, int k, unsigned long long* best)
{
  unsigned long long mine[kTopKMax];
  for (int i = 0; i < k; i++) mine[i] = 0;
  for (int i = threadIdx.x; i < ncand; i += blockDim.x) keep_best(mine, k, cand[i]);
  block_topk(mine, k, best);
}

__global__ void k_bm25_dump(const uint32_t* __restrict__ touched, const unsigned long long* __restrict__ ctr,
                            const float* __restrict__ score, const uint32_t* __restrict__ id_of_pos, float* all,
                            uint8_t* act)
{
  const uint64_t n = ctr[0];
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
  {
    uint32_t d = touched[i];
    uint32_t id = id_of_pos[d];
    if (all) all[id] = score[d];
    if (act) act[id] = 1;
  }
}

__global__ void k_f32_by_id(uint32_t N, const uint32_t* __restrict__ id_of_pos, const float* __restrict__ v, float* out)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) out[id_of_pos[p]] = v[p];
}

static int bm25_scratch(la3g_graph* G, Bm25Scratch** out)
{
  Bm25Scratch* b = (Bm25Scratch*) G->slot[kSlotBm25];
  if (b) { *out = b; return LA3G_OK; }
  b = new (std::nothrow) Bm25Scratch();
  if (!b) return set_error(LA3G_ENOMEM, "out of host memory");
  G->slot[kSlotBm25] = b;
  G->slot_free[kSlotBm25] = bm25_scratch_free;
  const uint32_t N = G->g.nslots;
  LA3G_TRY(galloc(G, &b->length, N));
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

// First term row: positions ascend with ids, docs (ids <= D) come first.
int bipartite_first_term_row(la3g_graph* G, uint32_t* out)
{
  DevGraph& g = G->g;
  // binary search over id_of_pos[0, nreg) for the first id > nleft
  uint32_t lo = 0, hi = g.nreg;
  while (lo < hi)
  {
    uint32_t mid = (lo + hi) / 2, id = 0;
    LA3G_CUDA(cudaMemcpy(&id, g.id_of_pos + mid, 4, cudaMemcpyDeviceToHost));
    if (id <= g.nleft) lo = mid + 1;
    else hi = mid;
  }
  *out = lo;
  return LA3G_OK;
}

}  // namespace la3g

using namespace la3g;

extern "C" int la3g_bm25_prepare(la3g_graph* G, uint64_t* ntokens_out, float* avg_out, float* length_out)
{
  if (!G) return set_error(LA3G_EINVAL, "null graph");
  DevGraph& g = G->g;
  if (!(g.flags & LA3G_BIPARTITE) || g.directed() || !g.weighted())
    return set_error(LA3G_EINVAL, "bm25 needs a graph loaded with LA3G_BIPARTITE | LA3G_WEIGHTED (undirected)");
  Bm25Scratch* b = nullptr;
  LA3G_TRY(bm25_scratch(G, &b));
  cudaStream_t s = G->stream;
  const uint32_t N = g.nslots;
  LA3G_CUDA(cudaStreamSynchronize(s));
  uint32_t tb = 0;
  LA3G_TRY(bipartite_first_term_row(G, &tb));
  b->term_row0 = tb;
  LA3G_CUDA(cudaMemsetAsync(b->length, 0, (size_t) N * 4, s));
  LA3G_CUDA(cudaMemsetAsync(b->ctr, 0, 4 * 8, s));
  {
    ProfileScope p("bm25_idf", s, 4.0 * (g.nreg - tb + 1) + 4.0 * (g.nreg - tb));
    k_bm25_idf<<<grid_for(g.nreg - tb, 256), 256, 0, s>>>(g.in_ptr, tb, g.nreg, g.nleft, b->length);
    LA3G_LAUNCHED();
  }
  {
    ProfileScope p("bm25_dl", s, 8.0 * g.nent / 2);
    k_bm25_dl<<<grid_for(tb, 256), 256, 0, s>>>(g.in_ptr, g.in_w, 0, tb, 0.0f, b->length);
    LA3G_LAUNCHED();
  }
  k_bm25_tokens<<<grid_for(N, 256), 256, 0, s>>>(b->length, N, b->ctr + 1);
  LA3G_LAUNCHED();
  unsigned long long tok = 0;
  LA3G_CUDA(cudaMemcpyAsync(&tok, b->ctr + 1, 8, cudaMemcpyDeviceToHost, s));
  LA3G_CUDA(cudaStreamSynchronize(s));
  // avg = collection_ntokens / (float) ndocs (bm25.cpp:38): uint64 -> float, float divide
  const float avg = (float) tok / (float) g.nleft;
  {
    ProfileScope p("bm25_dl", s, 8.0 * g.nent / 2);
    k_bm25_dl<<<grid_for(tb, 256), 256, 0, s>>>(g.in_ptr, g.in_w, 0, tb, avg, b->length);
    LA3G_LAUNCHED();
  }
  b->tokens = tok;
  b->avg = avg;
  b->prepared = true;
  if (ntokens_out) *ntokens_out = tok;
  if (avg_out) *avg_out = avg;
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

extern "C" int la3g_bm25_query(la3g_graph* G, const uint32_t* term_vids, uint32_t nterms, uint32_t k,
                               uint32_t* ids_out, float* scores_out, uint32_t* nout, float* all_scores_out,
                               uint8_t* active_out, la3g_stats* st)
{
  if (!G) return set_error(LA3G_EINVAL, "null graph");
  if (nterms && !term_vids) return set_error(LA3G_EINVAL, "term_vids is null");
  if (k > kTopKMax) return set_error(LA3G_EINVAL, "k = %u exceeds the maximum of %d", k, kTopKMax);
  Bm25Scratch* b = (Bm25Scratch*) G->slot[kSlotBm25];
  if (!b || !b->prepared) return set_error(LA3G_EINVAL, "call la3g_bm25_prepare first");
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
  // the distinct regular terms, ascending; at most nterms launches
  for (uint32_t j = 0; j < nterms; j++)
  {
    ProfileScope p("bm25_term", s, 0.0);
    k_bm25_term<<<num_sms() * 4, 256, 0, s>>>(g.in_ptr, g.in_col, g.in_w, b->qpos, nterms, j, b->length, b->term_row0,
                                        b->score, b->stamp, b->query_id, b->touched, b->ctr);
    LA3G_LAUNCHED();
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
  // algorithmic bytes: doc id + tf per posting walked, K(d) read and score
  // written per touched doc, the top-k pass over the touched docs
  const double bytes = 8.0 * (double) postings + 12.0 * (double) ntouched;
  profile_add_bytes("bm25_term", bytes);
  if (st)
  {
    st->iterations = 1;
    st->teps_edges = ntouched;
    st->edges_examined = postings;
    st->algo_bytes = (uint64_t) bytes;
  }
  return LA3G_OK;
}
