// Seeded synthetic inputs for the LA3 path: R-MAT and Erdos-Renyi edge lists
// (LA3 pairs or u32-weighted triples, 1-based ids) and a bipartite doc-term
// corpus for BM25.  Host code; deterministic for a given seed on any machine
// and any thread count (every draw is a pure function of (seed, index)).
//
// The on-disk record layout is the reference's Triple<W>
// (utils/common.h:14-35, 65-83): {u32 src, u32 dst[, u32 w]} little-endian,
// with the optional 16-byte header {u32 n-1, u32 m-1, u64 nnz} that
// tools/mtx2bin.cpp:77-84 writes and matrix/graph.hpp:89-117 reads.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "la3g.h"
#include "la3g_internal.h"

namespace la3g {

static inline uint64_t mix64(uint64_t x)
{
  // splitmix64 finaliser
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

static inline uint64_t draw(uint64_t key, uint64_t i, uint64_t k)
{
  return mix64(key ^ mix64(i * 0xD6E8FEB86659FD93ull + k));
}

unsigned host_threads()
{
  unsigned t = std::thread::hardware_concurrency();
  if (t == 0) t = 1;
  if (t > 64) t = 64;
  const char* e = std::getenv("LA3G_THREADS");
  if (e && std::atoi(e) > 0) t = (unsigned) std::atoi(e);
  return t;
}

template <class F>
void parallel_for(uint64_t n, F f)
{
  unsigned T = host_threads();
  if (n < 65536 || T == 1) { f(0, n, 0u); return; }
  std::vector<std::thread> th;
  for (unsigned t = 0; t < T; t++)
  {
    uint64_t lo = n * t / T, hi = n * (t + 1) / T;
    th.emplace_back([=]() { f(lo, hi, t); });
  }
  for (auto& x : th) x.join();
}

// Random permutation of [0, n) by Fisher-Yates on a seeded stream.
static std::vector<uint32_t> permutation(uint32_t n, uint64_t seed)
{
  std::vector<uint32_t> p(n);
  for (uint32_t i = 0; i < n; i++) p[i] = i;
  uint64_t key = mix64(seed ^ 0x7065726D75746531ull);
  for (uint32_t i = n; i > 1; i--)
  {
    uint64_t j = draw(key, i, 0) % i;
    std::swap(p[i - 1], p[j]);
  }
  return p;
}

struct EdgeKey
{
  uint64_t key;  // src << 32 | dst (1-based ids)
  uint64_t idx;  // generation index (first occurrence wins for the weight)
  bool operator<(const EdgeKey& o) const { return key < o.key || (key == o.key && idx < o.idx); }
};

// Sorts by (src, dst, idx), drops duplicates (keeping the first generated)
// and fills the output arrays in (src, dst) order.  Partition by the top
// bits of the key, then sort the partitions on all threads.
static int finish_edges(std::vector<EdgeKey>& e, uint32_t n, bool weighted, uint64_t wseed,
                        la3g_edges* out)
{
  const unsigned T = host_threads();
  const uint32_t NB = 1024;
  int shift = 0;
  while (shift < 32 && ((uint64_t) n >> shift) >= NB) shift++;
  auto bucket = [&](uint64_t key) -> uint32_t {
    uint64_t b = (key >> 32) >> shift;
    return (uint32_t) (b < NB ? b : NB - 1);
  };
  std::vector<uint64_t> hist((size_t) T * NB, 0);
  uint64_t m = e.size();
  parallel_for(m, [&](uint64_t lo, uint64_t hi, unsigned t) {
    for (uint64_t i = lo; i < hi; i++) hist[(size_t) t * NB + bucket(e[i].key)]++;
  });
  std::vector<uint64_t> start(NB + 1, 0);
  {
    uint64_t s = 0;
    for (uint32_t b = 0; b < NB; b++)
    {
      start[b] = s;
      for (unsigned t = 0; t < T; t++)
      {
        uint64_t c = hist[(size_t) t * NB + b];
        hist[(size_t) t * NB + b] = s;
        s += c;
      }
    }
    start[NB] = s;
  }
  std::vector<EdgeKey> tmp;
  try { tmp.resize(m); } catch (const std::bad_alloc&) { return LA3G_ENOMEM; }
  parallel_for(m, [&](uint64_t lo, uint64_t hi, unsigned t) {
    for (uint64_t i = lo; i < hi; i++) tmp[hist[(size_t) t * NB + bucket(e[i].key)]++] = e[i];
  });
  // The same thread split is used by both passes so the scatter is stable.
  std::atomic<uint32_t> next(0);
  std::vector<std::thread> th;
  for (unsigned t = 0; t < T; t++)
    th.emplace_back([&]() {
      for (uint32_t b; (b = next.fetch_add(1)) < NB;) std::sort(tmp.begin() + start[b], tmp.begin() + start[b + 1]);
    });
  for (auto& x : th) x.join();
  uint64_t u = 0;
  for (uint64_t i = 0; i < m; i++)
    if (i == 0 || tmp[i].key != tmp[i - 1].key) tmp[u++] = tmp[i];
  std::vector<EdgeKey>().swap(e);
  out->n = n;
  out->m = u;
  out->weighted = weighted ? 1 : 0;
  out->src = (uint32_t*) std::malloc((u ? u : 1) * sizeof(uint32_t));
  out->dst = (uint32_t*) std::malloc((u ? u : 1) * sizeof(uint32_t));
  out->w = weighted ? (uint32_t*) std::malloc((u ? u : 1) * sizeof(uint32_t)) : nullptr;
  if (!out->src || !out->dst || (weighted && !out->w)) { la3g_edges_free(out); return LA3G_ENOMEM; }
  const uint64_t wkey = mix64(wseed ^ 0x7765696768747321ull);
  parallel_for(u, [&](uint64_t lo, uint64_t hi, unsigned) {
    for (uint64_t i = lo; i < hi; i++)
    {
      out->src[i] = (uint32_t) (tmp[i].key >> 32);
      out->dst[i] = (uint32_t) tmp[i].key;
      // weights uniform in [1, 128] from their own stream
      if (weighted) out->w[i] = 1u + (uint32_t) (draw(wkey, tmp[i].idx, 0) & 127u);
    }
  });
  return LA3G_OK;
}

}  // namespace la3g

using namespace la3g;

extern "C" int la3g_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                             uint64_t seed, int weighted, uint64_t wseed, la3g_edges* out)
{
  std::memset(out, 0, sizeof *out);
  if (scale < 1 || scale > 31 || edge_factor == 0 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
    return set_error(LA3G_EINVAL, "gen_rmat: bad parameters");
  const uint32_t n = 1u << scale;
  const uint64_t m0 = (uint64_t) edge_factor * n;
  const uint64_t ta = (uint64_t) std::ldexp(a, 32), tb = (uint64_t) std::ldexp(a + b, 32),
                 tc = (uint64_t) std::ldexp(a + b + c, 32);
  std::vector<uint32_t> perm = permutation(n, seed);
  std::vector<EdgeKey> e;
  try { e.resize(m0); } catch (const std::bad_alloc&) { return set_error(LA3G_ENOMEM, "gen_rmat: out of host memory"); }
  const uint64_t key = mix64(seed ^ 0x726D61745F676E21ull);
  std::atomic<uint64_t> kept(0);
  // Each thread writes its kept edges compactly into its own slice first.
  std::vector<uint64_t> cnt(host_threads() + 1, 0);
  parallel_for(m0, [&](uint64_t lo, uint64_t hi, unsigned t) {
    uint64_t w = lo;
    for (uint64_t i = lo; i < hi; i++)
    {
      uint32_t s = 0, d = 0;
      for (uint32_t l = 0; l < scale; l++)
      {
        uint64_t r = draw(key, i, l + 1) >> 32;
        uint32_t rb = r >= tb, cb = (r >= ta && r < tb) || r >= tc;
        s = (s << 1) | rb;
        d = (d << 1) | cb;
      }
      s = perm[s] + 1;
      d = perm[d] + 1;
      if (s == d) continue;
      e[w].key = ((uint64_t) s << 32) | d;
      e[w].idx = i;
      w++;
    }
    cnt[t] = w - lo;
  });
  // compact the per-thread slices
  {
    unsigned T = host_threads();
    uint64_t pos = 0;
    if (m0 < 65536 || T == 1) pos = cnt[0];
    else
      for (unsigned t = 0; t < T; t++)
      {
        uint64_t lo = m0 * t / T;
        if (pos != lo) std::memmove(&e[pos], &e[lo], cnt[t] * sizeof(EdgeKey));
        pos += cnt[t];
      }
    e.resize(pos);
  }
  return finish_edges(e, n, weighted != 0, wseed, out);
}

extern "C" int la3g_gen_er(uint32_t n, uint64_t m0, uint64_t seed, int weighted, uint64_t wseed,
                           la3g_edges* out)
{
  std::memset(out, 0, sizeof *out);
  if (n < 2 || m0 == 0) return set_error(LA3G_EINVAL, "gen_er: bad parameters");
  std::vector<EdgeKey> e;
  try { e.resize(m0); } catch (const std::bad_alloc&) { return set_error(LA3G_ENOMEM, "gen_er: out of host memory"); }
  const uint64_t key = mix64(seed ^ 0x65726465736E7921ull);
  std::vector<uint64_t> cnt(host_threads() + 1, 0);
  parallel_for(m0, [&](uint64_t lo, uint64_t hi, unsigned t) {
    uint64_t w = lo;
    for (uint64_t i = lo; i < hi; i++)
    {
      uint64_t r = draw(key, i, 1);
      uint32_t s = (uint32_t) ((r >> 32) % n) + 1, d = (uint32_t) ((uint32_t) r % n) + 1;
      if (s == d) continue;
      e[w].key = ((uint64_t) s << 32) | d;
      e[w].idx = i;
      w++;
    }
    cnt[t] = w - lo;
  });
  {
    unsigned T = host_threads();
    uint64_t pos = 0;
    if (m0 < 65536 || T == 1) pos = cnt[0];
    else
      for (unsigned t = 0; t < T; t++)
      {
        uint64_t lo = m0 * t / T;
        if (pos != lo) std::memmove(&e[pos], &e[lo], cnt[t] * sizeof(EdgeKey));
        pos += cnt[t];
      }
    e.resize(pos);
  }
  return finish_edges(e, n, weighted != 0, wseed, out);
}

// Bipartite doc-term corpus: doc d (1..ndocs) holds between terms_per_doc/2
// and 3*terms_per_doc/2 distinct terms drawn by Zipf(zipf_s) over term rank
// (alias method); term ids are a seeded permutation of the ranks (1..nterms);
// tf = 1 + Geometric(1/2), at most 64.  A term whose document frequency
// reaches df_cap * ndocs keeps each posting with probability
// 0.95 * df_cap * ndocs / df, and is trimmed further if it is still at the cap,
// so every df stays below df_cap * ndocs.  Records are (doc, term, tf), in
// doc order.
extern "C" int la3g_gen_bipartite(uint32_t ndocs, uint32_t nterms, uint32_t terms_per_doc,
                                  double zipf_s, double df_cap, uint64_t seed, la3g_edges* out)
{
  std::memset(out, 0, sizeof *out);
  if (ndocs == 0 || nterms == 0 || terms_per_doc == 0 || terms_per_doc * 3 / 2 > nterms || zipf_s <= 0 ||
      df_cap <= 0 || df_cap > 1)
    return set_error(LA3G_EINVAL, "gen_bipartite: bad parameters");
  // Alias table over ranks 0..nterms-1 with weight (rank+1)^-s.
  std::vector<double> prob(nterms);
  std::vector<uint32_t> alias(nterms);
  {
    std::vector<double> wgt(nterms);
    double sum = 0;
    for (uint32_t k = 0; k < nterms; k++) sum += (wgt[k] = std::pow((double) k + 1.0, -zipf_s));
    std::vector<uint32_t> small, large;
    for (uint32_t k = 0; k < nterms; k++)
    {
      wgt[k] = wgt[k] * nterms / sum;
      (wgt[k] < 1.0 ? small : large).push_back(k);
    }
    while (!small.empty() && !large.empty())
    {
      uint32_t s = small.back(), l = large.back();
      small.pop_back();
      prob[s] = wgt[s];
      alias[s] = l;
      wgt[l] = (wgt[l] + wgt[s]) - 1.0;
      if (wgt[l] < 1.0) { large.pop_back(); small.push_back(l); }
    }
    for (uint32_t k : large) { prob[k] = 1.0; alias[k] = k; }
    for (uint32_t k : small) { prob[k] = 1.0; alias[k] = k; }
  }
  std::vector<uint32_t> term_of_rank = permutation(nterms, seed ^ 0x7465726D73ull);
  const uint64_t key = mix64(seed ^ 0x636F72707573ull);
  const uint32_t lo_len = std::max(1u, terms_per_doc / 2), span = terms_per_doc + 1;
  std::vector<uint64_t> doc_ptr((size_t) ndocs + 1, 0);
  for (uint32_t d = 0; d < ndocs; d++) doc_ptr[d + 1] = doc_ptr[d] + lo_len + draw(key, d, 0) % span;
  const uint64_t total = doc_ptr[ndocs];
  std::vector<uint32_t> term, tf;
  try { term.resize(total); tf.resize(total); } catch (const std::bad_alloc&) { return set_error(LA3G_ENOMEM, "gen_bipartite: out of host memory"); }
  parallel_for(ndocs, [&](uint64_t lo, uint64_t hi, unsigned) {
    for (uint64_t d = lo; d < hi; d++)
    {
      uint64_t b = doc_ptr[d], len = doc_ptr[d + 1] - b;
      uint64_t k = 1;
      for (uint64_t j = 0; j < len;)
      {
        uint64_t r = draw(key, d, k++);
        uint32_t slot = (uint32_t) ((r >> 32) % nterms);
        double u = (double) (r & 0xFFFFFFFFull) * (1.0 / 4294967296.0);
        uint32_t rank = u < prob[slot] ? slot : alias[slot];
        uint32_t t = term_of_rank[rank] + 1;
        bool dup = false;
        for (uint64_t q = b; q < b + j; q++) dup |= term[q] == t;
        if (dup) continue;
        term[b + j] = t;
        uint64_t g = draw(key, d, 1000003 + j) | (1ull << 6);
        tf[b + j] = 1u + (uint32_t) __builtin_ctzll(g);
        j++;
      }
      std::sort(term.begin() + b, term.begin() + b + len);
    }
  });
  // Document-frequency cap.
  std::vector<uint64_t> df((size_t) nterms + 1, 0);
  for (uint64_t i = 0; i < total; i++) df[term[i]]++;
  const double cap = df_cap * ndocs;
  const uint64_t tkey = mix64(seed ^ 0x646663617021ull);
  std::vector<uint8_t> keep(total, 1);
  for (uint64_t i = 0; i < total; i++)
  {
    uint32_t t = term[i];
    if ((double) df[t] < cap) continue;
    double p = 0.95 * cap / (double) df[t];
    keep[i] = (double) (draw(tkey, i, t) >> 11) * (1.0 / 9007199254740992.0) < p;
  }
  std::vector<uint64_t> df2((size_t) nterms + 1, 0);
  for (uint64_t i = 0; i < total; i++) df2[term[i]] += keep[i];
  for (uint64_t i = total; i-- > 0;)
    if (keep[i] && (double) df2[term[i]] >= cap) { keep[i] = 0; df2[term[i]]--; }
  uint64_t m = 0;
  for (uint64_t i = 0; i < total; i++) m += keep[i];
  out->n = ndocs;
  out->nright = nterms;
  out->m = m;
  out->weighted = 1;
  out->src = (uint32_t*) std::malloc((m ? m : 1) * sizeof(uint32_t));
  out->dst = (uint32_t*) std::malloc((m ? m : 1) * sizeof(uint32_t));
  out->w = (uint32_t*) std::malloc((m ? m : 1) * sizeof(uint32_t));
  if (!out->src || !out->dst || !out->w) { la3g_edges_free(out); return set_error(LA3G_ENOMEM, "gen_bipartite: out of host memory"); }
  uint64_t o = 0;
  for (uint32_t d = 0; d < ndocs; d++)
    for (uint64_t i = doc_ptr[d]; i < doc_ptr[d + 1]; i++)
      if (keep[i]) { out->src[o] = d + 1; out->dst[o] = term[i]; out->w[o] = tf[i]; o++; }
  return LA3G_OK;
}

extern "C" void la3g_edges_free(la3g_edges* e)
{
  if (!e) return;
  std::free(e->src);
  std::free(e->dst);
  std::free(e->w);
  e->src = e->dst = e->w = nullptr;
  e->m = 0;
}

extern "C" int la3g_edges_write(const la3g_edges* e, const char* path, int header)
{
  FILE* f = std::fopen(path, "wb");
  if (!f) return set_error(LA3G_EIO, "cannot open %s for writing", path);
  const size_t rec = e->weighted ? 12 : 8;
  if (header)
  {
    uint32_t h[4];
    uint64_t nnz = e->m;
    h[0] = e->n - 1;
    h[1] = (e->nright ? e->nright : e->n) - 1;
    std::memcpy(&h[2], &nnz, 8);
    if (std::fwrite(h, 16, 1, f) != 1) { std::fclose(f); return set_error(LA3G_EIO, "write failed: %s", path); }
  }
  const uint64_t chunk = 1 << 20;
  std::vector<uint32_t> buf(chunk * 3);
  for (uint64_t lo = 0; lo < e->m; lo += chunk)
  {
    uint64_t hi = std::min<uint64_t>(e->m, lo + chunk), k = 0;
    for (uint64_t i = lo; i < hi; i++)
    {
      buf[k++] = e->src[i];
      buf[k++] = e->dst[i];
      if (e->weighted) buf[k++] = e->w[i];
    }
    if (std::fwrite(buf.data(), rec, hi - lo, f) != hi - lo)
    {
      std::fclose(f);
      return set_error(LA3G_EIO, "write failed: %s", path);
    }
  }
  if (std::fclose(f) != 0) return set_error(LA3G_EIO, "close failed: %s", path);
  return LA3G_OK;
}
