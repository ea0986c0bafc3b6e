/*
 * la3_oracle.c — CPU restatement of the LA3 vertex-program path at np = 1.
 *
 * TEST INFRASTRUCTURE ONLY (see la3_oracle.h).  It is the checker the GPU
 * path is compared against; it is never part of the product.
 *
 * Layout.  Vertices live in the reference's "internal order": the position
 * of a vertex is its index in the dashboard locator (locator.h:84-120):
 * regular vertices first, then sinks, sources and isolated vertices, each
 * class ascending by hashed id.  The matrix is one CSC whose columns are
 * positions and whose entries (row positions) are sorted ascending, which is
 * the union of the reference's regular `csc` and `sink_csc`
 * (csc_matrix2d.hpp:62-80, csc.h:76-130): regular rows come first because
 * their positions are smaller.
 */
#include "la3_oracle.h"

#include <math.h>
#include <stdarg.h>
#include <stdbool.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

static char og_err[512];

const char* og_last_error(void) { return og_err; }

static int og_fail(int code, const char* fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(og_err, sizeof og_err, fmt, ap);
  va_end(ap);
  return code;
}

struct og_graph
{
  uint32_t flags;
  uint32_t nvertices;   /* n (or ndocs + nterms)                            */
  uint32_t nslots;      /* nvertices + 1 = tile_height at one rank          */
  uint32_t nleft;       /* bipartite: ndocs                                 */
  int null_hash;
  uint64_t hb_height, hb_max_range;
  uint32_t nreg, nsink, nsrc;
  uint32_t* pos_of_hash;
  uint32_t* hash_of_pos;
  uint64_t* col_ptr;    /* nslots + 1                                       */
  uint32_t* ent_row;    /* row position of each entry                       */
  uint32_t* ent_w;      /* weight, or NULL                                  */
  uint64_t nent;
};

/* ---------------------------------------------------------------------- */
/* Hashing: SimpleBucketHasher(max_domain = nvertices, nbuckets = nranks)  */
/* at one rank (hashers.h:39-68), NullHasher for bipartite (hashers.h:25). */
/* ---------------------------------------------------------------------- */

static uint32_t hb_hash(const og_graph* g, uint64_t v)
{
  if (g->null_hash || v >= g->hb_max_range) return (uint32_t) v;
  uint64_t col = (uint32_t) v % 128u;
  uint64_t row = v / 128u;
  return (uint32_t) (row + col * g->hb_height);
}

static uint32_t hb_unhash(const og_graph* g, uint64_t v)
{
  if (g->null_hash || v >= g->hb_max_range) return (uint32_t) v;
  uint64_t col = v / g->hb_height;
  uint64_t row = v % g->hb_height;
  return (uint32_t) (col + row * 128u);
}

uint32_t og_hash(const og_graph* g, uint32_t v) { return hb_hash(g, v); }
uint32_t og_nslots(const og_graph* g) { return g->nslots; }
uint64_t og_nedges(const og_graph* g) { return g->nent; }

void og_classes(const og_graph* g, uint32_t* nregular, uint32_t* nsink, uint32_t* nsource)
{
  *nregular = g->nreg;
  *nsink = g->nsink;
  *nsource = g->nsrc;
}

void og_positions(const og_graph* g, uint32_t* pos_of_orig, uint32_t* orig_of_pos)
{
  for (uint32_t p = 0; p < g->nslots; p++)
  {
    uint32_t o = hb_unhash(g, g->hash_of_pos[p]);
    if (orig_of_pos) orig_of_pos[p] = o;
    if (pos_of_orig) pos_of_orig[o] = p;
  }
}

/* ---------------------------------------------------------------------- */
/* Stable LSD radix sort of 64-bit keys carrying a 32-bit payload.          */
/* ---------------------------------------------------------------------- */

typedef struct { uint64_t key; uint32_t val; uint32_t pad; } og_kv;

static int og_radix_sort(og_kv* a, uint64_t n, uint64_t max_key)
{
  int bits = 0;
  while (bits < 64 && (max_key >> bits) != 0) bits++;
  if (n < 2 || bits == 0) return OG_OK;
  og_kv* tmp = (og_kv*) malloc(n * sizeof(og_kv));
  uint64_t* cnt = (uint64_t*) malloc(65536 * sizeof(uint64_t));
  if (!tmp || !cnt) { free(tmp); free(cnt); return og_fail(OG_ENOMEM, "out of memory in sort"); }
  og_kv *src = a, *dst = tmp;
  for (int shift = 0; shift < bits; shift += 16)
  {
    memset(cnt, 0, 65536 * sizeof(uint64_t));
    for (uint64_t i = 0; i < n; i++) cnt[(src[i].key >> shift) & 0xFFFF]++;
    uint64_t s = 0;
    for (int d = 0; d < 65536; d++) { uint64_t c = cnt[d]; cnt[d] = s; s += c; }
    for (uint64_t i = 0; i < n; i++) dst[cnt[(src[i].key >> shift) & 0xFFFF]++] = src[i];
    og_kv* t = src; src = dst; dst = t;
  }
  if (src != a) memcpy(a, src, n * sizeof(og_kv));
  free(tmp);
  free(cnt);
  return OG_OK;
}

/* ---------------------------------------------------------------------- */
/* Ingest: Graph::load_binary (graph.hpp:37-214), classification           */
/* (processed_matrix2d.hpp:203-228), locators (locator.h:84-155) and the   */
/* per-tile dedup + CSC build (csc_matrix2d.hpp:62-80, csc.h:76-130).      */
/* ---------------------------------------------------------------------- */

int og_load(const char* path, uint32_t n, uint32_t nright, uint32_t flags, og_graph** out)
{
  *out = NULL;
  const bool weighted = flags & OG_WEIGHTED;
  const bool bipartite = flags & OG_BIPARTITE;
  const bool directed = flags & OG_DIRECTED;
  const bool reverse = flags & OG_REVERSE;
  const bool acyclic = flags & OG_ACYCLIC;
  const size_t rec = weighted ? 12 : 8;

  og_graph* g = (og_graph*) calloc(1, sizeof(og_graph));
  if (!g) return og_fail(OG_ENOMEM, "out of memory");
  g->flags = flags;

  uint32_t nrows = n, ncols = bipartite ? nright : n;
  g->nvertices = bipartite ? nrows + ncols : nrows;
  g->nleft = nrows;

  FILE* f = fopen(path, "rb");
  if (!f) { og_free(g); return og_fail(OG_EIO, "cannot open %s", path); }
  struct stat st;
  if (stat(path, &st) != 0) { fclose(f); og_free(g); return og_fail(OG_EIO, "cannot stat %s", path); }
  uint64_t filesize = (uint64_t) st.st_size, offset = 0;

  /* graph.hpp:195-235: n == 0 means a 16-byte header {u32 n-1, u32 m-1, u64 nnz}.
   * The reference only derives nvertices from the header for bipartite graphs;
   * here it is derived in both cases (the reference's directed/undirected header
   * path builds a zero-sized matrix). */
  if (n == 0)
  {
    uint32_t h[4];
    if (fread(h, 16, 1, f) != 1) { fclose(f); og_free(g); return og_fail(OG_EFORMAT, "short header"); }
    nrows = h[0] + 1;
    ncols = h[1] + 1;
    g->nleft = nrows;
    g->nvertices = bipartite ? nrows + ncols : nrows;
    offset = 16;
  }
  g->nslots = g->nvertices + 1;  /* tile_height = nrows / nrowgrps + 1 (matrix2d.hpp:8) */
  g->null_hash = bipartite;
  if (!bipartite)
  {
    g->hb_height = (uint64_t) g->nvertices / 128u;
    g->hb_max_range = g->hb_height * 128u;
  }

  uint64_t nrec = (filesize - offset) / rec;  /* a trailing partial record is ignored */
  uint8_t* buf = (uint8_t*) malloc(nrec * rec + 1);
  if (!buf) { fclose(f); og_free(g); return og_fail(OG_ENOMEM, "out of memory"); }
  if (nrec && fread(buf, rec, nrec, f) != nrec)
  { free(buf); fclose(f); og_free(g); return og_fail(OG_EIO, "short read"); }
  fclose(f);

  const uint64_t N = g->nslots;
  uint64_t cap = nrec * (directed ? 1 : 2);
  og_kv* kv = (og_kv*) malloc((cap ? cap : 1) * sizeof(og_kv));
  uint32_t* wseq = weighted ? (uint32_t*) malloc((cap ? cap : 1) * sizeof(uint32_t)) : NULL;
  if (!kv || (weighted && !wseq)) { free(buf); free(kv); free(wseq); og_free(g); return og_fail(OG_ENOMEM, "out of memory"); }
  uint64_t m = 0;
  for (uint64_t i = 0; i < nrec; i++)
  {
    uint32_t t[3] = {0, 0, 0};
    memcpy(t, buf + i * rec, rec);
    uint32_t row = t[0], col = t[1], w = t[2];
    if (bipartite) col += nrows;                       /* graph.hpp:162-163 */
    if (row == col) continue;                          /* graph.hpp:166-167 */
    if (directed && !reverse) { uint32_t s = row; row = col; col = s; }  /* :171-172 */
    if (acyclic && ((!reverse && col > row) || (reverse && col < row)))  /* :174-179 */
    { uint32_t s = row; row = col; col = s; }
    uint32_t hr = hb_hash(g, row), hc = hb_hash(g, col);                 /* :181-182 */
    if (hr >= N || hc >= N)
    {
      free(buf); free(kv); free(wseq); og_free(g);
      return og_fail(OG_EINVAL, "record %llu: vertex id out of range (nslots %llu)",
                     (unsigned long long) i, (unsigned long long) N);
    }
    /* Insertion order = file order (np = 1 keeps the tile's triples in
     * place, dist_matrix2d.hpp:145-152); the payload is the insertion index. */
    if (weighted) wseq[m] = w;
    kv[m].key = (uint64_t) hr * N + hc; kv[m].val = (uint32_t) m; m++;
    if (!directed)                                     /* graph.hpp:187-191 */
    {
      if (weighted) wseq[m] = w;
      kv[m].key = (uint64_t) hc * N + hr; kv[m].val = (uint32_t) m; m++;
    }
  }
  free(buf);

  /* Dedup (csc_matrix2d.hpp:62-72): an unordered_set keyed on (row, col)
   * keeps the first inserted triple.  A stable sort by key keeps insertion
   * order among equal keys; the first of each run wins. */
  int rc = og_radix_sort(kv, m, N * N - 1);
  if (rc) { free(kv); free(wseq); og_free(g); return rc; }
  uint64_t u = 0;
  for (uint64_t i = 0; i < m; i++)
    if (i == 0 || kv[i].key != kv[i - 1].key) kv[u++] = kv[i];
  g->nent = u;

  /* Row / column non-emptiness and classes (processed_matrix2d.hpp:203-228,
   * CONSIDER_DANGLING_PRIMARY false). */
  uint8_t* rowne = (uint8_t*) calloc(N, 1);
  uint8_t* colne = (uint8_t*) calloc(N, 1);
  g->pos_of_hash = (uint32_t*) malloc(N * sizeof(uint32_t));
  g->hash_of_pos = (uint32_t*) malloc(N * sizeof(uint32_t));
  if (!rowne || !colne || !g->pos_of_hash || !g->hash_of_pos)
  { free(rowne); free(colne); free(kv); free(wseq); og_free(g); return og_fail(OG_ENOMEM, "out of memory"); }
  for (uint64_t i = 0; i < u; i++) { rowne[kv[i].key / N] = 1; colne[kv[i].key % N] = 1; }
  uint32_t pos = 0;
  for (int cls = 0; cls < 4; cls++)  /* regular, sink, source, rest (locator.h:105-113) */
  {
    for (uint64_t h = 0; h < N; h++)
    {
      int c = (rowne[h] && colne[h]) ? 0 : rowne[h] ? 1 : colne[h] ? 2 : 3;
      if (c != cls) continue;
      g->pos_of_hash[h] = pos;
      g->hash_of_pos[pos] = (uint32_t) h;
      pos++;
      if (cls == 0) g->nreg++;
      else if (cls == 1) g->nsink++;
      else if (cls == 2) g->nsrc++;
    }
  }
  free(rowne);
  free(colne);

  /* CSC in positions: columns in locator order, entries sorted by row
   * position (csc.h:124-125 sorts each column by global_idx). */
  for (uint64_t i = 0; i < u; i++)
  {
    uint64_t hr = kv[i].key / N, hc = kv[i].key % N;
    kv[i].key = (uint64_t) g->pos_of_hash[hc] * N + g->pos_of_hash[hr];
  }
  rc = og_radix_sort(kv, u, N * N - 1);
  if (rc) { free(kv); free(wseq); og_free(g); return rc; }
  g->col_ptr = (uint64_t*) calloc(N + 1, sizeof(uint64_t));
  g->ent_row = (uint32_t*) malloc((u ? u : 1) * sizeof(uint32_t));
  g->ent_w = weighted ? (uint32_t*) malloc((u ? u : 1) * sizeof(uint32_t)) : NULL;
  if (!g->col_ptr || !g->ent_row || (weighted && !g->ent_w))
  { free(kv); free(wseq); og_free(g); return og_fail(OG_ENOMEM, "out of memory"); }
  for (uint64_t i = 0; i < u; i++)
  {
    g->col_ptr[kv[i].key / N + 1]++;
    g->ent_row[i] = (uint32_t) (kv[i].key % N);
    if (weighted) g->ent_w[i] = wseq[kv[i].val];
  }
  for (uint64_t c = 0; c < N; c++) g->col_ptr[c + 1] += g->col_ptr[c];
  free(kv);
  free(wseq);
  *out = g;
  return OG_OK;
}

void og_free(og_graph* g)
{
  if (!g) return;
  free(g->pos_of_hash);
  free(g->hash_of_pos);
  free(g->col_ptr);
  free(g->ent_row);
  free(g->ent_w);
  free(g);
}

/* ---------------------------------------------------------------------- */
/* Generic BSP engine: a restatement of VertexProgram::execute and its     */
/* specialisations (vertex_program_execute.hpp:11-345, 564-724).           */
/* ---------------------------------------------------------------------- */

typedef struct og_prog
{
  size_t msz, asz, ssz;
  bool stationary;
  bool gather_state;  /* gather(edge, msg, state) overridden                */
  bool apply_iter;    /* apply(y, state, iter) overridden                   */
  void* ctx;
  void (*scatter)(void* ctx, const void* s, void* m);
  void (*gather)(void* ctx, uint32_t src, uint32_t dst, uint32_t w, const void* m,
                 const void* dst_state, void* a);
  void (*combine)(void* ctx, const void* y1, void* y2);
  bool (*apply)(void* ctx, const void* y, void* s, uint32_t iter);
  void (*acc_zero)(void* ctx, void* a); /* A() */
} og_prog;

/* StreamingArray (streaming_array.h:92-108): values are packed in push
 * order while the indices live in a bitmap; iteration walks the bitmap in
 * ascending order and pairs the j-th index with the j-th packed value. */
typedef struct
{
  uint32_t n, cnt;
  uint8_t* bit;
  char* vals;
  size_t msz;
} og_xseg;

static bool xseg_init(og_xseg* x, uint32_t n, size_t msz)
{
  x->n = n;
  x->cnt = 0;
  x->msz = msz;
  x->bit = (uint8_t*) calloc(n + 1, 1);
  x->vals = (char*) calloc((size_t) n + 1, msz ? msz : 1);
  return x->bit && x->vals;
}
static void xseg_free(og_xseg* x) { free(x->bit); free(x->vals); }
static void xseg_clear(og_xseg* x) { memset(x->bit, 0, x->n + 1); x->cnt = 0; }
static void xseg_push(og_xseg* x, uint32_t idx, const void* val)
{
  if (x->msz) memcpy(x->vals + (size_t) x->cnt * x->msz, val, x->msz);
  if (!x->bit[idx]) { x->bit[idx] = 1; x->cnt++; }
}

typedef struct og_vp
{
  const og_graph* g;
  og_prog* p;
  char* S;          /* states, in positions                                 */
  char* mirror;     /* state snapshot read by gather(..., state)            */
  char* Y;          /* accumulators, in positions                           */
  uint8_t* touched; /* accumulator activity                                 */
  uint8_t* active;  /* vertex activity (vseg.activity)                      */
  og_xseg xr;       /* regular messages, index = regular position           */
  og_xseg xs;       /* source messages, index = position - nreg - nsink     */
  char* tmp_m;
  char* tmp_a;
  char* tmp_a2;
} og_vp;

#define SPTR(vp, i_) ((vp)->S + (size_t) (i_) * (vp)->p->ssz)
#define YPTR(vp, i_) ((vp)->Y + (size_t) (i_) * (vp)->p->asz)

static int vp_init(og_vp* vp, const og_graph* g, og_prog* p, char* states)
{
  memset(vp, 0, sizeof *vp);
  vp->g = g;
  vp->p = p;
  vp->S = states;
  uint32_t N = g->nslots;
  vp->Y = (char*) malloc((size_t) N * p->asz);
  vp->touched = (uint8_t*) calloc(N, 1);
  vp->active = (uint8_t*) calloc(N, 1);
  vp->tmp_m = (char*) calloc(1, p->msz ? p->msz : 1);
  vp->tmp_a = (char*) calloc(1, p->asz);
  vp->tmp_a2 = (char*) calloc(1, p->asz);
  if (!vp->Y || !vp->touched || !vp->active || !vp->tmp_m || !vp->tmp_a || !vp->tmp_a2 ||
      !xseg_init(&vp->xr, g->nreg, p->msz) || !xseg_init(&vp->xs, g->nsrc, p->msz))
    return og_fail(OG_ENOMEM, "out of memory");
  for (uint32_t i = 0; i < N; i++) p->acc_zero(p->ctx, YPTR(vp, i));
  return OG_OK;
}

static void vp_free(og_vp* vp)
{
  free(vp->Y);
  free(vp->touched);
  free(vp->active);
  free(vp->mirror);
  free(vp->tmp_m);
  free(vp->tmp_a);
  free(vp->tmp_a2);
  xseg_free(&vp->xr);
  xseg_free(&vp->xs);
}

/* Mirrors (vertex_program.hpp:159-173): the states of active vertices (all
 * of them if stationary) are copied once, at the first initialize; gather
 * reads those copies afterwards. */
static int vp_mirror(og_vp* vp)
{
  if (!vp->p->gather_state || vp->mirror) return OG_OK;
  size_t bytes = (size_t) vp->g->nslots * vp->p->ssz;
  vp->mirror = (char*) calloc(1, bytes);
  if (!vp->mirror) return og_fail(OG_ENOMEM, "out of memory");
  for (uint32_t i = 0; i < vp->g->nslots; i++)
    if (vp->p->stationary || vp->active[i])
      memcpy(vp->mirror + (size_t) i * vp->p->ssz, SPTR(vp, i), vp->p->ssz);
  memset(vp->active, 0, vp->g->nslots);
  return OG_OK;
}

/* VertexProgram::SpMV (vertex_program_execute.hpp:564-603) restricted to the
 * rows [row_lo, row_hi): for each active column in ascending order, each of
 * its entries in ascending row position, y[row] = combine(gather(...), y[row]). */
static void vp_spmv(og_vp* vp, const og_xseg* x, uint32_t col_base, uint32_t row_lo, uint32_t row_hi)
{
  const og_graph* g = vp->g;
  og_prog* p = vp->p;
  uint32_t j = 0;
  for (uint32_t i = 0; i < x->n; i++)
  {
    if (!x->bit[i]) continue;
    const char* msg = x->vals + (size_t) j * x->msz;
    j++;
    uint32_t c = col_base + i;
    for (uint64_t e = g->col_ptr[c]; e < g->col_ptr[c + 1]; e++)
    {
      uint32_t r = g->ent_row[e];
      if (r < row_lo) continue;
      if (r >= row_hi) break;
      const void* st = p->gather_state ? (const void*) (vp->mirror + (size_t) r * p->ssz) : NULL;
      p->gather(p->ctx, g->hash_of_pos[c], g->hash_of_pos[r], g->ent_w ? g->ent_w[e] : 0, msg, st, vp->tmp_a);
      p->combine(p->ctx, vp->tmp_a, YPTR(vp, r));
      vp->touched[r] = 1;
    }
  }
}

/* produce_messages + combine_accumulators + apply_and_scatter_messages
 * (vertex_program_execute.hpp:606-724). */
static bool vp_produce(og_vp* vp, bool sink, bool single_iter, uint32_t iter)
{
  const og_graph* g = vp->g;
  og_prog* p = vp->p;
  bool any = false;
  uint32_t lo = sink ? g->nreg : 0, hi = sink ? g->nreg + g->nsink : g->nreg;
  if (!sink) xseg_clear(&vp->xr);
  for (uint32_t r = lo; r < hi; r++)
  {
    if (!vp->touched[r]) continue;
    vp->touched[r] = 0;
    /* final = combine(partial, A()) */
    p->acc_zero(p->ctx, vp->tmp_a2);
    p->combine(p->ctx, YPTR(vp, r), vp->tmp_a2);
    p->acc_zero(p->ctx, YPTR(vp, r));
    bool act = p->apply(p->ctx, vp->tmp_a2, SPTR(vp, r), iter);
    if (sink)
    {
      if (act) vp->active[r] = 1;  /* sink activations do not count (:684-698) */
    }
    else
    {
      any |= act;
      if (act || p->stationary)
      {
        vp->active[r] = 1;
        if (!single_iter)
        {
          p->scatter(p->ctx, SPTR(vp, r), vp->tmp_m);
          xseg_push(&vp->xr, r, vp->tmp_m);
        }
      }
    }
  }
  return any;
}

static void vp_process(og_vp* vp, bool sink, uint32_t iter)
{
  const og_graph* g = vp->g;
  uint32_t lo = sink ? g->nreg : 0, hi = sink ? g->nreg + g->nsink : g->nreg;
  uint32_t src_base = g->nreg + g->nsink;
  /* process_ready_messages (:433-492): source messages first, then regular. */
  if (sink || vp->p->stationary || iter == 0) vp_spmv(vp, &vp->xs, src_base, lo, hi);
  vp_spmv(vp, &vp->xr, 0, lo, hi);
}

/* execute (vertex_program_execute.hpp:11-52).  Returns iterations run. */
static uint32_t vp_execute(og_vp* vp, uint32_t max_iters)
{
  const og_graph* g = vp->g;
  og_prog* p = vp->p;
  const bool directed = g->flags & OG_DIRECTED;
  const bool optimizable = directed && !p->gather_state && !p->apply_iter;  /* :77 */
  if (max_iters == 1)
  {
    /* execute_single (:251-302) / execute_single_undirected (:305-345) */
    vp_process(vp, false, 0);
    if (directed) vp_process(vp, true, 0);
    vp_produce(vp, false, true, 0);
    if (directed) vp_produce(vp, true, true, 0);
    return 1;
  }
  uint32_t iter = 0;
  bool until = max_iters == 0, converged = false;
  if (optimizable)
  {
    /* execute_ (:55-163) */
    while (until ? !converged : iter < max_iters)
    {
      vp_process(vp, false, iter);
      converged = !vp_produce(vp, false, false, iter);
      iter++;
    }
    /* Sink pass (:131-148): re-scatter every regular vertex, then gather
     * source + regular messages into the sink rows once. */
    xseg_clear(&vp->xr);
    for (uint32_t r = 0; r < g->nreg; r++)
    {
      p->scatter(p->ctx, SPTR(vp, r), vp->tmp_m);
      xseg_push(&vp->xr, r, vp->tmp_m);
    }
    vp_process(vp, true, iter);
    vp_produce(vp, true, false, iter);
  }
  else
  {
    /* execute_non_opt (:166-248) */
    while (until ? !converged : iter < max_iters)
    {
      vp_process(vp, false, iter);
      if (directed) vp_process(vp, true, iter);
      converged = !vp_produce(vp, false, false, iter);
      if (directed) converged &= !vp_produce(vp, true, false, iter);
      iter++;
    }
  }
  return iter;
}

/* initialize() (vertex_program.hpp:84-174) with an init callback by
 * original id.  Regular and source vertices whose init returns true push
 * their scatter; init runs for every vertex in internal order. */
typedef bool (*og_init_fn)(void* ctx, uint32_t vid, uint32_t pos, void* s);

static int vp_initialize(og_vp* vp, og_init_fn init, void* ictx)
{
  const og_graph* g = vp->g;
  og_prog* p = vp->p;
  const bool directed = g->flags & OG_DIRECTED;
  uint32_t src_base = g->nreg + g->nsink, iso_base = src_base + g->nsrc;
  for (uint32_t i = 0; i < g->nslots; i++)
  {
    uint32_t vid = hb_unhash(g, g->hash_of_pos[i]);
    bool act = init(ictx, vid, i, SPTR(vp, i));
    if (!act) continue;
    if (i < g->nreg)
    {
      p->scatter(p->ctx, SPTR(vp, i), vp->tmp_m);
      xseg_push(&vp->xr, i, vp->tmp_m);
    }
    else if (directed && i >= src_base && i < iso_base)
    {
      p->scatter(p->ctx, SPTR(vp, i), vp->tmp_m);
      xseg_push(&vp->xs, i - src_base, vp->tmp_m);
    }
  }
  return vp_mirror(vp);
}

/* ---------------------------------------------------------------------- */
/* PageRank (pr.h:12-46, pr.cpp:11-55) and out-degree (degree.h:17-35).    */
/* ---------------------------------------------------------------------- */

typedef struct { double rank; uint32_t degree; uint32_t pad; } pr_state;
static const double PR_ALPHA = 0.15, PR_TOL = 1e-5;

static void pr_scatter(void* c, const void* s, void* m)
{ const pr_state* st = (const pr_state*) s; *(double*) m = st->rank / (double) st->degree; }
static void pr_gather(void* c, uint32_t src, uint32_t dst, uint32_t w, const void* m, const void* ds, void* a)
{ *(double*) a = *(const double*) m; }
static void pr_combine(void* c, const void* y1, void* y2) { *(double*) y2 += *(const double*) y1; }
static bool pr_apply(void* c, const void* y, void* s, uint32_t iter)
{
  pr_state* st = (pr_state*) s;
  double tmp = st->rank;
  st->rank = PR_ALPHA + (1.0 - PR_ALPHA) * *(const double*) y;
  return fabs(st->rank - tmp) > PR_TOL;
}
static void pr_zero(void* c, void* a) { *(double*) a = 0.0; }
static bool pr_init(void* ctx, uint32_t vid, uint32_t pos, void* s)
{
  /* PrVertex::init(vid, other, s) copies the out-degree (pr.h:34-35); the
   * out-degree of a vertex is the number of distinct out-neighbours, i.e.
   * the length of its column (DegVertex on the reversed graph, pr.cpp:14-21). */
  const og_graph* g = (const og_graph*) ctx;
  ((pr_state*) s)->degree = (uint32_t) (g->col_ptr[pos + 1] - g->col_ptr[pos]);
  return true;
}

int og_pagerank(const og_graph* g, uint32_t iters, double* rank, uint32_t* degree)
{
  if (!(g->flags & OG_DIRECTED)) return og_fail(OG_EINVAL, "pagerank needs a directed graph");
  og_prog p = {sizeof(double), sizeof(double), sizeof(pr_state), true, false, false, NULL,
               pr_scatter, pr_gather, pr_combine, pr_apply, pr_zero};
  pr_state* S = (pr_state*) calloc(g->nslots, sizeof(pr_state));
  if (!S) return og_fail(OG_ENOMEM, "out of memory");
  for (uint32_t i = 0; i < g->nslots; i++) S[i].rank = PR_ALPHA;
  og_vp vp;
  int rc = vp_init(&vp, g, &p, (char*) S);
  if (!rc) rc = vp_initialize(&vp, pr_init, (void*) g);
  if (!rc)
  {
    vp_execute(&vp, iters);
    for (uint32_t i = 0; i < g->nslots; i++)
    {
      uint32_t o = hb_unhash(g, g->hash_of_pos[i]);
      if (rank) rank[o] = S[i].rank;
      if (degree) degree[o] = S[i].degree;
    }
  }
  vp_free(&vp);
  free(S);
  return rc;
}

/* ---------------------------------------------------------------------- */
/* BFS (bfs.h:11-49, bfs.cpp:11-37).                                       */
/* ---------------------------------------------------------------------- */

typedef struct { uint32_t parent; uint8_t hops; uint8_t pad[3]; } bfs_state;

static void bfs_scatter(void* c, const void* s, void* m) {}
static void bfs_gather(void* c, uint32_t src, uint32_t dst, uint32_t w, const void* m, const void* ds, void* a)
{ *(uint32_t*) a = src; }
static void bfs_combine(void* c, const void* y1, void* y2) { *(uint32_t*) y2 = *(const uint32_t*) y1; }
static bool bfs_apply(void* c, const void* y, void* s, uint32_t iter)
{
  bfs_state* st = (bfs_state*) s;
  if (st->hops != 255) return false;
  st->hops = (uint8_t) (iter + 1);
  st->parent = *(const uint32_t*) y;
  return true;
}
static void u32_zero(void* c, void* a) { *(uint32_t*) a = 0; }
static bool bfs_init(void* ctx, uint32_t vid, uint32_t pos, void* s)
{
  if (vid == *(const uint32_t*) ctx) { ((bfs_state*) s)->hops = 0; return true; }
  return false;
}

int og_bfs(const og_graph* g, uint32_t root, uint8_t* hops, uint32_t* parent, uint32_t* niters)
{
  og_prog p = {0, sizeof(uint32_t), sizeof(bfs_state), false, false, true, NULL,
               bfs_scatter, bfs_gather, bfs_combine, bfs_apply, u32_zero};
  bfs_state* S = (bfs_state*) calloc(g->nslots, sizeof(bfs_state));
  if (!S) return og_fail(OG_ENOMEM, "out of memory");
  for (uint32_t i = 0; i < g->nslots; i++) S[i].hops = 255;
  og_vp vp;
  int rc = vp_init(&vp, g, &p, (char*) S);
  if (!rc) rc = vp_initialize(&vp, bfs_init, &root);
  if (!rc)
  {
    uint32_t it = vp_execute(&vp, 0);
    if (niters) *niters = it;
    for (uint32_t i = 0; i < g->nslots; i++)
    {
      uint32_t o = hb_unhash(g, g->hash_of_pos[i]);
      if (hops) hops[o] = S[i].hops;
      if (parent) parent[o] = S[i].parent;
    }
  }
  vp_free(&vp);
  free(S);
  return rc;
}

/* ---------------------------------------------------------------------- */
/* SSSP (sssp.h:11-46, sssp.cpp:11-37).  INF = UINT32_MAX / 2.             */
/* ---------------------------------------------------------------------- */

static const uint32_t SP_INF = 0x7FFFFFFFu;

static void sp_scatter(void* c, const void* s, void* m) { *(uint32_t*) m = *(const uint32_t*) s; }
static void sp_gather(void* c, uint32_t src, uint32_t dst, uint32_t w, const void* m, const void* ds, void* a)
{ *(uint32_t*) a = *(const uint32_t*) m + w; }
static void sp_combine(void* c, const void* y1, void* y2)
{
  uint32_t a = *(const uint32_t*) y1, *b = (uint32_t*) y2;
  if (a < *b) *b = a;
}
static bool sp_apply(void* c, const void* y, void* s, uint32_t iter)
{
  uint32_t* d = (uint32_t*) s;
  uint32_t tmp = *d, v = *(const uint32_t*) y;
  if (v < *d) *d = v;
  return tmp != *d;
}
static void sp_zero(void* c, void* a) { *(uint32_t*) a = SP_INF; }
static bool sp_init(void* ctx, uint32_t vid, uint32_t pos, void* s)
{
  if (vid == *(const uint32_t*) ctx) { *(uint32_t*) s = 0; return true; }
  return false;
}

int og_sssp(const og_graph* g, uint32_t root, uint32_t* dist, uint32_t* niters)
{
  if (!(g->flags & OG_DIRECTED) || !g->ent_w) return og_fail(OG_EINVAL, "sssp needs a weighted directed graph");
  og_prog p = {sizeof(uint32_t), sizeof(uint32_t), sizeof(uint32_t), false, false, false, NULL,
               sp_scatter, sp_gather, sp_combine, sp_apply, sp_zero};
  uint32_t* S = (uint32_t*) malloc((size_t) g->nslots * sizeof(uint32_t));
  if (!S) return og_fail(OG_ENOMEM, "out of memory");
  for (uint32_t i = 0; i < g->nslots; i++) S[i] = SP_INF;
  og_vp vp;
  int rc = vp_init(&vp, g, &p, (char*) S);
  if (!rc) rc = vp_initialize(&vp, sp_init, &root);
  if (!rc)
  {
    uint32_t it = vp_execute(&vp, 0);
    if (niters) *niters = it;
    for (uint32_t i = 0; i < g->nslots; i++)
      if (dist) dist[hb_unhash(g, g->hash_of_pos[i])] = S[i];
  }
  vp_free(&vp);
  free(S);
  return rc;
}

/* ---------------------------------------------------------------------- */
/* CC (cc.h:11-38, cc.cpp:11-31).  combine treats 0 as "no value yet".     */
/* ---------------------------------------------------------------------- */

static void cc_gather(void* c, uint32_t src, uint32_t dst, uint32_t w, const void* m, const void* ds, void* a)
{ *(uint32_t*) a = *(const uint32_t*) m; }
static void cc_combine(void* c, const void* y1, void* y2)
{
  uint32_t a = *(const uint32_t*) y1, *b = (uint32_t*) y2;
  *b = (*b == 0) ? a : (a < *b ? a : *b);
}
static bool cc_init(void* ctx, uint32_t vid, uint32_t pos, void* s) { *(uint32_t*) s = vid; return true; }

int og_cc(const og_graph* g, uint32_t* label, uint32_t* niters)
{
  og_prog p = {sizeof(uint32_t), sizeof(uint32_t), sizeof(uint32_t), false, false, false, NULL,
               sp_scatter, cc_gather, cc_combine, sp_apply, u32_zero};
  uint32_t* S = (uint32_t*) calloc(g->nslots, sizeof(uint32_t));
  if (!S) return og_fail(OG_ENOMEM, "out of memory");
  og_vp vp;
  int rc = vp_init(&vp, g, &p, (char*) S);
  if (!rc) rc = vp_initialize(&vp, cc_init, NULL);
  if (!rc)
  {
    uint32_t it = vp_execute(&vp, 0);
    if (niters) *niters = it;
    for (uint32_t i = 0; i < g->nslots; i++)
      if (label) label[hb_unhash(g, g->hash_of_pos[i])] = S[i];
  }
  vp_free(&vp);
  free(S);
  return rc;
}

/* ---------------------------------------------------------------------- */
/* Triangle counting (tc.h:47-99, tc.cpp:11-52).                            */
/* ---------------------------------------------------------------------- */

static int u32_cmp(const void* a, const void* b)
{
  uint32_t x = *(const uint32_t*) a, y = *(const uint32_t*) b;
  return x < y ? -1 : x > y;
}

int og_tc(const og_graph* g, uint32_t* ntriangles, uint64_t* total)
{
  if ((g->flags & (OG_DIRECTED | OG_ACYCLIC | OG_REVERSE)) != (OG_DIRECTED | OG_ACYCLIC))
    return og_fail(OG_EINVAL, "tc needs load_directed(reverse=false, remove_cycles=true)");
  const uint32_t N = g->nslots;
  /* P1, GnVertex on G (rows = higher endpoint, columns = lower endpoint):
   * each vertex collects the hashed ids of its lower-id neighbours, sorted
   * (tc.h:53-63).  Indexed here by hashed id. */
  uint64_t* lptr = (uint64_t*) calloc((size_t) N + 1, sizeof(uint64_t));
  uint32_t* lst = (uint32_t*) malloc((g->nent ? g->nent : 1) * sizeof(uint32_t));
  uint32_t* fill = (uint32_t*) calloc(N, sizeof(uint32_t));
  uint32_t* ntri = (uint32_t*) calloc(N, sizeof(uint32_t));
  if (!lptr || !lst || !fill || !ntri)
  { free(lptr); free(lst); free(fill); free(ntri); return og_fail(OG_ENOMEM, "out of memory"); }
  for (uint32_t c = 0; c < N; c++)
    for (uint64_t e = g->col_ptr[c]; e < g->col_ptr[c + 1]; e++) lptr[g->hash_of_pos[g->ent_row[e]] + 1]++;
  for (uint32_t h = 0; h < N; h++) lptr[h + 1] += lptr[h];
  for (uint32_t c = 0; c < N; c++)
    for (uint64_t e = g->col_ptr[c]; e < g->col_ptr[c + 1]; e++)
    {
      uint32_t hr = g->hash_of_pos[g->ent_row[e]];
      lst[lptr[hr] + fill[hr]++] = g->hash_of_pos[c];
    }
  /* the rows and the per-u intersections below are independent: shared over
   * the host's threads (the reference runs its row tiles under OpenMP too) */
#pragma omp parallel for schedule(dynamic, 1024)
  for (uint32_t h = 0; h < N; h++) qsort(lst + lptr[h], lptr[h + 1] - lptr[h], sizeof(uint32_t), u32_cmp);
  /* P2, CtVertex on the reversed acyclic graph (rows = lower endpoint u,
   * columns = higher endpoint v): u accumulates |N<(u) ∩ N<(v)| over its
   * higher neighbours v by a sorted merge (tc.h:84-97), as uint32.  The
   * reversed graph holds the same oriented edges, so the walk goes over G's
   * entries: in G the column is the lower endpoint and the row the higher. */
#pragma omp parallel for schedule(dynamic, 256)
  for (uint32_t c = 0; c < N; c++)
  {
    uint32_t hu = g->hash_of_pos[c];
    for (uint64_t e = g->col_ptr[c]; e < g->col_ptr[c + 1]; e++)
    {
      uint32_t hv = g->hash_of_pos[g->ent_row[e]];
      const uint32_t *a = lst + lptr[hu], *ae = lst + lptr[hu + 1];
      const uint32_t *b = lst + lptr[hv], *be = lst + lptr[hv + 1];
      uint32_t t = 0;
      while (a != ae && b != be)
      {
        if (*a == *b) { t++; a++; b++; }
        else if (*a < *b) a++;
        else b++;
      }
      ntri[hu] += t;
    }
  }
  uint64_t sum = 0;
  for (uint32_t h = 0; h < N; h++)
  {
    sum += ntri[h];
    if (ntriangles) ntriangles[hb_unhash(g, h)] = ntri[h];
  }
  if (total) *total = sum;
  free(lptr); free(lst); free(fill); free(ntri);
  return OG_OK;
}

/* ---------------------------------------------------------------------- */
/* BM25 (bm25.h:11-92, bm25.cpp:8-114).                                    */
/* ---------------------------------------------------------------------- */

typedef struct { float length; float score; } dt_state;
static const float BM25_K1 = 1.2f, BM25_B = 0.75f;

struct og_bm25
{
  const og_graph* g;
  dt_state* S;
  og_vp vp;     /* TFIDF program; mirrors hold the states after the DL passes */
  og_prog prog;
  uint32_t ndocs;
  float avg_doc_length;
};

static void empty_scatter(void* c, const void* s, void* m) {}
static void f32_combine(void* c, const void* y1, void* y2) { *(float*) y2 += *(const float*) y1; }
static void f32_zero(void* c, void* a) { *(float*) a = 0.0f; }
static void idf_gather(void* c, uint32_t src, uint32_t dst, uint32_t w, const void* m, const void* ds, void* a)
{ *(float*) a = 1.0f; }
static bool idf_apply(void* c, const void* y, void* s, uint32_t iter)
{
  /* s.length = log10((ndocs - y + 0.5) / (y + 0.5)) (bm25.h:42-43): ndocs - y
   * is float arithmetic, the +0.5 promotes to double, log10 is double and the
   * result is stored as float. */
  uint32_t ndocs = *(const uint32_t*) c;
  float yv = *(const float*) y;
  float t = (float) ndocs - yv;
  ((dt_state*) s)->length = (float) log10(((double) t + 0.5) / ((double) yv + 0.5));
  return true;
}
static void dl_gather(void* c, uint32_t src, uint32_t dst, uint32_t w, const void* m, const void* ds, void* a)
{ *(float*) a = (float) w; }
static bool dl_apply(void* c, const void* y, void* s, uint32_t iter)
{
  float avg = *(const float*) c, yv = *(const float*) y;
  dt_state* st = (dt_state*) s;
  if (avg == 0.0f) st->length = yv;
  else st->length = BM25_K1 * ((1.0f - BM25_B) + BM25_B * (yv / avg));  /* bm25.h:65-68 */
  return true;
}
static void tfidf_scatter(void* c, const void* s, void* m) { *(float*) m = ((const dt_state*) s)->length; }
static void tfidf_gather(void* c, uint32_t src, uint32_t dst, uint32_t w, const void* m, const void* ds, void* a)
{
  /* (w * (k1 + 1)) / (w + s.length) * msg, all in float (bm25.h:84-89) */
  const float k1p1 = BM25_K1 + 1.0f;
  float wf = (float) w;
  float num = wf * k1p1;
  float den = wf + ((const dt_state*) ds)->length;
  float q = num / den;
  *(float*) a = q * *(const float*) m;
}
static bool tfidf_apply(void* c, const void* y, void* s, uint32_t iter)
{ ((dt_state*) s)->score = *(const float*) y; return true; }

typedef struct { const og_graph* g; bool left, right; } bip_ctx;
static bool bip_init(void* ctx, uint32_t vid, uint32_t pos, void* s)
{
  /* initialize_bipartite_undirected<left, right> (vertex_program.hpp:350-412):
   * default init returns `stationary` (true for IDF and DL). */
  const bip_ctx* b = (const bip_ctx*) ctx;
  return (b->left && vid <= b->g->nleft) || (b->right && vid > b->g->nleft);
}

static int run_bipartite(const og_graph* g, og_prog* p, dt_state* S, bool left, bool right, uint8_t* active_out)
{
  og_vp vp;
  int rc = vp_init(&vp, g, p, (char*) S);
  bip_ctx bc = {g, left, right};
  if (!rc) rc = vp_initialize(&vp, bip_init, &bc);
  if (!rc)
  {
    vp_execute(&vp, 1);
    if (active_out) memcpy(active_out, vp.active, g->nslots);
  }
  vp_free(&vp);
  return rc;
}

int og_bm25_prepare(const og_graph* g, og_bm25** out, uint64_t* collection_ntokens,
                    float* avg_doc_length, float* length)
{
  *out = NULL;
  if (!(g->flags & OG_BIPARTITE) || (g->flags & OG_DIRECTED))
    return og_fail(OG_EINVAL, "bm25 needs load_bipartite(directed=false)");
  og_bm25* b = (og_bm25*) calloc(1, sizeof(og_bm25));
  dt_state* S = (dt_state*) calloc(g->nslots, sizeof(dt_state));
  uint8_t* active = (uint8_t*) calloc(g->nslots, 1);
  if (!b || !S || !active) { free(b); free(S); free(active); return og_fail(OG_ENOMEM, "out of memory"); }
  b->g = g;
  b->S = S;
  b->ndocs = g->nleft;
  /* Step 1: IDF over docs -> terms (bm25.cpp:19-22). */
  og_prog pidf = {0, sizeof(float), sizeof(dt_state), true, false, false, &b->ndocs,
                  empty_scatter, idf_gather, f32_combine, idf_apply, f32_zero};
  int rc = run_bipartite(g, &pidf, S, true, false, NULL);
  /* Step 2: DL pass 1 (avg 0 => length = sum of tf), the token count over
   * ALL vertices (terms contribute their truncated idf), then pass 2
   * (bm25.cpp:24-47). */
  float avg = 0.0f;
  og_prog pdl = {0, sizeof(float), sizeof(dt_state), true, false, false, &avg,
                 empty_scatter, dl_gather, f32_combine, dl_apply, f32_zero};
  if (!rc) rc = run_bipartite(g, &pdl, S, false, true, NULL);
  uint64_t ntok = 0;
  for (uint32_t i = 0; i < g->nslots && !rc; i++)
  {
    float f = S[i].length;
    /* (uint64_t) of a float: exact for f > -1.  At or below -1 the
     * conversion is undefined in C++ (x86 and AArch64 disagree); the
     * AArch64 / CUDA result, 0, is used. */
    ntok += (f <= -1.0f) ? 0u : (uint64_t) f;
  }
  avg = (float) ntok / (float) b->ndocs;
  if (!rc) rc = run_bipartite(g, &pdl, S, false, true, active);
  if (rc) { free(active); free(S); free(b); return rc; }
  b->avg_doc_length = avg;
  /* TFIDF program.  Its mirrors are taken at its first initialize, when the
   * active vertices are the docs the second DL pass touched
   * (vertex_program.hpp:244-258). */
  og_prog pt = {sizeof(float), sizeof(float), sizeof(dt_state), false, true, false, NULL,
                tfidf_scatter, tfidf_gather, f32_combine, tfidf_apply, f32_zero};
  b->prog = pt;
  rc = vp_init(&b->vp, g, &b->prog, (char*) S);
  if (!rc)
  {
    memcpy(b->vp.active, active, g->nslots);
    rc = vp_mirror(&b->vp);
  }
  free(active);
  if (rc) { og_bm25_free(b); return rc; }
  b->prog.gather_state = true;
  if (collection_ntokens) *collection_ntokens = ntok;
  if (avg_doc_length) *avg_doc_length = avg;
  if (length)
    for (uint32_t i = 0; i < g->nslots; i++) length[hb_unhash(g, g->hash_of_pos[i])] = S[i].length;
  *out = b;
  return OG_OK;
}

typedef struct { uint32_t id; float score; } iv_t;
static int iv_cmp(const void* a, const void* b)
{
  const iv_t *x = (const iv_t*) a, *y = (const iv_t*) b;
  if (x->score > y->score) return -1;
  if (x->score < y->score) return 1;
  return x->id < y->id ? -1 : x->id > y->id;
}

/* One query of the BM25 / LM TFIDF program over the shared states S. */
static int ir_query(const og_graph* g, og_vp* vp, const dt_state* S, const uint32_t* term_vids, uint32_t nterms,
                    uint32_t k, float* scores, uint8_t* active, uint32_t* topk_ids, float* topk_scores,
                    uint32_t* ntopk)
{
  /* reset() then initialize(vids) (vertex_program.hpp:51-63, 177-259): each
   * listed vertex is initialised in list order; regular ones push their
   * scatter.  The pushes go through the StreamingArray, so a list that is
   * not ascending pairs values with indices the way the reference does. */
  xseg_clear(&vp->xr);
  xseg_clear(&vp->xs);
  for (uint32_t q = 0; q < nterms; q++)
  {
    uint32_t v = term_vids[q];
    if (v >= g->nslots) continue;
    uint32_t pos = g->pos_of_hash[hb_hash(g, v)];
    if (pos < g->nreg)
    {
      tfidf_scatter(NULL, SPTR(vp, pos), vp->tmp_m);
      xseg_push(&vp->xr, pos, vp->tmp_m);
    }
  }
  /* execute(1) on an undirected graph = execute_single_undirected. */
  vp_process(vp, false, 0);
  vp_produce(vp, false, true, 0);
  /* topk(k, ..., active_only = true) (vertex_program.hpp:607-680). */
  uint32_t na = 0;
  for (uint32_t i = 0; i < g->nslots; i++) na += vp->active[i];
  iv_t* ivs = (iv_t*) malloc((na ? na : 1) * sizeof(iv_t));
  if (!ivs) return og_fail(OG_ENOMEM, "out of memory");
  uint32_t j = 0;
  if (scores) memset(scores, 0, (size_t) g->nslots * sizeof(float));
  if (active) memset(active, 0, g->nslots);
  for (uint32_t i = 0; i < g->nslots; i++)
  {
    if (!vp->active[i]) continue;
    uint32_t o = hb_unhash(g, g->hash_of_pos[i]);
    ivs[j].id = o;
    ivs[j].score = S[i].score;
    if (scores) scores[o] = S[i].score;
    if (active) active[o] = 1;
    j++;
  }
  qsort(ivs, na, sizeof(iv_t), iv_cmp);
  uint32_t kk = k < na ? k : na;
  for (uint32_t i = 0; i < kk; i++)
  {
    if (topk_ids) topk_ids[i] = ivs[i].id;
    if (topk_scores) topk_scores[i] = ivs[i].score;
  }
  if (ntopk) *ntopk = kk;
  free(ivs);
  memset(vp->active, 0, g->nslots);  /* tfidf.reset_activity() (bm25.cpp:79, lm.cpp:86) */
  return OG_OK;
}

int og_bm25_query(og_bm25* b, const uint32_t* term_vids, uint32_t nterms, uint32_t k,
                  float* scores, uint8_t* active, uint32_t* topk_ids, float* topk_scores,
                  uint32_t* ntopk)
{
  return ir_query(b->g, &b->vp, b->S, term_vids, nterms, k, scores, active, topk_ids, topk_scores, ntopk);
}

void og_bm25_free(og_bm25* b)
{
  if (!b) return;
  vp_free(&b->vp);
  free(b->S);
  free(b);
}

/* ---------------------------------------------------------------------- */
/* LM: query likelihood with Dirichlet smoothing (lm.h:16-75,             */
/* lm.cpp:8-144).                                                          */
/* ---------------------------------------------------------------------- */

static const float LM_MU = 2000.0f;

struct og_lm
{
  const og_graph* g;
  dt_state* S;
  og_vp vp;       /* TFIDF program */
  og_prog prog;
  uint32_t query_nterms;
};

static bool tl_apply(void* c, const void* y, void* s, uint32_t iter)
{
  /* s.length = y / collection_ntokens (lm.h:55): the uint64 count converts to
   * float, then a float divide */
  uint64_t ntok = *(const uint64_t*) c;
  ((dt_state*) s)->length = *(const float*) y / (float) ntok;
  return true;
}
static void lm_gather(void* c, uint32_t src, uint32_t dst, uint32_t w, const void* m, const void* ds, void* a)
{
  /* log10(1.0 + w / (mu * msg)) (lm.h:71): the quotient is float, 1.0
   * promotes it to double, log10 is the double function and the result is
   * stored as float */
  float q = (float) w / (LM_MU * *(const float*) m);
  *(float*) a = (float) log10(1.0 + (double) q);
}
static bool lm_apply(void* c, const void* y, void* s, uint32_t iter)
{
  /* s.score = y + query_nterms * log10(mu / (s.length + mu)) (lm.h:73-74):
   * the argument is float, so log10 resolves to the float overload (log10f
   * of the platform's libm, which is not correctly rounded), and the rest is
   * float arithmetic */
  uint32_t nq = *(const uint32_t*) c;
  dt_state* st = (dt_state*) s;
  float t = log10f(LM_MU / (st->length + LM_MU));
  st->score = *(const float*) y + (float) nq * t;
  return true;
}

int og_lm_prepare(const og_graph* g, og_lm** out, uint64_t* collection_ntokens, float* length)
{
  *out = NULL;
  if (!(g->flags & OG_BIPARTITE) || (g->flags & OG_DIRECTED))
    return og_fail(OG_EINVAL, "lm needs load_bipartite(directed=false)");
  og_lm* b = (og_lm*) calloc(1, sizeof(og_lm));
  dt_state* S = (dt_state*) calloc(g->nslots, sizeof(dt_state));
  uint8_t* active = (uint8_t*) calloc(g->nslots, 1);
  if (!b || !S || !active) { free(b); free(S); free(active); return og_fail(OG_ENOMEM, "out of memory"); }
  b->g = g;
  b->S = S;
  /* Step 1: DL over terms -> docs (lm.cpp:18-22): length(d) = sum of tf. */
  float avg0 = 0.0f;
  og_prog pdl = {0, sizeof(float), sizeof(dt_state), true, false, false, &avg0,
                 empty_scatter, dl_gather, f32_combine, dl_apply, f32_zero};
  int rc = run_bipartite(g, &pdl, S, false, true, NULL);
  /* collection_ntokens = sum over every vertex of (uint64) its float length
   * (lm.cpp:26-29); terms still hold 0 here */
  uint64_t ntok = 0;
  for (uint32_t i = 0; i < g->nslots && !rc; i++)
  {
    float f = S[i].length;
    ntok += (f <= -1.0f) ? 0u : (uint64_t) f;
  }
  /* Step 2: TL over docs -> terms (lm.cpp:33-39). */
  og_prog ptl = {0, sizeof(float), sizeof(dt_state), true, false, false, &ntok,
                 empty_scatter, dl_gather, f32_combine, tl_apply, f32_zero};
  if (!rc) rc = run_bipartite(g, &ptl, S, true, false, active);
  if (rc) { free(active); free(S); free(b); return rc; }
  /* TFIDF program (lm.cpp:46), sharing the states.  Its gather reads no
   * state, so no mirrors are taken at its first initialize and the activity
   * the TL pass left (every term it reached) is still set in the first
   * query's top-k pool (score 0); tfidf.reset_activity() clears it after. */
  og_prog pt = {sizeof(float), sizeof(float), sizeof(dt_state), false, false, false, &b->query_nterms,
                tfidf_scatter, lm_gather, f32_combine, lm_apply, f32_zero};
  b->prog = pt;
  rc = vp_init(&b->vp, g, &b->prog, (char*) S);
  if (!rc) memcpy(b->vp.active, active, g->nslots);
  free(active);
  if (rc) { og_lm_free(b); return rc; }
  if (collection_ntokens) *collection_ntokens = ntok;
  if (length)
    for (uint32_t i = 0; i < g->nslots; i++) length[hb_unhash(g, g->hash_of_pos[i])] = S[i].length;
  *out = b;
  return OG_OK;
}

int og_lm_query(og_lm* b, const uint32_t* term_vids, uint32_t nterms, uint32_t k, float* scores,
                uint8_t* active, uint32_t* topk_ids, float* topk_scores, uint32_t* ntopk)
{
  b->query_nterms = nterms;  /* tfidf.query_nterms = queries[q].size() (lm.cpp:66) */
  return ir_query(b->g, &b->vp, b->S, term_vids, nterms, k, scores, active, topk_ids, topk_scores, ntopk);
}

void og_lm_free(og_lm* b)
{
  if (!b) return;
  vp_free(&b->vp);
  free(b->S);
  free(b);
}

/* ---------------------------------------------------------------------- */
/* Graph simulation (graphsim.h:60-184, graphsim.cpp:45-90) on the data   */
/* graph loaded reversed.  Labels are integer ids (equal strings, equal  */
/* ids; 0 = the empty string); the query has at most 32 vertices, its     */
/* children lists in file order.                                          */
/* ---------------------------------------------------------------------- */

#define GS_QMAX 32

typedef struct
{
  uint32_t vid, label;
  int32_t degree, deps;
  uint32_t mm;           /* temp mismatches, bit i = query vertex i */
  int32_t pm[GS_QMAX];   /* potential matches */
  char res[GS_QMAX];     /* 'U' | '0' | '1' */
} gs_state;

typedef struct
{
  uint32_t qsize;
  const uint32_t* qlabel;
  const uint32_t* cptr;  /* children of query vertex i: cidx[cptr[i] .. cptr[i + 1]) */
  const uint32_t* cidx;
  const uint32_t* vlabel;  /* by vertex id */
} gs_ctx;

/* InitVertex (graphsim.h:70-92): label and out-degree (in-degree of the
 * reversed graph), stationary, one pass. */
static bool gsi_init(void* ctx, uint32_t vid, uint32_t pos, void* s)
{
  gs_state* st = (gs_state*) s;
  st->vid = vid;
  st->label = ((const gs_ctx*) ctx)->vlabel[vid];
  return true;
}
static void gsi_gather(void* c, uint32_t src, uint32_t dst, uint32_t w, const void* m, const void* ds, void* a)
{ *(int32_t*) a = 1; }
static void i32_combine(void* c, const void* y1, void* y2) { *(int32_t*) y2 += *(const int32_t*) y1; }
static void i32_zero(void* c, void* a) { *(int32_t*) a = 0; }
static bool gsi_apply(void* c, const void* y, void* s, uint32_t iter)
{ ((gs_state*) s)->degree = *(const int32_t*) y; return true; }

/* GsVertex (graphsim.h:100-184). */
static bool gs_init(void* ctx, uint32_t vid, uint32_t pos, void* s)
{
  const gs_ctx* q = (const gs_ctx*) ctx;
  gs_state* st = (gs_state*) s;
  st->mm = 0;
  for (uint32_t i = 0; i < q->qsize; i++) { st->res[i] = 'U'; st->pm[i] = -1; }
  for (uint32_t i = 0; i < q->qsize; i++)
  {
    const bool same = st->label == q->qlabel[i];
    if (same && q->cptr[i] == q->cptr[i + 1]) st->res[i] = '1';
    else if (same && st->degree > 0)
    {
      st->deps++;
      for (uint32_t e = q->cptr[i]; e < q->cptr[i + 1]; e++) st->pm[q->cidx[e]] = st->degree;
    }
    else
    {
      st->res[i] = '0';
      st->mm |= 1u << i;
    }
  }
  return st->mm != 0;
}
static void gs_scatter(void* c, const void* s, void* m) { *(uint32_t*) m = ((const gs_state*) s)->mm; }
static void gs_gather(void* c, uint32_t src, uint32_t dst, uint32_t w, const void* m, const void* ds, void* a)
{
  const gs_ctx* q = (const gs_ctx*) c;
  uint32_t mask = *(const uint32_t*) m;
  for (uint32_t i = 0; i < q->qsize; i++) ((int32_t*) a)[i] = (mask >> i) & 1u;
}
static void gs_combine(void* c, const void* y1, void* y2)
{
  const gs_ctx* q = (const gs_ctx*) c;
  for (uint32_t i = 0; i < q->qsize; i++) ((int32_t*) y2)[i] += ((const int32_t*) y1)[i];
}
static void gs_zero(void* c, void* a) { memset(a, 0, (size_t) ((const gs_ctx*) c)->qsize * sizeof(int32_t)); }
static bool gs_apply(void* c, const void* yv, void* s, uint32_t iter)
{
  const gs_ctx* q = (const gs_ctx*) c;
  const int32_t* y = (const int32_t*) yv;
  gs_state* st = (gs_state*) s;
  if (st->label == 0) return false;  /* s.label.empty() */
  st->mm = 0;
  for (uint32_t i = 0; i < q->qsize; i++)
  {
    if (st->res[i] != 'U') continue;
    /* only the first undecided query vertex is looked at (the loop breaks
     * after it, graphsim.h:172) */
    for (uint32_t e = q->cptr[i]; e < q->cptr[i + 1]; e++)
    {
      uint32_t j = q->cidx[e];
      if (st->pm[j] > 0)
      {
        st->pm[j] -= y[j];
        if (st->pm[j] == 0)
        {
          st->res[i] = '0';
          st->mm |= 1u << i;
          st->deps--;
          break;
        }
      }
    }
    break;
  }
  return st->mm != 0;
}

int og_graphsim(const og_graph* g, const uint32_t* vlabel, uint32_t qsize, const uint32_t* qlabel,
                const uint32_t* qedges, uint32_t nqedges, uint8_t* matched, char* res, uint32_t* nmatches,
                uint32_t* niters)
{
  if (!(g->flags & OG_DIRECTED) || !(g->flags & OG_REVERSE))
    return og_fail(OG_EINVAL, "graphsim needs load_directed(..., reverse=true)");
  if (qsize == 0 || qsize > GS_QMAX) return og_fail(OG_EINVAL, "query size must be 1..32");
  for (uint32_t e = 0; e < 2 * nqedges; e++)
    if (qedges[e] >= qsize) return og_fail(OG_EINVAL, "query edge endpoint out of range");
  uint32_t* cptr = (uint32_t*) calloc(qsize + 1, sizeof(uint32_t));
  uint32_t* cidx = (uint32_t*) malloc((nqedges ? nqedges : 1) * sizeof(uint32_t));
  uint32_t* fill = (uint32_t*) calloc(qsize, sizeof(uint32_t));
  gs_state* S = (gs_state*) calloc(g->nslots, sizeof(gs_state));
  if (!cptr || !cidx || !fill || !S)
  { free(cptr); free(cidx); free(fill); free(S); return og_fail(OG_ENOMEM, "out of memory"); }
  for (uint32_t e = 0; e < nqedges; e++) cptr[qedges[2 * e] + 1]++;
  for (uint32_t i = 0; i < qsize; i++) cptr[i + 1] += cptr[i];
  for (uint32_t e = 0; e < nqedges; e++) cidx[cptr[qedges[2 * e]] + fill[qedges[2 * e]]++] = qedges[2 * e + 1];
  gs_ctx q = {qsize, qlabel, cptr, cidx, vlabel};
  /* InitVertex vp_init(vp, true); vp_init.execute(1) (graphsim.cpp:55-64) */
  og_prog pi = {0, sizeof(int32_t), sizeof(gs_state), true, false, false, &q,
                empty_scatter, gsi_gather, i32_combine, gsi_apply, i32_zero};
  og_vp vp;
  int rc = vp_init(&vp, g, &pi, (char*) S);
  if (!rc) rc = vp_initialize(&vp, gsi_init, &q);
  if (!rc) vp_execute(&vp, 1);
  vp_free(&vp);
  /* vp.execute() until convergence (graphsim.cpp:72) */
  og_prog pg = {sizeof(uint32_t), qsize * sizeof(int32_t), sizeof(gs_state), false, false, true, &q,
                gs_scatter, gs_gather, gs_combine, gs_apply, gs_zero};
  uint32_t it = 0;
  if (!rc) rc = vp_init(&vp, g, &pg, (char*) S);
  if (!rc) rc = vp_initialize(&vp, gs_init, &q);
  if (!rc) it = vp_execute(&vp, 0);
  vp_free(&vp);
  if (!rc)
  {
    uint32_t nm = 0;
    for (uint32_t i = 0; i < g->nslots; i++)
    {
      uint32_t o = hb_unhash(g, g->hash_of_pos[i]);
      bool m = false;
      for (uint32_t k = 0; k < qsize; k++) m |= S[i].res[k] != '0';  /* is_matched (graphsim.h:50-57) */
      nm += m;
      if (matched) matched[o] = m;
      if (res) memcpy(res + (size_t) o * qsize, S[i].res, qsize);
    }
    if (nmatches) *nmatches = nm;
    if (niters) *niters = it;
  }
  free(cptr); free(cidx); free(fill); free(S);
  return rc;
}
