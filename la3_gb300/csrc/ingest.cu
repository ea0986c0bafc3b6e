// Device ingest: LA3 records -> the device matrix in internal order.
//
// Follows Graph::load_binary (src/matrix/graph.hpp:37-214) record by record,
// the per-tile dedup that keeps the first inserted triple
// (src/matrix/csc_matrix2d.hpp:62-72), the regular/sink/source/isolated
// classification (src/matrix/processed_matrix2d.hpp:203-228) and the locator
// order (src/utils/locator.h:84-155).  The reference builds one CSC per tile
// on the host with hash sets; here the records are transformed on the
// device, sorted (stable radix sort keeps insertion order among duplicates),
// deduplicated, ranked per class, and laid out as CSR arrays.
#include <sys/stat.h>

#include <algorithm>
#include <cstring>
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>

#include "la3g_internal.h"

namespace la3g {

struct IngestParams
{
  uint64_t N;            // nslots
  uint64_t invalid_key;  // N * N: dropped records sort last
  uint32_t nleft;        // bipartite column shift
  bool bipartite, directed, reverse, acyclic;
  Hasher h;
};

// One thread per record: graph.hpp:160-191.  Undirected records emit the
// edge and its mirror at slots 2i, 2i+1 (insertion order of the reference).
__global__ void k_transform(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, uint32_t stride,
                            uint64_t nrec, IngestParams P, uint64_t* __restrict__ keys,
                            uint32_t* __restrict__ vals, unsigned long long* bad)
{
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < nrec;
       i += (uint64_t) gridDim.x * blockDim.x)
  {
    uint32_t row = a[i * stride], col = b[i * stride];
    uint64_t k0 = P.invalid_key, k1 = P.invalid_key;
    if (P.bipartite) col += P.nleft;
    if (row != col)
    {
      if (P.directed && !P.reverse) { uint32_t t = row; row = col; col = t; }
      if (P.acyclic && ((!P.reverse && col > row) || (P.reverse && col < row))) { uint32_t t = row; row = col; col = t; }
      uint64_t hr = P.h.hash(row), hc = P.h.hash(col);
      if (hr >= P.N || hc >= P.N) atomicMin(bad, (unsigned long long) i);
      else { k0 = hr * P.N + hc; k1 = hc * P.N + hr; }
    }
    if (P.directed) { keys[i] = k0; vals[i] = (uint32_t) i; }
    else { keys[2 * i] = k0; vals[2 * i] = (uint32_t) i; keys[2 * i + 1] = k1; vals[2 * i + 1] = (uint32_t) i; }
  }
}

__global__ void k_mark(const uint64_t* __restrict__ keys, uint64_t m, uint64_t N, uint8_t* rowne, uint8_t* colne)
{
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t) gridDim.x * blockDim.x)
  {
    uint64_t k = keys[i];
    rowne[k / N] = 1;
    colne[k % N] = 1;
  }
}

__global__ void k_class_flags(uint32_t N, const uint8_t* rowne, const uint8_t* colne, uint32_t* f_reg,
                              uint32_t* f_sink, uint32_t* f_src)
{
  for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h < N; h += gridDim.x * blockDim.x)
  {
    uint8_t r = rowne[h], c = colne[h];
    f_reg[h] = r & c;
    f_sink[h] = r & !c;
    f_src[h] = !r & c;
  }
}

// Exclusive per-class ranks -> positions (regular, sink, source, rest).
__global__ void k_positions(uint32_t N, const uint8_t* rowne, const uint8_t* colne, const uint32_t* s_reg,
                            const uint32_t* s_sink, const uint32_t* s_src, uint32_t nreg, uint32_t nsink,
                            uint32_t nsrc, Hasher hs, uint32_t* hash_of_pos, uint32_t* pos_of_hash,
                            uint32_t* id_of_pos, uint32_t* pos_of_id)
{
  for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h < N; h += gridDim.x * blockDim.x)
  {
    uint8_t r = rowne[h], c = colne[h];
    uint32_t p;
    if (r & c) p = s_reg[h];
    else if (r) p = nreg + s_sink[h];
    else if (c) p = nreg + nsink + s_src[h];
    else p = nreg + nsink + nsrc + (h - s_reg[h] - s_sink[h] - s_src[h]);
    hash_of_pos[p] = h;
    pos_of_hash[h] = p;
    uint32_t id = hs.unhash(h);
    id_of_pos[p] = id;
    pos_of_id[id] = p;
  }
}

// (hashed row, hashed col) -> (row position, column key); the column key
// puts source columns before regular ones (process_ready_messages runs the
// source SpMV first, vertex_program_execute.hpp:479-482).
__global__ void k_pull_keys(const uint64_t* __restrict__ keys, uint64_t m, uint64_t N,
                            const uint32_t* __restrict__ pos_of_hash, uint32_t src_base, uint32_t nsrc,
                            uint64_t* __restrict__ out)
{
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t) gridDim.x * blockDim.x)
  {
    uint64_t k = keys[i];
    uint32_t rp = pos_of_hash[k / N], cp = pos_of_hash[k % N];
    uint32_t ck = cp >= src_base ? cp - src_base : cp + nsrc;
    out[i] = (uint64_t) rp * N + ck;
  }
}

__global__ void k_pull_fill(const uint64_t* __restrict__ k2, const uint32_t* __restrict__ vals, uint64_t m,
                            uint64_t N, uint32_t src_base, uint32_t nsrc, const uint32_t* __restrict__ wsrc,
                            uint32_t wstride, uint32_t* __restrict__ col, uint32_t* __restrict__ w)
{
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t) gridDim.x * blockDim.x)
  {
    uint32_t ck = (uint32_t) (k2[i] % N);
    col[i] = ck < nsrc ? src_base + ck : ck - nsrc;
    if (w) w[i] = wsrc[(uint64_t) vals[i] * wstride];
  }
}

// Row pointers from row-sorted keys: entry i writes ptr[q] = i for every
// row q in (row(i - 1), row(i)]; the virtual entry m closes the last rows.
__global__ void k_ptr_from_sorted(const uint64_t* __restrict__ k, uint64_t m, uint64_t N, uint32_t nrows_total,
                                  uint32_t* __restrict__ ptr)
{
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i <= m; i += (uint64_t) gridDim.x * blockDim.x)
  {
    int64_t r = i < m ? (int64_t) (k[i] / N) : (int64_t) nrows_total;
    int64_t rp = i == 0 ? -1 : (int64_t) (k[i - 1] / N);
    for (int64_t q = rp + 1; q <= r; q++) ptr[q] = (uint32_t) i;
  }
}

static int cub_sort_pairs(const uint64_t* kin, uint64_t* kout, const uint32_t* vin, uint32_t* vout, uint64_t n,
                          int end_bit, cudaStream_t s)
{
  size_t tb = 0;
  LA3G_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, kin, kout, vin, vout, n, 0, end_bit, s));
  DevBuf tmp;
  LA3G_TRY(tmp.alloc(tb));
  LA3G_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tb, kin, kout, vin, vout, n, 0, end_bit, s));
  return LA3G_OK;
}

static int bits_for(uint64_t v)
{
  int b = 0;
  while (b < 64 && (v >> b) != 0) b++;
  return b < 1 ? 1 : b;
}

// Builds the device graph from records already on the device.  `a`, `b`,
// `w` point at the src / dst / weight words with the given stride (3 or 2
// for on-disk records, 1 for separate arrays).
static int build_graph(la3g_graph* G, const uint32_t* a, const uint32_t* b, const uint32_t* w, uint32_t stride,
                       uint64_t nrec)
{
  DevGraph& g = G->g;
  cudaStream_t s = G->stream;
  const uint64_t N = g.nslots;
  if (N > (1ull << 31)) return set_error(LA3G_EINVAL, "too many vertices (%llu)", (unsigned long long) N);
  if (nrec >= (1ull << 32) - 1) return set_error(LA3G_EINVAL, "too many records");
  const bool directed = g.flags & LA3G_DIRECTED;
  const uint64_t m0 = directed ? nrec : 2 * nrec;
  IngestParams P;
  P.N = N;
  P.invalid_key = N * N;
  P.nleft = g.nleft;
  P.bipartite = g.flags & LA3G_BIPARTITE;
  P.directed = directed;
  P.reverse = g.flags & LA3G_REVERSE;
  P.acyclic = g.flags & LA3G_ACYCLIC;
  P.h = g.hasher;
  const int end_bit = bits_for(N * N);

  DevBuf keys, keys2, vals, vals2, bad, nsel;
  LA3G_TRY(keys.alloc(m0 * 8 + 8));
  LA3G_TRY(keys2.alloc(m0 * 8 + 8));
  LA3G_TRY(vals.alloc(m0 * 4 + 4));
  LA3G_TRY(vals2.alloc(m0 * 4 + 4));
  LA3G_TRY(bad.alloc(8));
  LA3G_TRY(nsel.alloc(8));
  LA3G_CUDA(cudaMemsetAsync(bad.p, 0xFF, 8, s));
  if (nrec)
  {
    k_transform<<<grid_for(nrec, 256), 256, 0, s>>>(a, b, stride, nrec, P, keys.as<uint64_t>(), vals.as<uint32_t>(),
                                                    bad.as<unsigned long long>());
    LA3G_LAUNCHED();
  }
  unsigned long long badi = ~0ull;
  LA3G_CUDA(cudaMemcpyAsync(&badi, bad.p, 8, cudaMemcpyDeviceToHost, s));
  LA3G_CUDA(cudaStreamSynchronize(s));
  if (badi != ~0ull)
    return set_error(LA3G_EINVAL, "record %llu: vertex id out of range for %llu slots", badi, (unsigned long long) N);

  // Stable sort by (row, col); the first of each run of equal keys wins.
  if (m0) LA3G_TRY(cub_sort_pairs(keys.as<uint64_t>(), keys2.as<uint64_t>(), vals.as<uint32_t>(), vals2.as<uint32_t>(), m0, end_bit, s));
  uint64_t mu = 0;
  if (m0)
  {
    size_t tb = 0;
    LA3G_CUDA(cub::DeviceSelect::UniqueByKey(nullptr, tb, keys2.as<uint64_t>(), vals2.as<uint32_t>(), keys.as<uint64_t>(),
                                             vals.as<uint32_t>(), nsel.as<unsigned long long>(), m0, s));
    DevBuf tmp;
    LA3G_TRY(tmp.alloc(tb));
    LA3G_CUDA(cub::DeviceSelect::UniqueByKey(tmp.p, tb, keys2.as<uint64_t>(), vals2.as<uint32_t>(), keys.as<uint64_t>(),
                                             vals.as<uint32_t>(), nsel.as<unsigned long long>(), m0, s));
    unsigned long long nu = 0, lastk = 0;
    LA3G_CUDA(cudaMemcpyAsync(&nu, nsel.p, 8, cudaMemcpyDeviceToHost, s));
    LA3G_CUDA(cudaStreamSynchronize(s));
    if (nu) LA3G_CUDA(cudaMemcpy(&lastk, keys.as<uint64_t>() + nu - 1, 8, cudaMemcpyDeviceToHost));
    mu = nu;
    if (nu && lastk == P.invalid_key) mu--;
  }
  if (mu >= (1ull << 32) - 1) return set_error(LA3G_EINVAL, "too many stored entries (%llu)", (unsigned long long) mu);
  g.nent = mu;
  uint64_t* ukeys = keys.as<uint64_t>();
  uint32_t* uvals = vals.as<uint32_t>();

  // Classes and positions.
  DevBuf rowne, colne, f0, f1, f2, s0, s1, s2;
  LA3G_TRY(rowne.alloc(N));
  LA3G_TRY(colne.alloc(N));
  LA3G_TRY(f0.alloc(N * 4 + 4));
  LA3G_TRY(f1.alloc(N * 4 + 4));
  LA3G_TRY(f2.alloc(N * 4 + 4));
  LA3G_TRY(s0.alloc(N * 4 + 4));
  LA3G_TRY(s1.alloc(N * 4 + 4));
  LA3G_TRY(s2.alloc(N * 4 + 4));
  LA3G_CUDA(cudaMemsetAsync(rowne.p, 0, N, s));
  LA3G_CUDA(cudaMemsetAsync(colne.p, 0, N, s));
  if (mu)
  {
    k_mark<<<grid_for(mu, 256), 256, 0, s>>>(ukeys, mu, N, rowne.as<uint8_t>(), colne.as<uint8_t>());
    LA3G_LAUNCHED();
  }
  k_class_flags<<<grid_for(N, 256), 256, 0, s>>>((uint32_t) N, rowne.as<uint8_t>(), colne.as<uint8_t>(), f0.as<uint32_t>(),
                                                 f1.as<uint32_t>(), f2.as<uint32_t>());
  LA3G_LAUNCHED();
  {
    size_t tb = 0;
    LA3G_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, f0.as<uint32_t>(), s0.as<uint32_t>(), N, s));
    DevBuf tmp;
    LA3G_TRY(tmp.alloc(tb));
    LA3G_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, tb, f0.as<uint32_t>(), s0.as<uint32_t>(), N, s));
    LA3G_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, tb, f1.as<uint32_t>(), s1.as<uint32_t>(), N, s));
    LA3G_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, tb, f2.as<uint32_t>(), s2.as<uint32_t>(), N, s));
  }
  uint32_t tail[6];
  LA3G_CUDA(cudaMemcpyAsync(&tail[0], s0.as<uint32_t>() + N - 1, 4, cudaMemcpyDeviceToHost, s));
  LA3G_CUDA(cudaMemcpyAsync(&tail[1], f0.as<uint32_t>() + N - 1, 4, cudaMemcpyDeviceToHost, s));
  LA3G_CUDA(cudaMemcpyAsync(&tail[2], s1.as<uint32_t>() + N - 1, 4, cudaMemcpyDeviceToHost, s));
  LA3G_CUDA(cudaMemcpyAsync(&tail[3], f1.as<uint32_t>() + N - 1, 4, cudaMemcpyDeviceToHost, s));
  LA3G_CUDA(cudaMemcpyAsync(&tail[4], s2.as<uint32_t>() + N - 1, 4, cudaMemcpyDeviceToHost, s));
  LA3G_CUDA(cudaMemcpyAsync(&tail[5], f2.as<uint32_t>() + N - 1, 4, cudaMemcpyDeviceToHost, s));
  LA3G_CUDA(cudaStreamSynchronize(s));
  g.nreg = tail[0] + tail[1];
  g.nsink = tail[2] + tail[3];
  g.nsrc = tail[4] + tail[5];

  uint32_t* pos_of_hash = f0.as<uint32_t>();  // reuse
  LA3G_TRY(galloc(G, &g.hash_of_pos, N));
  LA3G_TRY(galloc(G, &g.id_of_pos, N));
  LA3G_TRY(galloc(G, &g.pos_of_id, N));
  k_positions<<<grid_for(N, 256), 256, 0, s>>>((uint32_t) N, rowne.as<uint8_t>(), colne.as<uint8_t>(), s0.as<uint32_t>(),
                                               s1.as<uint32_t>(), s2.as<uint32_t>(), g.nreg, g.nsink, g.nsrc, g.hasher,
                                               g.hash_of_pos, pos_of_hash, g.id_of_pos, g.pos_of_id);
  LA3G_LAUNCHED();

  // Pull CSR.
  LA3G_TRY(galloc(G, &g.in_ptr, N + 1));
  LA3G_TRY(galloc(G, &g.in_col, mu + 1));
  if (g.weighted()) LA3G_TRY(galloc(G, &g.in_w, mu + 1));
  if (mu)
  {
    k_pull_keys<<<grid_for(mu, 256), 256, 0, s>>>(ukeys, mu, N, pos_of_hash, g.src_base(), g.nsrc, keys2.as<uint64_t>());
    LA3G_LAUNCHED();
    LA3G_TRY(cub_sort_pairs(keys2.as<uint64_t>(), ukeys, uvals, vals2.as<uint32_t>(), mu, end_bit, s));
    k_pull_fill<<<grid_for(mu, 256), 256, 0, s>>>(ukeys, vals2.as<uint32_t>(), mu, N, g.src_base(), g.nsrc,
                                                  w, stride, g.in_col, g.in_w);
    LA3G_LAUNCHED();
  }
  k_ptr_from_sorted<<<grid_for(mu + 1, 256), 256, 0, s>>>(ukeys, mu, N, (uint32_t) N, g.in_ptr);
  LA3G_LAUNCHED();
  if (!directed)
  {
    g.out_ptr = g.in_ptr;
    g.out_row = g.in_col;
    g.out_w = g.in_w;
  }
  LA3G_CUDA(cudaStreamSynchronize(s));
  return LA3G_OK;
}

// Push CSR for directed graphs: (column position, row position) sorted.
__global__ void k_expand_rows(const uint32_t* __restrict__ ptr, uint32_t nrows, uint32_t* __restrict__ row_of)
{
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x)
    for (uint32_t e = ptr[r]; e < ptr[r + 1]; e++) row_of[e] = r;
}

__global__ void k_push_keys(const uint32_t* __restrict__ row_of, const uint32_t* __restrict__ col, uint64_t m,
                            uint64_t N, uint64_t* __restrict__ out, uint32_t* __restrict__ idx)
{
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t) gridDim.x * blockDim.x)
  {
    out[i] = (uint64_t) col[i] * N + row_of[i];
    idx[i] = (uint32_t) i;
  }
}

__global__ void k_push_fill(const uint64_t* __restrict__ k, const uint32_t* __restrict__ idx, uint64_t m, uint64_t N,
                            const uint32_t* __restrict__ win, uint32_t* __restrict__ row, uint32_t* __restrict__ w)
{
  for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t) gridDim.x * blockDim.x)
  {
    row[i] = (uint32_t) (k[i] % N);
    if (w) w[i] = win[idx[i]];
  }
}

int build_push_csr(la3g_graph* G)
{
  DevGraph& g = G->g;
  if (g.out_ptr) return LA3G_OK;
  cudaStream_t s = G->stream;
  const uint64_t N = g.nslots, m = g.nent;
  LA3G_TRY(galloc(G, &g.out_ptr, N + 1));
  LA3G_TRY(galloc(G, &g.out_row, m + 1));
  if (g.weighted()) LA3G_TRY(galloc(G, &g.out_w, m + 1));
  DevBuf row_of, k, k2, idx, idx2;
  LA3G_TRY(row_of.alloc(m * 4 + 4));
  LA3G_TRY(k.alloc(m * 8 + 8));
  LA3G_TRY(k2.alloc(m * 8 + 8));
  LA3G_TRY(idx.alloc(m * 4 + 4));
  LA3G_TRY(idx2.alloc(m * 4 + 4));
  if (m)
  {
    k_expand_rows<<<grid_for(g.nrows(), 256), 256, 0, s>>>(g.in_ptr, g.nrows(), row_of.as<uint32_t>());
    LA3G_LAUNCHED();
    k_push_keys<<<grid_for(m, 256), 256, 0, s>>>(row_of.as<uint32_t>(), g.in_col, m, N, k.as<uint64_t>(), idx.as<uint32_t>());
    LA3G_LAUNCHED();
    LA3G_TRY(cub_sort_pairs(k.as<uint64_t>(), k2.as<uint64_t>(), idx.as<uint32_t>(), idx2.as<uint32_t>(), m, bits_for(N * N), s));
    k_push_fill<<<grid_for(m, 256), 256, 0, s>>>(k2.as<uint64_t>(), idx2.as<uint32_t>(), m, N, g.in_w, g.out_row, g.out_w);
    LA3G_LAUNCHED();
  }
  k_ptr_from_sorted<<<grid_for(m + 1, 256), 256, 0, s>>>(k2.as<uint64_t>(), m, N, (uint32_t) N, g.out_ptr);
  LA3G_LAUNCHED();
  LA3G_CUDA(cudaStreamSynchronize(s));
  return LA3G_OK;
}

static int new_graph(uint32_t n, uint32_t nright, uint32_t flags, la3g_graph** out, la3g_graph** G)
{
  *out = nullptr;
  la3g_graph* g = new (std::nothrow) la3g_graph();
  if (!g) return set_error(LA3G_ENOMEM, "out of host memory");
  if (cudaStreamCreateWithFlags(&g->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&g->ev0) != cudaSuccess || cudaEventCreate(&g->ev1) != cudaSuccess)
  {
    cudaError_t e = cudaGetLastError();
    la3g_graph_free(g);
    return set_error(LA3G_ECUDA, "cannot create a CUDA stream: %s", cudaGetErrorString(e));
  }
  g->stream = g->own_stream;
  DevGraph& d = g->g;
  const bool bip = flags & LA3G_BIPARTITE;
  d.flags = flags;
  d.nleft = n;
  d.nvertices = bip ? n + nright : n;
  d.nslots = d.nvertices + 1;  // tile_height = nrows / nrowgrps + 1 (matrix2d.hpp:8)
  d.hasher.null_hash = bip;
  if (!bip)
  {
    d.hasher.height = (uint64_t) d.nvertices / 128u;
    d.hasher.max_range = d.hasher.height * 128u;
  }
  *G = g;
  return LA3G_OK;
}

static bool check_flags(uint32_t flags)
{
  if (flags & ~0x1Fu) return false;
  if ((flags & LA3G_BIPARTITE) && (flags & LA3G_ACYCLIC)) return false;
  if (!(flags & LA3G_DIRECTED) && (flags & (LA3G_REVERSE | LA3G_ACYCLIC))) return false;
  return true;
}

}  // namespace la3g

using namespace la3g;

extern "C" void la3g_graph_free(la3g_graph* g)
{
  if (!g) return;
  if (g->stream) cudaStreamSynchronize(g->stream);
  if (g->own_stream && g->own_stream != g->stream) cudaStreamSynchronize(g->own_stream);
  for (int i = 0; i < kSlotCount; i++)
    if (g->slot[i] && g->slot_free[i]) g->slot_free[i](g->slot[i]);
  for (void* p : g->allocations) cudaFree(p);
  if (g->ev0) cudaEventDestroy(g->ev0);
  if (g->ev1) cudaEventDestroy(g->ev1);
  if (g->own_stream) cudaStreamDestroy(g->own_stream);
  delete g;
}

extern "C" int la3g_graph_set_stream(la3g_graph* g, void* cuda_stream)
{
  if (!g) return set_error(LA3G_EINVAL, "null graph");
  LA3G_CUDA(cudaStreamSynchronize(g->stream));
  g->stream = cuda_stream ? (cudaStream_t) cuda_stream : g->own_stream;
  return LA3G_OK;
}

extern "C" int la3g_graph_from_records(const void* records, uint64_t nrec, uint32_t n, uint32_t nright,
                                       uint32_t flags, la3g_graph** out)
{
  if (!out) return set_error(LA3G_EINVAL, "out is null");
  *out = nullptr;
  if (!check_flags(flags)) return set_error(LA3G_EINVAL, "invalid flag combination 0x%x", flags);
  if (n == 0) return set_error(LA3G_EINVAL, "n must be > 0 for in-memory records");
  if (nrec && !records) return set_error(LA3G_EINVAL, "records is null");
  la3g_graph* G = nullptr;
  LA3G_TRY(new_graph(n, nright, flags, out, &G));
  const uint32_t wpr = (flags & LA3G_WEIGHTED) ? 3 : 2;
  DevBuf rec;
  int rc = rec.alloc(nrec * wpr * 4 + 16);
  if (!rc && nrec)
  {
    cudaError_t e = cudaMemcpyAsync(rec.p, records, nrec * wpr * 4, cudaMemcpyHostToDevice, G->stream);
    if (e != cudaSuccess) rc = set_error(LA3G_ECUDA, "record upload failed: %s", cudaGetErrorString(e));
  }
  G->g.nrecords = nrec;
  if (!rc) rc = build_graph(G, rec.as<uint32_t>(), rec.as<uint32_t>() + 1, rec.as<uint32_t>() + 2, wpr, nrec);
  if (rc) { la3g_graph_free(G); return rc; }
  *out = G;
  return LA3G_OK;
}

extern "C" int la3g_graph_from_edges(const la3g_edges* e, uint32_t n, uint32_t nright, uint32_t flags,
                                     la3g_graph** out)
{
  if (!out || !e) return set_error(LA3G_EINVAL, "null argument");
  *out = nullptr;
  if (!check_flags(flags)) return set_error(LA3G_EINVAL, "invalid flag combination 0x%x", flags);
  if ((flags & LA3G_WEIGHTED) && !e->w) return set_error(LA3G_EINVAL, "weighted load of an unweighted edge list");
  if (n == 0) { n = e->n; nright = e->nright; }
  la3g_graph* G = nullptr;
  LA3G_TRY(new_graph(n, nright, flags, out, &G));
  const uint64_t m = e->m;
  DevBuf a, b, w;
  int rc = a.alloc(m * 4 + 16);
  if (!rc) rc = b.alloc(m * 4 + 16);
  if (!rc && (flags & LA3G_WEIGHTED)) rc = w.alloc(m * 4 + 16);
  if (!rc && m)
  {
    cudaError_t c = cudaMemcpyAsync(a.p, e->src, m * 4, cudaMemcpyHostToDevice, G->stream);
    if (c == cudaSuccess) c = cudaMemcpyAsync(b.p, e->dst, m * 4, cudaMemcpyHostToDevice, G->stream);
    if (c == cudaSuccess && (flags & LA3G_WEIGHTED)) c = cudaMemcpyAsync(w.p, e->w, m * 4, cudaMemcpyHostToDevice, G->stream);
    if (c != cudaSuccess) rc = set_error(LA3G_ECUDA, "edge upload failed: %s", cudaGetErrorString(c));
  }
  G->g.nrecords = m;
  if (!rc) rc = build_graph(G, a.as<uint32_t>(), b.as<uint32_t>(), w.as<uint32_t>(), 1, m);
  if (rc) { la3g_graph_free(G); return rc; }
  *out = G;
  return LA3G_OK;
}

extern "C" int la3g_graph_load(const char* path, uint32_t n, uint32_t nright, uint32_t flags, la3g_graph** out)
{
  if (!out || !path) return set_error(LA3G_EINVAL, "null argument");
  *out = nullptr;
  if (!check_flags(flags)) return set_error(LA3G_EINVAL, "invalid flag combination 0x%x", flags);
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_error(LA3G_EIO, "cannot open %s", path);
  struct stat st;
  if (fstat(fileno(f), &st) != 0) { std::fclose(f); return set_error(LA3G_EIO, "cannot stat %s", path); }
  uint64_t size = (uint64_t) st.st_size, offset = 0;
  const uint32_t wpr = (flags & LA3G_WEIGHTED) ? 3 : 2;
  if (n == 0)
  {
    // 16-byte header {u32 n-1, u32 m-1, u64 nnz} (graph.hpp:207-235).  The
    // vertex count is taken from it for every graph kind.
    uint32_t h[4];
    if (std::fread(h, 16, 1, f) != 1) { std::fclose(f); return set_error(LA3G_EFORMAT, "%s: short header", path); }
    n = h[0] + 1;
    if (flags & LA3G_BIPARTITE) nright = h[1] + 1;
    offset = 16;
  }
  if ((size - offset) % (wpr * 4) != 0)
  {
    std::fclose(f);
    return set_error(LA3G_EFORMAT, "%s: %llu bytes is not a whole number of %u-byte records", path,
                     (unsigned long long) (size - offset), wpr * 4);
  }
  const uint64_t nrec = (size - offset) / (wpr * 4);
  la3g_graph* G = nullptr;
  int rc = new_graph(n, nright, flags, out, &G);
  if (rc) { std::fclose(f); return rc; }
  DevBuf rec;
  rc = rec.alloc(nrec * wpr * 4 + 16);
  // Stream the file through a pinned staging buffer.
  const size_t chunk = 64u << 20;
  void* stage = nullptr;
  if (!rc && cudaHostAlloc(&stage, chunk, cudaHostAllocDefault) != cudaSuccess)
  {
    cudaGetLastError();
    stage = nullptr;
    rc = set_error(LA3G_ENOMEM, "cannot allocate pinned staging memory");
  }
  uint64_t done = 0, total = nrec * wpr * 4;
  while (!rc && done < total)
  {
    size_t want = (size_t) std::min<uint64_t>(chunk, total - done);
    if (std::fread(stage, 1, want, f) != want) { rc = set_error(LA3G_EIO, "%s: short read", path); break; }
    cudaError_t e = cudaMemcpy((char*) rec.p + done, stage, want, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) rc = set_error(LA3G_ECUDA, "upload failed: %s", cudaGetErrorString(e));
    done += want;
  }
  if (stage) cudaFreeHost(stage);
  std::fclose(f);
  if (!rc)
  {
    G->g.nrecords = nrec;
    rc = build_graph(G, rec.as<uint32_t>(), rec.as<uint32_t>() + 1, rec.as<uint32_t>() + 2, wpr, nrec);
  }
  if (rc) { la3g_graph_free(G); return rc; }
  *out = G;
  return LA3G_OK;
}

extern "C" int la3g_graph_info_get(const la3g_graph* G, la3g_graph_info* out)
{
  if (!G || !out) return set_error(LA3G_EINVAL, "null argument");
  const DevGraph& g = G->g;
  std::memset(out, 0, sizeof *out);
  out->nslots = g.nslots;
  out->nvertices = g.nvertices;
  out->nleft = g.nleft;
  out->flags = g.flags;
  out->nrecords = g.nrecords;
  out->nentries = g.nent;
  out->nregular = g.nreg;
  out->nsink = g.nsink;
  out->nsource = g.nsrc;
  out->nisolated = g.nslots - g.nreg - g.nsink - g.nsrc;
  out->device_bytes = G->device_bytes;
  return LA3G_OK;
}

extern "C" int la3g_graph_positions(const la3g_graph* G, uint32_t* pos_of_id, uint32_t* id_of_pos)
{
  if (!G) return set_error(LA3G_EINVAL, "null graph");
  const DevGraph& g = G->g;
  if (pos_of_id) LA3G_CUDA(cudaMemcpy(pos_of_id, g.pos_of_id, (size_t) g.nslots * 4, cudaMemcpyDeviceToHost));
  if (id_of_pos) LA3G_CUDA(cudaMemcpy(id_of_pos, g.id_of_pos, (size_t) g.nslots * 4, cudaMemcpyDeviceToHost));
  return LA3G_OK;
}

extern "C" int la3g_graph_device_view(la3g_graph* G, la3g_device_graph* out)
{
  if (!G || !out) return set_error(LA3G_EINVAL, "null graph or output");
  const DevGraph& g = G->g;
  std::memset(out, 0, sizeof(*out));
  out->row_ptr = g.in_ptr;
  out->col = g.in_col;
  out->weight = g.weighted() ? g.in_w : nullptr;
  out->hash_of_pos = g.hash_of_pos;
  out->id_of_pos = g.id_of_pos;
  out->pos_of_id = g.pos_of_id;
  out->nslots = g.nslots;
  out->nregular = g.nreg;
  out->nsink = g.nsink;
  out->nsource = g.nsrc;
  out->flags = g.flags;
  out->nentries = g.nent;
  out->stream = (void*) G->stream;
  return LA3G_OK;
}

extern "C" int la3g_graph_push_view(la3g_graph* G, const uint32_t** out_ptr, const uint32_t** out_row)
{
  if (!G || !out_ptr || !out_row) return set_error(LA3G_EINVAL, "null graph or output");
  const DevGraph& g = G->g;
  if (g.directed()) LA3G_TRY(build_push_csr(G));
  *out_ptr = g.directed() ? g.out_ptr : g.in_ptr;
  *out_row = g.directed() ? g.out_row : g.in_col;
  return LA3G_OK;
}
