// Internal declarations shared by the library's translation units.
#ifndef LA3G_INTERNAL_H
#define LA3G_INTERNAL_H

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "la3g.h"

#ifdef __CUDACC__
#include <cuda_runtime.h>
#endif

namespace la3g {

// Records `code` and a printf-style message as the thread's last error and
// returns `code`.
int set_error(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
unsigned host_threads();

// Hashing of vertex ids: SimpleBucketHasher at one rank
// (src/matrix/hashers.h:39-68) or the identity (NullHasher) for bipartite
// graphs.
struct Hasher
{
  uint64_t height = 0, max_range = 0;
  bool null_hash = false;
#ifdef __CUDACC__
  __host__ __device__
#endif
  inline uint32_t hash(uint64_t v) const
  {
    if (null_hash || v >= max_range) return (uint32_t) v;
    return (uint32_t) (v / 128u + ((uint32_t) v % 128u) * height);
  }
#ifdef __CUDACC__
  __host__ __device__
#endif
  inline uint32_t unhash(uint64_t v) const
  {
    if (null_hash || v >= max_range) return (uint32_t) v;
    return (uint32_t) (v / height + (v % height) * 128u);
  }
};

}  // namespace la3g

#ifdef __CUDACC__

namespace la3g {

#define LA3G_CUDA(call)                                                                         \
  do {                                                                                          \
    cudaError_t err_ = (call);                                                                  \
    if (err_ != cudaSuccess)                                                                    \
      return ::la3g::set_error(LA3G_ECUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call,           \
                               cudaGetErrorString(err_));                                       \
  } while (0)

#define LA3G_TRY(expr)                \
  do {                                \
    int rc_ = (expr);                 \
    if (rc_ != LA3G_OK) return rc_;   \
  } while (0)

// Checks the launch that was just made (configuration errors only; the
// kernel itself is checked at the next synchronisation).
#define LA3G_LAUNCHED() LA3G_CUDA(cudaGetLastError())

// Streaming multiprocessors of the current device (152 on a GB300: 2 dies
// x 76), queried once per device; grid sizes are multiples of it.
int num_sms();

inline unsigned grid_for(uint64_t n, unsigned block, unsigned max_blocks = num_sms() * 16)
{
  uint64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > max_blocks) g = max_blocks;
  return (unsigned) g;
}

// Block-wide reductions for kernels that add their partial counts into one
// global counter: one atomic per block instead of one per warp (thousands of
// same-address atomics serialise in L2).  Every thread of the block must
// call them; the result is valid in thread 0.
__device__ __forceinline__ unsigned long long block_sum_u64(unsigned long long v)
{
  __shared__ unsigned long long s_part[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();  // s_part may still be read from a previous call
  if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32)
  {
    v = threadIdx.x < (blockDim.x + 31) / 32 ? s_part[threadIdx.x] : 0ull;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  }
  return v;
}

__device__ __forceinline__ uint32_t block_min_u32(uint32_t v)
{
  __shared__ uint32_t s_part[32];
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32)
  {
    v = threadIdx.x < (blockDim.x + 31) / 32 ? s_part[threadIdx.x] : 0xFFFFFFFFu;
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  }
  return v;
}

// Kernel-level profiling: when on, a launch is bracketed by events on its
// stream and its time accumulated under `name` with `bytes` algorithmic
// bytes.  Always counts the launch.
struct ProfileScope
{
  const char* name;
  cudaStream_t stream;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double bytes;
  ProfileScope(const char* name, cudaStream_t s, double bytes);
  ~ProfileScope();
};

// Adds algorithmic bytes to a kernel's profile entry when they are known
// only after its launches (e.g. from a count the kernels produced).
void profile_add_bytes(const char* name, double bytes);

extern thread_local uint32_t tls_launches;

// Scoped device buffer for temporaries.
struct DevBuf
{
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { if (p) cudaFree(p); }
  int alloc(size_t n)
  {
    if (n <= bytes && p) return LA3G_OK;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, n ? n : 16);
    if (e != cudaSuccess)
    {
      cudaGetLastError();
      p = nullptr;
      return set_error(LA3G_ENOMEM, "device allocation of %zu bytes failed: %s", n, cudaGetErrorString(e));
    }
    bytes = n;
    return LA3G_OK;
  }
  template <class T>
  T* as() const { return (T*) p; }
};

// The device image of a graph in internal order.
struct DevGraph
{
  uint32_t flags = 0;
  uint32_t nvertices = 0, nslots = 0, nleft = 0;
  uint64_t nrecords = 0, nent = 0;
  uint32_t nreg = 0, nsink = 0, nsrc = 0;
  Hasher hasher;
  bool directed() const { return flags & LA3G_DIRECTED; }
  bool weighted() const { return flags & LA3G_WEIGHTED; }
  uint32_t src_base() const { return nreg + nsink; }
  uint32_t iso_base() const { return nreg + nsink + nsrc; }
  uint32_t nrows() const { return nreg + nsink; }

  uint32_t* id_of_pos = nullptr;    // [nslots] original id of each position
  uint32_t* pos_of_id = nullptr;    // [nslots]
  uint32_t* hash_of_pos = nullptr;  // [nslots] hashed id (Edge::src / Edge::dst)

  // Pull CSR over rows = positions [0, nreg + nsink): in-neighbours (column
  // positions) in the reference's order: source columns first, then regular
  // columns, each ascending.  For undirected graphs this is the only CSR.
  uint32_t* in_ptr = nullptr;  // [nslots + 1]
  uint32_t* in_col = nullptr;  // [nent]
  uint32_t* in_w = nullptr;    // [nent] when weighted

  // Push CSR over columns = positions: out-neighbours (row positions),
  // ascending, so regular rows come before sink rows.  Built on demand for
  // directed graphs; the same arrays as the pull CSR for undirected graphs.
  uint32_t* out_ptr = nullptr;  // [nslots + 1]
  uint32_t* out_row = nullptr;
  uint32_t* out_w = nullptr;
};

// Per-app device scratch cached on a graph handle (allocated on first use).
enum AppSlot { kSlotPr = 0, kSlotBfs, kSlotSssp, kSlotCc, kSlotTc, kSlotBm25, kSlotBatch, kSlotVp, kSlotLm, kSlotCount };

}  // namespace la3g

struct la3g_graph
{
  la3g::DevGraph g;
  cudaStream_t stream = nullptr;       // stream the calls run on
  cudaStream_t own_stream = nullptr;   // the graph's own stream
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<void*> allocations;
  uint64_t device_bytes = 0;
  void* slot[la3g::kSlotCount] = {};
  void (*slot_free[la3g::kSlotCount])(void*) = {};
};

namespace la3g {

// Graph-owned device allocation (freed by la3g_graph_free).
int galloc_bytes(la3g_graph* G, void** p, size_t bytes);
template <class T>
int galloc(la3g_graph* G, T** p, size_t count)
{
  return galloc_bytes(G, (void**) p, count * sizeof(T));
}

int build_push_csr(la3g_graph* G);
// Bipartite corpus: the position of the first term row (docs come first).
int bipartite_first_term_row(la3g_graph* G, uint32_t* out);

// Bracket an app call: events on the graph's stream and the host clock.
struct CallTimer
{
  la3g_graph* G;
  la3g_stats* st;
  double t0;
  uint32_t launches0;
  CallTimer(la3g_graph* G, la3g_stats* st);
  void device_begin();
  void device_end();
  int finish();  // synchronises and fills st
};

double now_ms();

// True while kernel-level profiling is on (la3g_profile_enable).
bool profile_enabled();

// An iteration loop that runs on the device: one CUDA graph holding
//   while (cont) { decide; switch (mode) { body[0] ... body[n-1] } }
// The decide kernel reads the loop state the previous iteration left in
// device memory, picks the next body (push or pull, top-down or bottom-up,
// the ping-pong parity of the frontier buffers) and ends the loop, all with
// `cudaGraphSetConditional`; the host launches the graph once per call and
// synchronises once at the end.  The same decide kernel and bodies also run
// host-stepped (one mode read back per iteration) when profiling is on,
// since event-timed scopes cannot sit inside a conditional body.
struct DeviceLoop
{
  cudaGraphExec_t exec = nullptr;
  cudaGraphConditionalHandle cont = 0, mode = 0;
  int nbodies = 0;
  uint32_t body_launches[16] = {};  // kernels one pass through each body launches
  ~DeviceLoop();
};

// Builds `L`: `decide(cap, cont, mode)` enqueues the decide kernel on the
// capture stream, `body(cap, k)` enqueues body k's kernels and memsets.
template <class Decide, class Body>
int device_loop_build(DeviceLoop* L, int nbodies, Decide&& decide, Body&& body);

// Kernels of the loop state call this to end or steer the loop; in the
// host-stepped form (handles 0) nothing is set and the host reads the state.
__device__ __forceinline__ void loop_set(cudaGraphConditionalHandle h, unsigned v)
{
  if (h) cudaGraphSetConditional(h, v);
}

template <class Decide, class Body>
int device_loop_build(DeviceLoop* L, int nbodies, Decide&& decide, Body&& body)
{
  if (nbodies > 16) return set_error(LA3G_EINVAL, "device loop with %d bodies", nbodies);
  cudaGraph_t graph = nullptr;
  cudaStream_t cap = nullptr;
  const uint32_t launches0 = tls_launches;
  int rc = LA3G_OK;
  auto fail = [&](cudaError_t e) {
    if (e == cudaSuccess) return false;
    cudaGetLastError();
    rc = set_error(LA3G_ECUDA, "device loop graph: %s", cudaGetErrorString(e));
    return true;
  };
  do
  {
    if (fail(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking))) break;
    if (fail(cudaGraphCreate(&graph, 0))) break;
    if (fail(cudaGraphConditionalHandleCreate(&L->cont, graph, 1, cudaGraphCondAssignDefault))) break;
    if (fail(cudaGraphConditionalHandleCreate(&L->mode, graph, 0, cudaGraphCondAssignDefault))) break;
    cudaGraphNodeParams wp = {};
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = L->cont;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wnode;
    if (fail(cudaGraphAddNode(&wnode, graph, nullptr, nullptr, 0, &wp))) break;
    cudaGraph_t wbody = wp.conditional.phGraph_out[0];
    // the decide kernel, then the switch over the bodies
    if (fail(cudaStreamBeginCaptureToGraph(cap, wbody, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal))) break;
    rc = decide(cap, L->cont, L->mode);
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    if (rc == LA3G_OK && fail(cudaStreamGetCaptureInfo(cap, &cs, nullptr, nullptr, &deps, nullptr, &ndeps))) {}
    cudaGraphNode_t dnode = ndeps ? deps[0] : nullptr;
    cudaGraph_t dummy = nullptr;
    if (fail(cudaStreamEndCapture(cap, &dummy)) || rc != LA3G_OK || ndeps != 1) 
    {
      if (rc == LA3G_OK) rc = set_error(LA3G_ECUDA, "device loop graph: decide step is not one node");
      break;
    }
    cudaGraphNodeParams sp = {};
    sp.type = cudaGraphNodeTypeConditional;
    sp.conditional.handle = L->mode;
    sp.conditional.type = cudaGraphCondTypeSwitch;
    sp.conditional.size = (unsigned) nbodies;
    cudaGraphNode_t snode;
    if (fail(cudaGraphAddNode(&snode, wbody, &dnode, nullptr, 1, &sp))) break;
    for (int k = 0; k < nbodies && rc == LA3G_OK; k++)
    {
      if (fail(cudaStreamBeginCaptureToGraph(cap, sp.conditional.phGraph_out[k], nullptr, nullptr, 0,
                                             cudaStreamCaptureModeThreadLocal)))
        break;
      const uint32_t before = tls_launches;
      rc = body(cap, k);
      L->body_launches[k] = tls_launches - before;
      cudaGraph_t out = nullptr;
      if (fail(cudaStreamEndCapture(cap, &out))) break;
    }
    if (rc != LA3G_OK) break;
    if (fail(cudaGraphInstantiate(&L->exec, graph, 0))) break;
    L->nbodies = nbodies;
  } while (0);
  tls_launches = launches0;
  if (graph) cudaGraphDestroy(graph);
  if (cap) cudaStreamDestroy(cap);
  return rc;
}

}  // namespace la3g

#endif  // __CUDACC__

#endif
