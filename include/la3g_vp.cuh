/* la3g_vp.cuh: the vertex-program API as device functor templates.
 *
 * This is the plugin interface of the reference, VertexProgram<W, M, A, S>
 * (src/vprogram/vertex_program.h:99-180), re-expressed for the GPU: a user
 * program is a plain struct whose callbacks are __device__ member functions,
 * and Engine<Program> runs the reference's BSP loop over a graph loaded by
 * libla3g (la3g_graph_device_view).  Kernels are instantiated per program, so
 * no callback is dispatched indirectly.
 *
 * A program provides (types trivially copyable):
 *
 *   struct MyProgram {
 *     using Msg = ...; using Acc = ...; using State = ...;
 *     static constexpr bool stationary = ...;         // VertexProgram::stationary
 *     static constexpr bool gather_with_state = ...;  // gather(edge, msg, state) overridden
 *     static constexpr bool apply_with_iteration = ...;  // apply(y, state, iter) overridden
 *     __device__ bool  init(uint32_t vid, State& s) const;          // init(vid, s) -> activate
 *     __device__ Msg   scatter(const State& s) const;
 *     __device__ Acc   gather(const la3g_vp::Edge& e, const Msg& m, const State& row_state) const;
 *     __device__ void  combine(const Acc& y1, Acc& y2) const;      // y2 = y1 (+) y2
 *     __device__ bool  apply(const Acc& y, State& s, uint32_t iter) const;
 *     __device__ Acc   zero() const;                                // A()
 *   };
 *
 * Semantics kept from the reference (vertex_program_execute.hpp:11-724):
 *   - Edge{src, dst, weight}: src / dst are the hashed ids of the column
 *     and row vertex (types.h:29-40);
 *   - each row's accumulator starts at zero() and takes
 *     combine(gather(edge, msg), acc) for its active in-neighbours in the
 *     SpMV's order (source columns first, then regular, each ascending), one
 *     edge after another: combine need not be associative or commutative;
 *   - a touched row applies combine(acc, zero()); activated regular rows (all
 *     touched rows when stationary) scatter into the next iteration;
 *   - regular rows take the sources' messages in the first iteration only
 *     (every iteration when stationary), sink rows in every iteration;
 *   - directed programs without gather_with_state / apply_with_iteration
 *     ("optimizable", vertex_program.hpp:77) leave sinks out of the
 *     iterations and compute them once afterwards from every regular
 *     vertex's final scatter; the others process sinks every iteration;
 *   - gather_with_state reads the states as they were at initialize (of the
 *     vertices that were activated then, all of them when stationary; the
 *     others read a zero state), as the reference's mirrors do;
 *   - execute(0) runs until no regular vertex activates; execute(1) is the
 *     single-iteration variant (no scatter after apply).
 *
 * Engine methods return LA3G_OK or an la3g_status; error_string() says why.
 * An engine is bound to its graph's stream; it is not re-entrant.
 */
#ifndef LA3G_VP_CUH
#define LA3G_VP_CUH

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "la3g.h"

namespace la3g_vp {

struct Edge
{
  uint32_t src, dst, weight;
};

namespace detail {

struct View
{
  const uint32_t* row_ptr;
  const uint32_t* col;
  const uint32_t* weight;
  const uint32_t* hash_of_pos;
  uint32_t nreg, nsink, src_base, iso_base;
};

template <class P>
__global__ void k_init(P prog, View g, uint32_t nslots, bool directed, typename P::State* S,
                       typename P::Msg* xr, uint8_t* xr_act, typename P::Msg* xs, uint8_t* xs_act,
                       const uint32_t* id_of_pos, uint8_t* active)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < nslots; p += gridDim.x * blockDim.x)
  {
    typename P::State s{};
    const bool act = prog.init(id_of_pos[p], s);
    S[p] = s;
    active[p] = act ? 1 : 0;
    if (!act) continue;
    if (p < g.nreg)
    {
      xr[p] = prog.scatter(s);
      xr_act[p] = 1;
    }
    else if (directed && p >= g.src_base && p < g.iso_base)
    {
      xs[p - g.src_base] = prog.scatter(s);
      xs_act[p - g.src_base] = 1;
    }
  }
}

template <class P>
__global__ void k_mirror(uint32_t nslots, const typename P::State* S, const uint8_t* active,
                         typename P::State* mirror)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < nslots; p += gridDim.x * blockDim.x)
  {
    typename P::State z;
    memset(&z, 0, sizeof z);  // mirrors of vertices not active at initialize read zero bytes
    mirror[p] = (P::stationary || active[p]) ? S[p] : z;
  }
}

// One thread per row: the row's in-edges in order, then apply.  Rows in
// [row_lo, row_hi); sources' messages are read when with_sources.
template <class P>
__global__ void k_row_pass(P prog, View g, uint32_t row_lo, uint32_t row_hi, bool with_sources, bool single_iter,
                           uint32_t iter, typename P::State* S, const typename P::State* mirror,
                           const typename P::Msg* xr, const uint8_t* xr_act, const typename P::Msg* xs,
                           const uint8_t* xs_act, typename P::Msg* xr_next, uint8_t* xr_next_act, int* any)
{
  for (uint32_t r = row_lo + blockIdx.x * blockDim.x + threadIdx.x; r < row_hi; r += gridDim.x * blockDim.x)
  {
    typename P::Acc acc = prog.zero();
    bool touched = false;
    const uint32_t dst = g.hash_of_pos[r];
    typename P::State zs{};
    const typename P::State& rs = P::gather_with_state ? mirror[r] : zs;
    for (uint32_t e = g.row_ptr[r]; e < g.row_ptr[r + 1]; e++)
    {
      const uint32_t c = g.col[e];
      const typename P::Msg* m;
      if (c >= g.src_base)
      {
        if (!with_sources || !xs_act[c - g.src_base]) continue;
        m = &xs[c - g.src_base];
      }
      else
      {
        if (!xr_act[c]) continue;
        m = &xr[c];
      }
      const Edge ed{g.hash_of_pos[c], dst, g.weight ? g.weight[e] : 0u};
      prog.combine(prog.gather(ed, *m, rs), acc);
      touched = true;
    }
    if (!touched) continue;
    typename P::Acc fin = prog.zero();
    prog.combine(acc, fin);
    const bool act = prog.apply(fin, S[r], iter);
    if (r >= g.nreg) continue;  // sink activations do not count
    if (act) *any = 1;
    if ((act || P::stationary) && !single_iter)
    {
      xr_next[r] = prog.scatter(S[r]);
      xr_next_act[r] = 1;
    }
  }
}

template <class P>
__global__ void k_scatter_all(P prog, uint32_t nreg, const typename P::State* S, typename P::Msg* xr, uint8_t* act)
{
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < nreg; r += gridDim.x * blockDim.x)
  {
    xr[r] = prog.scatter(S[r]);
    act[r] = 1;
  }
}

template <class T>
__global__ void k_by_id(uint32_t n, const uint32_t* id_of_pos, const T* in, T* out)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) out[id_of_pos[p]] = in[p];
}

// Blocks of 256 threads for n items, at most 16 per streaming multiprocessor
// of the current device.
inline unsigned blocks_for(uint64_t n)
{
  static thread_local int sms = 0;
  if (!sms)
  {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        sms <= 0)
    {
      cudaGetLastError();
      sms = 152;
    }
  }
  const uint64_t cap = (uint64_t) sms * 16;
  uint64_t b = (n + 255) / 256;
  return (unsigned) (b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace detail

template <class P>
class Engine
{
 public:
  using Msg = typename P::Msg;
  using Acc = typename P::Acc;
  using State = typename P::State;

  Engine(la3g_graph* g, const P& prog) : prog_(prog)
  {
    if (la3g_graph_device_view(g, &dv_) != LA3G_OK)
    {
      fail(LA3G_EINVAL, "graph view unavailable");
      return;
    }
    s_ = (cudaStream_t) dv_.stream;
    directed_ = dv_.flags & LA3G_DIRECTED;
    v_ = detail::View{dv_.row_ptr, dv_.col, dv_.weight, dv_.hash_of_pos, dv_.nregular, dv_.nsink,
                      dv_.nregular + dv_.nsink, dv_.nregular + dv_.nsink + dv_.nsource};
    const uint32_t N = dv_.nslots;
    alloc(&S_, (size_t) N * sizeof(State));
    alloc(&mirror_, P::gather_with_state ? (size_t) N * sizeof(State) : 16);
    alloc(&xr_[0], (size_t) (dv_.nregular + 1) * sizeof(Msg));
    alloc(&xr_[1], (size_t) (dv_.nregular + 1) * sizeof(Msg));
    alloc(&xra_[0], dv_.nregular + 1);
    alloc(&xra_[1], dv_.nregular + 1);
    alloc(&xs_, (size_t) (dv_.nsource + 1) * sizeof(Msg));
    alloc(&xsa_, dv_.nsource + 1);
    alloc(&active_, N);
    alloc(&any_, sizeof(int));
  }

  ~Engine()
  {
    for (void* p : owned_) cudaFree(p);
  }

  Engine(const Engine&) = delete;
  Engine& operator=(const Engine&) = delete;

  // initialize() (vertex_program.hpp:84-174): init on every vertex.
  int initialize()
  {
    if (status_ != LA3G_OK) return status_;
    const uint32_t N = dv_.nslots;
    cur_ = 0;
    ck(cudaMemsetAsync(xra_[0], 0, dv_.nregular + 1, s_));
    ck(cudaMemsetAsync(xsa_, 0, dv_.nsource + 1, s_));
    detail::k_init<P><<<detail::blocks_for(N), 256, 0, s_>>>(prog_, v_, N, directed_, (State*) S_, (Msg*) xr_[0],
                                                             (uint8_t*) xra_[0], (Msg*) xs_, (uint8_t*) xsa_,
                                                             dv_.id_of_pos, (uint8_t*) active_);
    ck(cudaGetLastError());
    if (P::gather_with_state && !mirrored_)
    {
      detail::k_mirror<P><<<detail::blocks_for(N), 256, 0, s_>>>(N, (const State*) S_, (const uint8_t*) active_,
                                                                 (State*) mirror_);
      ck(cudaGetLastError());
      mirrored_ = true;
    }
    return sync();
  }

  // execute(num_iterations) (vertex_program_execute.hpp:11-52); 0 = until
  // no regular vertex activates.  *iters_out = iterations run.
  int execute(uint32_t max_iters, uint32_t* iters_out = nullptr)
  {
    if (status_ != LA3G_OK) return status_;
    const bool optimizable = directed_ && !P::gather_with_state && !P::apply_with_iteration;
    const uint32_t nreg = dv_.nregular, nrows = dv_.nregular + dv_.nsink;
    uint32_t it = 0;
    if (max_iters == 1)
    {
      // execute_single (:251-345): regular rows, then sinks; no scatter
      pass(0, nreg, true, true, 0);
      if (directed_ && dv_.nsink) pass(nreg, nrows, true, true, 0);
      it = 1;
    }
    else
    {
      const bool until = max_iters == 0;
      for (;;)
      {
        if (!until && it >= max_iters) break;
        ck(cudaMemsetAsync(any_, 0, sizeof(int), s_));
        const bool with_src = P::stationary || it == 0;
        ck(cudaMemsetAsync(xra_[cur_ ^ 1], 0, nreg + 1, s_));
        pass(0, nreg, with_src, false, it);
        // sink rows take the sources' messages in every iteration
        // (vertex_program_execute.hpp:464-468)
        if (!optimizable && directed_ && dv_.nsink) pass(nreg, nrows, true, false, it);
        cur_ ^= 1;
        it++;
        int any = 0;
        ck(cudaMemcpyAsync(&any, any_, sizeof(int), cudaMemcpyDeviceToHost, s_));
        if (sync() != LA3G_OK) return status_;
        if (until && !any) break;
        if (it > 100000000u) return fail(LA3G_ETIMEOUT, "execute did not converge");
      }
      if (optimizable && dv_.nsink)
      {
        // sinks once (:131-148): every regular vertex scatters its final
        // state; sources' messages as they stand
        detail::k_scatter_all<P><<<detail::blocks_for(nreg), 256, 0, s_>>>(prog_, nreg, (const State*) S_,
                                                                          (Msg*) xr_[cur_], (uint8_t*) xra_[cur_]);
        ck(cudaGetLastError());
        pass(nreg, nrows, true, false, it);
      }
    }
    if (iters_out) *iters_out = it;
    return sync();
  }

  // States by original vertex id (nslots entries).
  int states(State* host_out)
  {
    if (status_ != LA3G_OK) return status_;
    void* tmp = nullptr;
    if (cudaMalloc(&tmp, (size_t) dv_.nslots * sizeof(State)) != cudaSuccess) return fail(LA3G_ENOMEM, "states");
    detail::k_by_id<State><<<detail::blocks_for(dv_.nslots), 256, 0, s_>>>(dv_.nslots, dv_.id_of_pos,
                                                                           (const State*) S_, (State*) tmp);
    ck(cudaGetLastError());
    ck(cudaMemcpyAsync(host_out, tmp, (size_t) dv_.nslots * sizeof(State), cudaMemcpyDeviceToHost, s_));
    const int st = sync();
    cudaFree(tmp);
    return st;
  }

  // Device states by position (la3g_graph_positions order).
  State* device_states() { return (State*) S_; }
  const la3g_device_graph& view() const { return dv_; }
  int status() const { return status_; }
  const char* error_string() const { return msg_; }

 private:
  void pass(uint32_t lo, uint32_t hi, bool with_src, bool single, uint32_t iter)
  {
    if (hi <= lo) return;
    detail::k_row_pass<P><<<detail::blocks_for(hi - lo), 256, 0, s_>>>(
        prog_, v_, lo, hi, with_src, single, iter, (State*) S_, (const State*) mirror_, (const Msg*) xr_[cur_],
        (const uint8_t*) xra_[cur_], (const Msg*) xs_, (const uint8_t*) xsa_, (Msg*) xr_[cur_ ^ 1],
        (uint8_t*) xra_[cur_ ^ 1], (int*) any_);
    ck(cudaGetLastError());
  }

  void alloc(void** p, size_t bytes)
  {
    if (status_ != LA3G_OK) return;
    if (cudaMalloc(p, bytes ? bytes : 16) != cudaSuccess)
    {
      cudaGetLastError();
      *p = nullptr;
      fail(LA3G_ENOMEM, "device allocation failed");
      return;
    }
    owned_.push_back(*p);
  }

  void ck(cudaError_t e)
  {
    if (e != cudaSuccess && status_ == LA3G_OK)
    {
      std::snprintf(msg_, sizeof msg_, "CUDA: %s", cudaGetErrorString(e));
      status_ = LA3G_ECUDA;
    }
  }

  int sync()
  {
    ck(cudaStreamSynchronize(s_));
    return status_;
  }

  int fail(int code, const char* m)
  {
    if (status_ == LA3G_OK)
    {
      status_ = code;
      std::snprintf(msg_, sizeof msg_, "%s", m);
    }
    return status_;
  }

  P prog_;
  la3g_device_graph dv_{};
  detail::View v_{};
  cudaStream_t s_ = nullptr;
  bool directed_ = false, mirrored_ = false;
  int cur_ = 0;
  void *S_ = nullptr, *mirror_ = nullptr, *xr_[2] = {nullptr, nullptr}, *xra_[2] = {nullptr, nullptr};
  void *xs_ = nullptr, *xsa_ = nullptr, *active_ = nullptr, *any_ = nullptr;
  std::vector<void*> owned_;
  int status_ = LA3G_OK;
  char msg_[160] = {0};
};

}  // namespace la3g_vp

#endif
