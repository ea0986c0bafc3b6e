/* la3g_vp.cuh: the vertex-program API as device functor templates.
 *
 * This is the plugin interface of the reference, VertexProgram<W, M, A, S>
 * (src/vprogram/vertex_program.h:99-263), re-expressed for the GPU: a user
 * program is a plain struct whose callbacks are __device__ member functions,
 * and Engine<Program> runs the reference's BSP loop over a graph loaded by
 * libla3g (la3g_graph_device_view, la3g_graph_push_view).  Kernels are
 * instantiated per program, so no callback is dispatched indirectly.
 *
 * A program provides (types trivially copyable):
 *
 *   struct MyProgram {
 *     using Msg = ...; using Acc = ...; using State = ...;
 *     static constexpr bool stationary = ...;         // VertexProgram::stationary
 *     static constexpr bool gather_with_state = ...;  // gather(edge, msg, state) overridden
 *     static constexpr bool apply_with_iteration = ...;  // apply(y, state, iter) overridden
 *     static constexpr bool associative = ...;        // optional, default false (below)
 *     __device__ bool  init(uint32_t vid, State& s) const;          // init(vid, s) -> activate
 *     __device__ Msg   scatter(const State& s) const;
 *     __device__ Acc   gather(const la3g_vp::Edge& e, const Msg& m, const State& row_state) const;
 *     __device__ void  combine(const Acc& y1, Acc& y2) const;      // y2 = y1 (+) y2
 *     __device__ bool  apply(const Acc& y, State& s, uint32_t iter) const;
 *     __device__ Acc   zero() const;                                // A()
 *   };
 *
 * Variable-size messages (the reference's Serializable messages,
 * streaming_array.hpp:81-211): a program with `var_msg = true` sets
 * `using Elem = ...; using Msg = la3g_vp::MsgView<Elem>;` and provides
 *     __device__ uint32_t msg_len(const State& s) const;          // elements it scatters
 *     __device__ void scatter_into(const State& s, Elem* out) const;
 * The engine sizes each iteration's messages (lengths, a prefix sum), keeps
 * them in a device arena that grows as needed, and hands gather() a view
 * (data, len) of the column's message; lengths are unbounded.
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
 *     single-iteration variant (no scatter after apply);
 *   - vertex activity (the reference's vseg.activity): apply marks the
 *     regular vertices it activates (all touched ones when stationary) and
 *     the sinks it activates; it accumulates until reset_activity();
 *     activate_all() marks every vertex (vertex_program.hpp:550-555);
 *   - reduce / topk / btopk (vertex_program.hpp:558-767) enumerate the
 *     vertices (all, or the active ones) in position order, by original id.
 *
 * How an iteration runs on the device.  The rows to process are either all
 * rows with in-edges ("dense", always for stationary programs) or only the
 * rows an active column reaches ("sparse": the active columns' out-edges
 * are pushed into a row bitmap first), whichever reads fewer edges: the
 * frontier's out-degree sum decides, as a direction-optimising BFS does.
 * The chosen rows are split by in-degree: rows of at most kSmallDeg in-edges
 * take kSmallLanes lanes each, longer rows a whole warp; the lanes load
 * edges, activity flags and messages and compute gather() in parallel, and
 * the row's combine() chain is then applied in edge order (one lane after
 * another, or, for associative programs, as an order-keeping tree over the
 * lanes).  Programs that declare `associative = true` (combine(a, combine(b,
 * c)) == combine(combine(a, b), c) for every a, b, c) also have rows above
 * kHubDeg in-edges cut into kHubTask-edge tasks spread over the grid, whose
 * partial results are combined in task order afterwards.  Every form gives
 * the result of the reference's edge-by-edge loop: the associative ones
 * regroup only what associativity lets them regroup, never reorder.
 *
 * Engine methods return LA3G_OK or an la3g_status; error_string() says why.
 * An engine is bound to its graph's stream; it is not re-entrant.
 */
#ifndef LA3G_VP_CUH
#define LA3G_VP_CUH

#include <cuda_runtime.h>

#include <cub/device/device_scan.cuh>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <utility>
#include <vector>

#include "la3g.h"

namespace la3g_vp {

struct Edge
{
  uint32_t src, dst, weight;
};

// A variable-size message (programs with `var_msg = true`): the elements a
// vertex scattered, in the engine's message arena for the iteration.
template <class T>
struct MsgView
{
  const T* data;
  uint32_t len;
};

// The (id, value) pair top-k comparators see: the members of the
// reference's std::pair<I, V> (first = vertex id, second = mapped value).
template <class I, class V>
struct Pair
{
  I first;
  V second;
};

namespace detail {

constexpr uint32_t kSmallDeg = 32;     // rows with at most this many in-edges: kSmallLanes lanes each
constexpr uint32_t kSmallLanes = 4;
constexpr uint32_t kHubDeg = 4096;     // associative programs: longer rows are cut into tasks
constexpr uint32_t kHubTask = 2048;    // in-edges per hub task (one warp)
constexpr int kHubShift = 40;          // packed hub counter: slots << kHubShift | tasks
constexpr double kDenseDivisor = 16.0; // dense when the frontier's out-edges exceed the edges / this
constexpr uint32_t kTopkTile = 1024;   // top-k: items sorted per block
constexpr uint32_t kTopkMaxK = 512;    // largest k (each round must shrink the candidates)

template <class P, class = void>
struct Assoc : std::false_type
{
};
template <class P>
struct Assoc<P, std::void_t<decltype(P::associative)>> : std::integral_constant<bool, P::associative>
{
};

template <class P, class = void>
struct VarMsg : std::false_type
{
};
template <class P>
struct VarMsg<P, std::void_t<decltype(P::var_msg)>> : std::integral_constant<bool, P::var_msg>
{
};

struct View
{
  const uint32_t* row_ptr;
  const uint32_t* col;
  const uint32_t* weight;
  const uint32_t* hash_of_pos;
  const uint32_t* out_ptr;  // push CSR (column -> rows)
  const uint32_t* out_row;
  uint32_t nreg, nsink, src_base, iso_base;
};

// A set of rows to process, split by in-degree (device arrays; counts in cnt:
// [0] small rows, [1] warp rows, [2] hubs << kHubShift | hub tasks).
struct RowSet
{
  uint32_t* small;
  uint32_t* mid;
  uint32_t* hub;
  uint32_t* hub_task0;
  unsigned long long* cnt;
};

// Iteration counters: [0] a regular vertex was activated, [1] next frontier
// size, [2] its out-degree sum.
template <class P>
struct Step
{
  using Msg = typename P::Msg;
  using State = typename P::State;
  bool with_sources, single_iter;
  uint32_t iter;
  State* S;
  const State* mirror;
  const Msg* xr;
  const uint8_t* xr_act;
  const Msg* xs;
  const uint8_t* xs_act;
  Msg* xr_next;
  uint8_t* xr_next_act;
  uint8_t* vact;
  uint32_t* next_list;
  unsigned long long* ctr;
};

// Warp shuffles of any trivially copyable value, 32 bits at a time.
template <class T>
__device__ __forceinline__ T shfl_idx(const T& v, int src, int width = 32)
{
  constexpr int W = (int) ((sizeof(T) + 3) / 4);
  uint32_t w[W] = {};
  memcpy(w, &v, sizeof(T));
#pragma unroll
  for (int i = 0; i < W; i++) w[i] = __shfl_sync(0xffffffffu, w[i], src, width);
  T r = v;
  memcpy(&r, w, sizeof(T));
  return r;
}

template <class T>
__device__ __forceinline__ T shfl_down(const T& v, unsigned off, int width)
{
  constexpr int W = (int) ((sizeof(T) + 3) / 4);
  uint32_t w[W] = {};
  memcpy(w, &v, sizeof(T));
#pragma unroll
  for (int i = 0; i < W; i++) w[i] = __shfl_down_sync(0xffffffffu, w[i], off, width);
  T r = v;
  memcpy(&r, w, sizeof(T));
  return r;
}

// Loads edge i of row r (if `live`): whether its column is active, its
// message, and the Edge the reference passes to gather.
template <class P>
__device__ __forceinline__ bool load_edge(const View& g, const Step<P>& st, bool live, uint32_t i, uint32_t dst,
                                          typename P::Msg& m, Edge& ed)
{
  if (!live) return false;
  const uint32_t c = g.col[i];
  bool act;
  if (c >= g.src_base)
  {
    act = st.with_sources && st.xs_act[c - g.src_base];
    if (act) m = st.xs[c - g.src_base];
  }
  else
  {
    act = st.xr_act[c] != 0;
    if (act) m = st.xr[c];
  }
  if (act) ed = Edge{g.hash_of_pos[c], dst, g.weight ? g.weight[i] : 0u};
  return act;
}

// One step of G lanes over G consecutive edges (one per lane, `act` where
// the edge's column is active): combines their gathers into `acc` in edge
// order.  Associative programs fold the lanes as a tree that keeps the
// order (later (+) earlier) and add the result to acc in the group's first
// lane; the others apply combine lane after lane, shuffling whichever of
// the gathered value or the (edge, message) pair is smaller.  Called by all
// 32 lanes of the warp.
template <class P, int G>
__device__ __forceinline__ void group_step(const P& prog, const typename P::State& rs, bool act, const Edge& ed,
                                           const typename P::Msg& m, typename P::Acc& acc, bool& touched, int lane)
{
  using Acc = typename P::Acc;
  using Msg = typename P::Msg;
  const int sub = lane & (G - 1), gbase = lane - sub;
  const unsigned all = __ballot_sync(0xffffffffu, act);
  const unsigned gm = (G == 32) ? all : ((all >> gbase) & ((1u << G) - 1u));
  if constexpr (Assoc<P>::value)
  {
    Acc x = act ? prog.gather(ed, m, rs) : prog.zero();
    bool v = act;
#pragma unroll
    for (int off = 1; off < G; off <<= 1)
    {
      const Acc y = shfl_down(x, off, G);
      const bool vy = __shfl_down_sync(0xffffffffu, v, off, G);
      if ((sub & (2 * off - 1)) == 0 && sub + off < G && vy)
      {
        if (v) prog.combine(y, x);  // x = later (+) earlier
        else x = y;
        v = true;
      }
    }
    if (sub == 0 && v)
    {
      prog.combine(x, acc);
      touched = true;
    }
  }
  else if constexpr (sizeof(Acc) <= sizeof(Msg) + sizeof(Edge))
  {
    const Acc gv = act ? prog.gather(ed, m, rs) : prog.zero();
    if (G == 32)
    {
      for (unsigned b = all; b; b &= b - 1)  // uniform over the warp
        prog.combine(shfl_idx(gv, __ffs(b) - 1), acc);
    }
    else
    {
#pragma unroll
      for (int j = 0; j < G; j++)
      {
        const Acc gj = shfl_idx(gv, gbase + j);
        if ((gm >> j) & 1u) prog.combine(gj, acc);
      }
    }
    touched |= gm != 0;
  }
  else
  {
    // large accumulators: every lane of the group recomputes the gathers in order
    if (G == 32)
    {
      for (unsigned b = all; b; b &= b - 1)
      {
        const int j = __ffs(b) - 1;
        const Edge ej = shfl_idx(ed, j);
        const Msg mj = shfl_idx(m, j);
        prog.combine(prog.gather(ej, mj, rs), acc);
      }
    }
    else
    {
#pragma unroll
      for (int j = 0; j < G; j++)
      {
        const Edge ej = shfl_idx(ed, gbase + j);
        const Msg mj = shfl_idx(m, gbase + j);
        if ((gm >> j) & 1u) prog.combine(prog.gather(ej, mj, rs), acc);
      }
    }
    touched |= gm != 0;
  }
}

// Applies the row's accumulator (lanes with `live`) and records what the
// reference's apply_and_scatter_messages records (:669-724): the state,
// the vertex activity, the next messages, `any` for activated regular
// rows, and, for non-stationary programs, the next frontier list with its
// out-degree sum.  Called by all 32 lanes.
template <class P>
__device__ __forceinline__ void apply_row(const P& prog, const View& g, const Step<P>& st, bool live, uint32_t r,
                                          const typename P::Acc& acc, int lane)
{
  bool scat = false, act = false;
  uint32_t odeg = 0;
  if (live)
  {
    typename P::Acc fin = prog.zero();
    prog.combine(acc, fin);
    act = prog.apply(fin, st.S[r], st.iter);
    if (r >= g.nreg)
    {
      if (act) st.vact[r] = 1;  // sink activations do not count
      act = false;
    }
    else if (act || P::stationary)
    {
      st.vact[r] = 1;
      if (!st.single_iter)
      {
        if constexpr (!VarMsg<P>::value) st.xr_next[r] = prog.scatter(st.S[r]);  // else filled after the step
        st.xr_next_act[r] = 1;
        scat = true;
        odeg = g.out_ptr[r + 1] - g.out_ptr[r];
      }
    }
  }
  if (__any_sync(0xffffffffu, act) && lane == 0) st.ctr[0] = 1;
  if (P::stationary) return;  // stationary steps are dense: no frontier list
  const unsigned m = __ballot_sync(0xffffffffu, scat);
  if (!m) return;
  unsigned long long d = odeg;
  for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
  uint32_t base = 0;
  if (lane == 0)
  {
    base = (uint32_t) atomicAdd(&st.ctr[1], (unsigned long long) __popc(m));
    atomicAdd(&st.ctr[2], d);
  }
  base = __shfl_sync(0xffffffffu, base, 0);
  if (scat) st.next_list[base + __popc(m & ((1u << lane) - 1u))] = r;
}

template <class P>
__global__ void k_init(P prog, View g, uint32_t nslots, bool directed, typename P::State* S,
                       typename P::Msg* xr, uint8_t* xr_act, typename P::Msg* xs, uint8_t* xs_act,
                       const uint32_t* id_of_pos, uint8_t* active, uint32_t* front, uint32_t* srcs,
                       unsigned long long* ctr)
{
  const int lane = threadIdx.x & 31;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t p0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); p0 < nslots; p0 += stride)
  {
    const uint32_t p = p0 + lane;
    bool reg = false, src = false;
    uint32_t odeg = 0;
    if (p < nslots)
    {
      typename P::State s{};
      const bool act = prog.init(id_of_pos[p], s);
      S[p] = s;
      active[p] = act ? 1 : 0;
      if (act && p < g.nreg)
      {
        if constexpr (!VarMsg<P>::value) xr[p] = prog.scatter(s);
        xr_act[p] = 1;
        reg = true;
      }
      else if (act && directed && p >= g.src_base && p < g.iso_base)
      {
        if constexpr (!VarMsg<P>::value) xs[p - g.src_base] = prog.scatter(s);
        xs_act[p - g.src_base] = 1;
        src = true;
      }
      if (reg || src) odeg = g.out_ptr[p + 1] - g.out_ptr[p];
    }
    // the first frontier (regular) and the active sources, with out-degree sums
    const unsigned mr = __ballot_sync(0xffffffffu, reg), ms = __ballot_sync(0xffffffffu, src);
    unsigned long long dr = reg ? odeg : 0, ds = src ? odeg : 0;
    for (int o = 16; o > 0; o >>= 1)
    {
      dr += __shfl_xor_sync(0xffffffffu, dr, o);
      ds += __shfl_xor_sync(0xffffffffu, ds, o);
    }
    uint32_t br = 0, bs = 0;
    if (lane == 0)
    {
      if (mr) br = (uint32_t) atomicAdd(&ctr[1], (unsigned long long) __popc(mr));
      if (mr) atomicAdd(&ctr[2], dr);
      if (ms) bs = (uint32_t) atomicAdd(&ctr[3], (unsigned long long) __popc(ms));
      if (ms) atomicAdd(&ctr[4], ds);
    }
    br = __shfl_sync(0xffffffffu, br, 0);
    bs = __shfl_sync(0xffffffffu, bs, 0);
    const unsigned lt = (1u << lane) - 1u;
    if (reg) front[br + __popc(mr & lt)] = p;
    if (src) srcs[bs + __popc(ms & lt)] = p;
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

// Rows of [lo, hi) with in-edges (those set in `bits` when given) into a row
// set; warps append a ballot at a time.
static __global__ void k_rowset(const uint32_t* __restrict__ ptr, uint32_t lo, uint32_t hi, const uint32_t* __restrict__ bits,
                         bool split_hubs, RowSet rs)
{
  const int lane = threadIdx.x & 31;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t r0 = lo + blockIdx.x * blockDim.x + (threadIdx.x & ~31u); r0 < hi; r0 += stride)
  {
    const uint32_t r = r0 + lane;
    uint32_t deg = 0;
    if (r < hi && (!bits || ((bits[r >> 5] >> (r & 31)) & 1u))) deg = ptr[r + 1] - ptr[r];
    const bool hub = split_hubs && deg > kHubDeg;
    const bool small = deg && deg <= kSmallDeg, mid = deg > kSmallDeg && !hub;
    const unsigned ms = __ballot_sync(0xffffffffu, small), mm = __ballot_sync(0xffffffffu, mid);
    uint32_t bs = 0, bm = 0;
    if (lane == 0)
    {
      if (ms) bs = (uint32_t) atomicAdd(&rs.cnt[0], (unsigned long long) __popc(ms));
      if (mm) bm = (uint32_t) atomicAdd(&rs.cnt[1], (unsigned long long) __popc(mm));
    }
    bs = __shfl_sync(0xffffffffu, bs, 0);
    bm = __shfl_sync(0xffffffffu, bm, 0);
    const unsigned lt = (1u << lane) - 1u;
    if (small) rs.small[bs + __popc(ms & lt)] = r;
    if (mid) rs.mid[bm + __popc(mm & lt)] = r;
    if (hub)
    {
      const uint32_t nt = (deg + kHubTask - 1) / kHubTask;
      const unsigned long long old = atomicAdd(&rs.cnt[2], (1ull << kHubShift) | nt);
      const uint32_t slot = (uint32_t) (old >> kHubShift);
      rs.hub[slot] = r;
      rs.hub_task0[slot] = (uint32_t) (old & ((1ull << kHubShift) - 1));
    }
  }
}

// Sparse step: the active columns' out-edges mark their rows.  Regular
// columns come from the frontier list; active sources reach sink rows in
// every iteration and regular rows when with_src_regular.
static __global__ void k_mark(const uint32_t* __restrict__ optr, const uint32_t* __restrict__ orow,
                       const uint32_t* __restrict__ front, uint32_t nfront, const uint32_t* __restrict__ srcs,
                       uint32_t nsrc, bool with_src_regular, uint32_t nreg, uint32_t* bits)
{
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t f = warp; f < nfront + nsrc; f += nwarps)
  {
    const bool src = f >= nfront;
    const uint32_t c = src ? srcs[f - nfront] : front[f];
    for (uint32_t i = optr[c] + lane; i < optr[c + 1]; i += 32)
    {
      const uint32_t r = orow[i];
      if (src && !with_src_regular && r < nreg) continue;
      atomicOr(&bits[r >> 5], 1u << (r & 31));
    }
  }
}

// Rows of a list, G lanes each; every lane walks the same number of edge
// steps (the warp's longest row), so the shuffles see all 32 lanes.  At
// least two blocks per SM: wide accumulators (graph simulation's 32
// counters, held three times in the tree) would otherwise take ~150
// registers and leave one block per SM (R-MAT s20: 8.1 -> 7.4 ms).
template <class P, int G>
__global__ void __launch_bounds__(256, 2)
k_pull_rows(P prog, View g, const uint32_t* __restrict__ rows, const unsigned long long* __restrict__ count, Step<P> st)
{
  using Acc = typename P::Acc;
  using State = typename P::State;
  using Msg = typename P::Msg;
  const uint32_t n = (uint32_t) *count;
  const int lane = threadIdx.x & 31, sub = lane & (G - 1);
  const uint32_t group = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * (32 / G) + lane / G;
  const uint32_t ngroups = ((gridDim.x * blockDim.x) >> 5) * (32 / G);
  const uint32_t rounds = (n + ngroups - 1) / ngroups;
  for (uint32_t k = 0; k < rounds; k++)
  {
    const uint32_t idx = group + k * ngroups;
    const bool have = idx < n;
    const uint32_t r = have ? rows[idx] : 0u;
    const uint32_t b = have ? g.row_ptr[r] : 0u, e = have ? g.row_ptr[r + 1] : 0u;
    const uint32_t dst = have ? g.hash_of_pos[r] : 0u;
    State rs{};
    if (P::gather_with_state && have) rs = st.mirror[r];
    Acc acc = prog.zero();
    bool touched = false;
    const uint32_t steps = __reduce_max_sync(0xffffffffu, (e - b + G - 1) / G);
    for (uint32_t j = 0; j < steps; j++)
    {
      const uint32_t i = b + j * G + sub;
      Msg m{};
      Edge ed{0, 0, 0};
      const bool act = load_edge<P>(g, st, i < e, i, dst, m, ed);
      group_step<P, G>(prog, rs, act, ed, m, acc, touched, lane);
    }
    apply_row<P>(prog, g, st, have && touched && sub == 0, r, acc, lane);
  }
}

// Slot whose task range holds task t (task0 ascends with the slot).
__device__ __forceinline__ uint32_t hub_of_task(const uint32_t* __restrict__ task0, uint32_t nbig, uint32_t t)
{
  uint32_t lo = 0, hi = nbig;
  while (hi - lo > 1)
  {
    const uint32_t mid = (lo + hi) >> 1;
    if (task0[mid] <= t) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Associative programs: one warp per hub task folds its edges in order into
// a partial accumulator (ok = some edge was active).
template <class P>
__global__ void __launch_bounds__(256)
k_pull_tasks(P prog, View g, RowSet rs, Step<P> st, typename P::Acc* part, uint8_t* part_ok)
{
  using Acc = typename P::Acc;
  using State = typename P::State;
  using Msg = typename P::Msg;
  const unsigned long long packed = rs.cnt[2];
  const uint32_t nh = (uint32_t) (packed >> kHubShift), nt = (uint32_t) (packed & ((1ull << kHubShift) - 1));
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t t = warp; t < nt; t += nwarps)
  {
    const uint32_t slot = hub_of_task(rs.hub_task0, nh, t);
    const uint32_t r = rs.hub[slot];
    const uint32_t b = g.row_ptr[r] + (t - rs.hub_task0[slot]) * kHubTask;
    const uint32_t e = min(b + kHubTask, g.row_ptr[r + 1]);
    const uint32_t dst = g.hash_of_pos[r];
    State st_row{};
    if (P::gather_with_state) st_row = st.mirror[r];
    Acc acc = prog.zero();
    bool ok = false;
    for (uint32_t i0 = b; i0 < e; i0 += 32)
    {
      Msg m{};
      Edge ed{0, 0, 0};
      const bool act = load_edge<P>(g, st, i0 + lane < e, i0 + lane, dst, m, ed);
      Acc x = act ? prog.gather(ed, m, st_row) : prog.zero();
      bool v = act;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1)
      {
        const Acc y = shfl_down(x, off, 32);
        const bool vy = __shfl_down_sync(0xffffffffu, v, off);
        if ((lane & (2 * off - 1)) == 0 && lane + off < 32 && vy)
        {
          if (v) prog.combine(y, x);
          else x = y;
          v = true;
        }
      }
      if (lane == 0 && v)
      {
        if (ok) prog.combine(x, acc);
        else acc = x;
        ok = true;
      }
    }
    if (lane == 0)
    {
      part[t] = acc;
      part_ok[t] = ok ? 1 : 0;
    }
  }
}

// The hubs' partial accumulators, combined in task order, then applied.
template <class P>
__global__ void k_hub_apply(P prog, View g, RowSet rs, Step<P> st, const typename P::Acc* part,
                            const uint8_t* part_ok)
{
  const unsigned long long packed = rs.cnt[2];
  const uint32_t nh = (uint32_t) (packed >> kHubShift), nt = (uint32_t) (packed & ((1ull << kHubShift) - 1));
  const int lane = threadIdx.x & 31;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t s0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); s0 < nh; s0 += stride)
  {
    const uint32_t slot = s0 + lane;
    const bool have = slot < nh;
    typename P::Acc acc = prog.zero();
    bool touched = false;
    uint32_t r = 0;
    if (have)
    {
      r = rs.hub[slot];
      const uint32_t t1 = slot + 1 < nh ? rs.hub_task0[slot + 1] : nt;
      for (uint32_t t = rs.hub_task0[slot]; t < t1; t++)
        if (part_ok[t])
        {
          prog.combine(part[t], acc);
          touched = true;
        }
    }
    apply_row<P>(prog, g, st, have && touched, r, acc, lane);
  }
}

template <class P>
__global__ void k_scatter_all(P prog, uint32_t nreg, const typename P::State* S, typename P::Msg* xr, uint8_t* act)
{
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < nreg; r += gridDim.x * blockDim.x)
  {
    if constexpr (!VarMsg<P>::value) xr[r] = prog.scatter(S[r]);
    act[r] = 1;
  }
}

// Variable-size messages, after the vertices that scatter are known
// (act[i] set for vertex base + i): their lengths, then (after an exclusive
// scan of the lengths) their elements copied into the arena and the views.
template <class P>
__global__ void k_msg_len(P prog, uint32_t n, uint32_t base, const typename P::State* S, const uint8_t* act,
                          unsigned long long* len)
{
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    len[i] = act[i] ? prog.msg_len(S[base + i]) : 0u;
}

template <class P>
__global__ void k_msg_fill(P prog, uint32_t n, uint32_t base, const typename P::State* S, const uint8_t* act,
                           const unsigned long long* off, typename P::Elem* arena, typename P::Msg* views)
{
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
  {
    if (!act[i]) continue;
    const typename P::State& s = S[base + i];
    typename P::Elem* out = arena + off[i];
    prog.scatter_into(s, out);
    views[i] = typename P::Msg{out, prog.msg_len(s)};
  }
}

template <class T>
__global__ void k_by_id(uint32_t n, const uint32_t* id_of_pos, const T* in, T* out)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) out[id_of_pos[p]] = in[p];
}

// ---- reduce / top-k ----------------------------------------------------------

// Top-k items: the mapped value, the vertex id and the enumeration position
// (ties under cmp keep that order; pos = ~0 marks an empty slot).
template <class I, class V>
struct TopItem
{
  V v;
  I i;
  uint32_t pos;
};

template <class I, class V, class Cmp>
__device__ __forceinline__ bool top_before(const Cmp& cmp, const TopItem<I, V>& a, const TopItem<I, V>& b)
{
  if (a.pos == 0xFFFFFFFFu) return false;
  if (b.pos == 0xFFFFFFFFu) return true;
  const Pair<I, V> pa{a.i, a.v}, pb{b.i, b.v};
  if (cmp(pa, pb)) return true;
  if (cmp(pb, pa)) return false;
  return a.pos < b.pos;
}

// Sorts kTopkTile items in shared memory (bitonic) and writes the first k
// of each tile.  The first pass maps the vertices of the tile's positions (all, or
// the active ones); later passes read the previous pass's items.  With
// batches, blockIdx.y is the batch b and map(id, state) returns an indexable
// array of values.
template <class P, class I, class V, class Map, class Cmp, bool BATCH>
__global__ void __launch_bounds__(kTopkTile / 2)
k_topk_round(Map map, Cmp cmp, uint32_t k, uint32_t n, const typename P::State* S, const uint32_t* id_of_pos,
             const uint8_t* vact, bool active_only, const TopItem<I, V>* in, TopItem<I, V>* out)
{
  __shared__ TopItem<I, V> sh[kTopkTile];
  const uint32_t b = blockIdx.y;
  const uint32_t base = blockIdx.x * kTopkTile;
  for (uint32_t t = threadIdx.x; t < kTopkTile; t += blockDim.x)
  {
    TopItem<I, V> it;
    memset(&it, 0, sizeof it);
    it.pos = 0xFFFFFFFFu;
    const uint32_t x = base + t;
    if (x < n)
    {
      if (S)
      {
        if (!active_only || vact[x])
        {
          const uint32_t id = id_of_pos[x];
          if constexpr (BATCH) it.v = map(id, S[x])[b];
          else it.v = map(id, S[x]);
          it.i = (I) id;
          it.pos = x;
        }
      }
      else it = in[(size_t) b * n + x];
    }
    sh[t] = it;
  }
  __syncthreads();
  for (uint32_t size = 2; size <= kTopkTile; size <<= 1)
    for (uint32_t stride = size >> 1; stride > 0; stride >>= 1)
    {
      for (uint32_t t = threadIdx.x; t < kTopkTile / 2; t += blockDim.x)
      {
        const uint32_t lo = 2 * t - (t & (stride - 1)), hi = lo + stride;
        const bool up = (lo & size) == 0;
        const bool swap = up ? top_before<I, V, Cmp>(cmp, sh[hi], sh[lo]) : top_before<I, V, Cmp>(cmp, sh[lo], sh[hi]);
        if (swap)
        {
          const TopItem<I, V> tmp = sh[lo];
          sh[lo] = sh[hi];
          sh[hi] = tmp;
        }
      }
      __syncthreads();
    }
  const uint32_t nout = gridDim.x * k;
  for (uint32_t t = threadIdx.x; t < k; t += blockDim.x) out[(size_t) b * nout + blockIdx.x * k + t] = sh[t];
}

// Blocks of 256 threads for n items, at most 16 per streaming multiprocessor
// of the current device.
inline unsigned sm_count()
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
  return (unsigned) sms;
}

inline unsigned blocks_for(uint64_t n)
{
  const uint64_t cap = (uint64_t) sm_count() * 16;
  uint64_t b = (n + 255) / 256;
  return (unsigned) (b < 1 ? 1 : (b > cap ? cap : b));
}

// reduce(): map(id, state) folded with red(acc, value) over each chunk of
// positions in order, the chunks' results folded in order on the host side
// of the call.
// Fewer than k candidates: the reference pads its list with value-
// initialised pairs and sorts them in (one rank: resize(k), partial_sort).
// Empty slots become such pairs, ordered after the real ones on ties, and
// the k items are sorted again (insertion sort, one thread per batch).
template <class I, class V, class Cmp>
__global__ void k_topk_pad(Cmp cmp, uint32_t k, TopItem<I, V>* items)
{
  TopItem<I, V>* it = items + (size_t) blockIdx.x * k;
  bool padded = false;
  for (uint32_t t = 0; t < k; t++)
    if (it[t].pos == 0xFFFFFFFFu)
    {
      TopItem<I, V> z;
      memset(&z, 0, sizeof z);
      z.v = V();
      z.i = I();
      z.pos = 0x80000000u + t;
      it[t] = z;
      padded = true;
    }
  if (!padded) return;
  for (uint32_t a = 1; a < k; a++)
  {
    const TopItem<I, V> x = it[a];
    uint32_t c = a;
    for (; c > 0 && top_before<I, V, Cmp>(cmp, x, it[c - 1]); c--) it[c] = it[c - 1];
    it[c] = x;
  }
}

template <class P, class V, class Map, class Red>
__global__ void k_reduce_chunks(Map map, Red red, uint32_t n, uint32_t chunk, const typename P::State* S,
                                const uint32_t* id_of_pos, const uint8_t* vact, bool active_only, V* part,
                                uint32_t nparts)
{
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nparts) return;
  V r = V();
  const uint32_t lo = t * chunk, hi = min(n, lo + chunk);
  for (uint32_t p = lo; p < hi; p++)
    if (!active_only || vact[p]) red(r, map(id_of_pos[p], S[p]));
  part[t] = r;
}

template <class V, class Red>
__global__ void k_reduce_final(Red red, const V* part, uint32_t nparts, V* out)
{
  V r = V();
  for (uint32_t t = 0; t < nparts; t++) red(r, part[t]);
  V f = V();
  red(f, r);  // the master's fold of the ranks' results (one rank)
  *out = f;
}

}  // namespace detail

template <class P>
class Engine
{
 public:
  using Msg = typename P::Msg;
  using Acc = typename P::Acc;
  using State = typename P::State;
  static constexpr bool kAssoc = detail::Assoc<P>::value;

  Engine(la3g_graph* g, const P& prog) : prog_(prog)
  {
    if (la3g_graph_device_view(g, &dv_) != LA3G_OK)
    {
      fail(LA3G_EINVAL, "graph view unavailable");
      return;
    }
    const uint32_t* optr = nullptr;
    const uint32_t* orow = nullptr;
    if (la3g_graph_push_view(g, &optr, &orow) != LA3G_OK)
    {
      fail(LA3G_ENOMEM, "push view unavailable");
      return;
    }
    s_ = (cudaStream_t) dv_.stream;
    directed_ = dv_.flags & LA3G_DIRECTED;
    v_ = detail::View{dv_.row_ptr, dv_.col, dv_.weight, dv_.hash_of_pos, optr, orow, dv_.nregular, dv_.nsink,
                      dv_.nregular + dv_.nsink, dv_.nregular + dv_.nsink + dv_.nsource};
    const uint32_t N = dv_.nslots, nrows = dv_.nregular + dv_.nsink;
    alloc(&S_, (size_t) N * sizeof(State));
    alloc(&mirror_, P::gather_with_state ? (size_t) N * sizeof(State) : 16);
    alloc(&xr_[0], (size_t) (dv_.nregular + 1) * sizeof(Msg));
    alloc(&xr_[1], (size_t) (dv_.nregular + 1) * sizeof(Msg));
    alloc(&xra_[0], dv_.nregular + 1);
    alloc(&xra_[1], dv_.nregular + 1);
    alloc(&xs_, (size_t) (dv_.nsource + 1) * sizeof(Msg));
    alloc(&xsa_, dv_.nsource + 1);
    alloc(&active_, N);
    alloc(&vact_, N + 1);
    alloc(&ctr_, 8 * sizeof(unsigned long long));
    alloc(&front_[0], (size_t) (dv_.nregular + 1) * 4);
    alloc(&front_[1], (size_t) (dv_.nregular + 1) * 4);
    alloc(&srcs_, (size_t) (dv_.nsource + 1) * 4);
    alloc(&bits_, (size_t) (nrows / 32 + 2) * 4);
    // hub tasks: at most edges / kHubTask + one per hub row
    const uint64_t maxtasks = kAssoc ? dv_.nentries / detail::kHubTask + dv_.nentries / detail::kHubDeg + 2 : 1;
    alloc(&part_, (size_t) maxtasks * sizeof(Acc));
    alloc(&part_ok_, (size_t) maxtasks);
    for (int k = 0; k < 3; k++) make_rowset(&sets_[k], k == 1 ? dv_.nsink : (k == 0 ? dv_.nregular : nrows));
    if (status_ != LA3G_OK) return;
    // the dense row sets of the regular and the sink rows (fixed per graph)
    ck(cudaMemsetAsync(sets_[0].cnt, 0, 3 * sizeof(unsigned long long), s_));
    ck(cudaMemsetAsync(sets_[1].cnt, 0, 3 * sizeof(unsigned long long), s_));
    if (dv_.nregular)
      detail::k_rowset<<<detail::blocks_for(dv_.nregular), 256, 0, s_>>>(dv_.row_ptr, 0, dv_.nregular, nullptr,
                                                                         kAssoc, sets_[0]);
    if (dv_.nsink)
      detail::k_rowset<<<detail::blocks_for(dv_.nsink), 256, 0, s_>>>(dv_.row_ptr, dv_.nregular, nrows, nullptr,
                                                                      kAssoc, sets_[1]);
    ck(cudaGetLastError());
    ck(cudaMemsetAsync(vact_, 0, N + 1, s_));
    sync();
  }

  ~Engine()
  {
    for (void* p : owned_) cudaFree(p);
    for (void* p : arena_)
      if (p) cudaFree(p);
    if (scan_tmp_) cudaFree(scan_tmp_);
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
    ck(cudaMemsetAsync(ctr_, 0, 8 * sizeof(unsigned long long), s_));
    detail::k_init<P><<<detail::blocks_for(N), 256, 0, s_>>>(
        prog_, v_, N, directed_, (State*) S_, (Msg*) xr_[0], (uint8_t*) xra_[0], (Msg*) xs_, (uint8_t*) xsa_,
        dv_.id_of_pos, (uint8_t*) active_, (uint32_t*) front_[0], (uint32_t*) srcs_, (unsigned long long*) ctr_);
    ck(cudaGetLastError());
    if (P::gather_with_state && !mirrored_)
    {
      detail::k_mirror<P><<<detail::blocks_for(N), 256, 0, s_>>>(N, (const State*) S_, (const uint8_t*) active_,
                                                                 (State*) mirror_);
      ck(cudaGetLastError());
      mirrored_ = true;
      // vertex activity is kept only for mirroring up to here (initialize :166-172)
      ck(cudaMemsetAsync(vact_, 0, N + 1, s_));
    }
    // variable-size messages of the vertices init activated
    fill_messages(dv_.nregular, 0, xra_[0], xr_[0], 0);
    if (directed_) fill_messages(dv_.nsource, v_.src_base, xsa_, xs_, 2);
    unsigned long long h[8];
    ck(cudaMemcpyAsync(h, ctr_, sizeof h, cudaMemcpyDeviceToHost, s_));
    if (sync() != LA3G_OK) return status_;
    nfront_ = h[1];
    front_deg_ = h[2];
    nsrc_act_ = h[3];
    src_deg_ = h[4];
    return LA3G_OK;
  }

  // execute(num_iterations) (vertex_program_execute.hpp:11-52); 0 = until
  // no regular vertex activates.  *iters_out = iterations run.
  int execute(uint32_t max_iters, uint32_t* iters_out = nullptr)
  {
    if (status_ != LA3G_OK) return status_;
    const bool optimizable = directed_ && !P::gather_with_state && !P::apply_with_iteration;
    const uint32_t nreg = dv_.nregular;
    uint32_t it = 0;
    if (max_iters == 1)
    {
      // execute_single (:251-345): regular rows, then sinks; no scatter
      step(true, true, 0, directed_ && dv_.nsink);
      it = 1;
    }
    else
    {
      const bool until = max_iters == 0;
      for (;;)
      {
        if (!until && it >= max_iters) break;
        const bool with_src = P::stationary || it == 0;
        ck(cudaMemsetAsync(xra_[cur_ ^ 1], 0, nreg + 1, s_));
        // sink rows take the sources' messages in every iteration
        // (vertex_program_execute.hpp:464-468)
        step(with_src, false, it, !optimizable && directed_ && dv_.nsink);
        fill_messages(nreg, 0, xra_[cur_ ^ 1], xr_[cur_ ^ 1], cur_ ^ 1);
        cur_ ^= 1;
        it++;
        unsigned long long h[3];
        ck(cudaMemcpyAsync(h, ctr_, sizeof h, cudaMemcpyDeviceToHost, s_));
        if (sync() != LA3G_OK) return status_;
        nfront_ = h[1];
        front_deg_ = h[2];
        if (until && !h[0]) break;
        if (it > 100000000u) return fail(LA3G_ETIMEOUT, "execute did not converge");
      }
      if (optimizable && dv_.nsink)
      {
        // sinks once (:131-148): every regular vertex scatters its final
        // state; sources' messages as they stand
        detail::k_scatter_all<P><<<detail::blocks_for(nreg), 256, 0, s_>>>(prog_, nreg, (const State*) S_,
                                                                          (Msg*) xr_[cur_], (uint8_t*) xra_[cur_]);
        ck(cudaGetLastError());
        fill_messages(nreg, 0, xra_[cur_], xr_[cur_], cur_);
        ck(cudaMemsetAsync(ctr_, 0, 3 * sizeof(unsigned long long), s_));
        run_rows(sets_[1], make_step(true, false, it));
      }
    }
    if (iters_out) *iters_out = it;
    return sync();
  }

  // reset_activity() / activate_all() (vertex_program.hpp:550-555).
  int reset_activity()
  {
    ck(cudaMemsetAsync(vact_, 0, dv_.nslots + 1, s_));
    return sync();
  }
  int activate_all()
  {
    ck(cudaMemsetAsync(vact_, 1, dv_.nslots, s_));
    return sync();
  }

  // reduce(map, reduce, active_only) (vertex_program.hpp:558-604): map(id,
  // state) -> Value folded with red(Value& acc, const Value& v), over the
  // vertices in position order.  The device folds chunks of positions in
  // order and then the chunks in order, so red must be associative with
  // Value() as its identity: what the reference's own fold of the ranks'
  // results assumes.  Map and Red are device functors.
  template <class Value, class Map, class Red>
  int reduce(Value* out, Map map, Red red, bool active_only = false)
  {
    if (status_ != LA3G_OK) return status_;
    const uint32_t n = dv_.nslots, nparts = detail::sm_count() * 256;
    const uint32_t chunk = (n + nparts - 1) / nparts;
    void* part = nullptr;
    void* res = nullptr;
    if (cudaMalloc(&part, (size_t) nparts * sizeof(Value)) != cudaSuccess ||
        cudaMalloc(&res, sizeof(Value)) != cudaSuccess)
    {
      cudaGetLastError();
      cudaFree(part);
      return fail(LA3G_ENOMEM, "reduce");
    }
    detail::k_reduce_chunks<P, Value, Map, Red><<<(nparts + 255) / 256, 256, 0, s_>>>(
        map, red, n, chunk, (const State*) S_, dv_.id_of_pos, (const uint8_t*) vact_, active_only, (Value*) part,
        nparts);
    detail::k_reduce_final<Value, Red><<<1, 1, 0, s_>>>(red, (const Value*) part, nparts, (Value*) res);
    ck(cudaGetLastError());
    ck(cudaMemcpyAsync(out, res, sizeof(Value), cudaMemcpyDeviceToHost, s_));
    const int st = sync();
    cudaFree(part);
    cudaFree(res);
    return st;
  }

  // topk(k, out, map, cmp, active_only) (vertex_program.hpp:607-680): the k
  // first (id, map(id, state)) pairs under cmp(pair a, pair b) ("a before
  // b"), k <= kTopkMaxK.  As at one rank of the reference, fewer than k
  // candidates are padded with value-initialised pairs before the final
  // sort, so out always holds k pairs.  Pairs that cmp leaves unordered
  // keep the enumeration (position) order, where the reference's
  // partial_sort leaves their order unspecified.  Map and Cmp are device
  // functors; Cmp takes la3g_vp::Pair<I, V> (first = id, second = value).
  template <class I, class V, class Map, class Cmp>
  int topk(uint32_t k, std::vector<std::pair<I, V>>& out, Map map, Cmp cmp, bool active_only = false)
  {
    std::vector<std::pair<I, V>>* o = &out;
    return topk_impl<I, V, Map, Cmp, false>(k, 1, o, map, cmp, active_only);
  }

  // btopk<B>(k, out[B], map, cmp, active_only) (vertex_program.hpp:682-767):
  // B top-k lists over the same vertices; map(id, state) returns an
  // indexable array of B values (e.g. a pointer into the state).
  template <uint32_t B, class I, class V, class Map, class Cmp>
  int btopk(uint32_t k, std::vector<std::pair<I, V>>* out, Map map, Cmp cmp, bool active_only = false)
  {
    return topk_impl<I, V, Map, Cmp, true>(k, B, out, map, cmp, active_only);
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
  // Steps of the last execute() that ran sparse (frontier-driven) / dense.
  uint32_t sparse_steps() const { return sparse_steps_; }
  uint32_t dense_steps() const { return dense_steps_; }

 private:
  detail::Step<P> make_step(bool with_src, bool single, uint32_t iter)
  {
    return detail::Step<P>{with_src,
                           single,
                           iter,
                           (State*) S_,
                           (const State*) mirror_,
                           (const Msg*) xr_[cur_],
                           (const uint8_t*) xra_[cur_],
                           (const Msg*) xs_,
                           (const uint8_t*) xsa_,
                           (Msg*) xr_[cur_ ^ 1],
                           (uint8_t*) xra_[cur_ ^ 1],
                           (uint8_t*) vact_,
                           (uint32_t*) front_[cur_ ^ 1],
                           (unsigned long long*) ctr_};
  }

  // One iteration: the regular rows (and, when `sinks`, the sink rows) that
  // an active column reaches, dense or sparse.
  void step(bool with_src, bool single, uint32_t iter, bool sinks)
  {
    const uint32_t nreg = dv_.nregular, nrows = dv_.nregular + dv_.nsink;
    const double deg = (double) front_deg_ + (double) src_deg_;
    const bool dense = P::stationary || deg * detail::kDenseDivisor > (double) dv_.nentries;
    const uint64_t nfront = nfront_;
    ck(cudaMemsetAsync(ctr_, 0, 3 * sizeof(unsigned long long), s_));
    const detail::Step<P> st = make_step(with_src, single, iter);
    const detail::Step<P> st_sink = make_step(true, single, iter);  // sinks take the sources' messages every time
    if (dense)
    {
      dense_steps_++;
      run_rows(sets_[0], st);
      if (sinks) run_rows(sets_[1], st_sink);
      return;
    }
    sparse_steps_++;
    ck(cudaMemsetAsync(bits_, 0, (size_t) (nrows / 32 + 2) * 4, s_));
    // sources reach regular rows when with_src, sink rows in every iteration
    const uint64_t nsrc = with_src || sinks ? nsrc_act_ : 0;
    if (nfront + nsrc)
      detail::k_mark<<<detail::blocks_for(32 * (nfront + nsrc)), 256, 0, s_>>>(
          v_.out_ptr, v_.out_row, (const uint32_t*) front_[cur_], (uint32_t) nfront, (const uint32_t*) srcs_,
          (uint32_t) nsrc, with_src, nreg, (uint32_t*) bits_);
    ck(cudaGetLastError());
    build_and_run(0, nreg, st);
    if (sinks) build_and_run(nreg, nrows, st_sink);
  }

  void build_and_run(uint32_t lo, uint32_t hi, const detail::Step<P>& st)
  {
    if (hi <= lo) return;
    detail::RowSet& rs = sets_[2];
    ck(cudaMemsetAsync(rs.cnt, 0, 3 * sizeof(unsigned long long), s_));
    detail::k_rowset<<<detail::blocks_for(hi - lo), 256, 0, s_>>>(dv_.row_ptr, lo, hi, (const uint32_t*) bits_,
                                                                   kAssoc, rs);
    ck(cudaGetLastError());
    run_rows(rs, st);
  }

  void run_rows(const detail::RowSet& rs, const detail::Step<P>& st)
  {
    const unsigned grid = detail::sm_count() * 8;
    detail::k_pull_rows<P, (int) detail::kSmallLanes><<<grid, 256, 0, s_>>>(prog_, v_, rs.small, rs.cnt, st);
    detail::k_pull_rows<P, 32><<<grid, 256, 0, s_>>>(prog_, v_, rs.mid, rs.cnt + 1, st);
    if constexpr (kAssoc)
    {
      detail::k_pull_tasks<P><<<grid, 256, 0, s_>>>(prog_, v_, rs, st, (Acc*) part_, (uint8_t*) part_ok_);
      detail::k_hub_apply<P><<<detail::sm_count(), 256, 0, s_>>>(prog_, v_, rs, st, (const Acc*) part_,
                                                                 (const uint8_t*) part_ok_);
    }
    ck(cudaGetLastError());
  }

  template <class I, class V, class Map, class Cmp, bool BATCH>
  int topk_impl(uint32_t k, uint32_t nb, std::vector<std::pair<I, V>>* out, Map map, Cmp cmp, bool active_only)
  {
    using Item = detail::TopItem<I, V>;
    if (status_ != LA3G_OK) return status_;
    if (k == 0 || k > detail::kTopkMaxK) return fail(LA3G_EINVAL, "topk: k must be in [1, 512]");
    const uint32_t T = detail::kTopkTile;
    uint32_t n = dv_.nslots;
    uint32_t tiles = (n + T - 1) / T;
    void* bufs[2] = {nullptr, nullptr};
    const size_t cap = (size_t) nb * (size_t) tiles * k;
    if (cudaMalloc(&bufs[0], cap * sizeof(Item)) != cudaSuccess || cudaMalloc(&bufs[1], cap * sizeof(Item)) != cudaSuccess)
    {
      cudaGetLastError();
      cudaFree(bufs[0]);
      return fail(LA3G_ENOMEM, "topk");
    }
    // the first pass maps the vertices; every pass keeps k items per tile
    detail::k_topk_round<P, I, V, Map, Cmp, BATCH><<<dim3(tiles, nb), T / 2, 0, s_>>>(
        map, cmp, k, n, (const State*) S_, dv_.id_of_pos, (const uint8_t*) vact_, active_only, nullptr, (Item*) bufs[0]);
    ck(cudaGetLastError());
    int cur = 0;
    n = tiles * k;
    while (tiles > 1)
    {
      tiles = (n + T - 1) / T;
      detail::k_topk_round<P, I, V, Map, Cmp, BATCH><<<dim3(tiles, nb), T / 2, 0, s_>>>(
          map, cmp, k, n, nullptr, nullptr, nullptr, false, (const Item*) bufs[cur], (Item*) bufs[cur ^ 1]);
      ck(cudaGetLastError());
      cur ^= 1;
      n = tiles * k;
    }
    detail::k_topk_pad<I, V, Cmp><<<nb, 1, 0, s_>>>(cmp, k, (Item*) bufs[cur]);
    ck(cudaGetLastError());
    std::vector<Item> h((size_t) nb * k);
    ck(cudaMemcpyAsync(h.data(), bufs[cur], h.size() * sizeof(Item), cudaMemcpyDeviceToHost, s_));
    const int st = sync();
    cudaFree(bufs[0]);
    cudaFree(bufs[1]);
    if (st != LA3G_OK) return st;
    for (uint32_t b = 0; b < nb; b++)
    {
      out[b].clear();
      for (uint32_t t = 0; t < k; t++) out[b].emplace_back(h[(size_t) b * k + t].i, h[(size_t) b * k + t].v);
    }
    return LA3G_OK;
  }

  // Variable-size messages of the n vertices base.. whose act flag is set:
  // lengths, exclusive scan, arena `which` (0 / 1 regular ping-pong, 2
  // sources) grown to the total, then elements and views.  One host round
  // trip (the total) per call.
  void fill_messages(uint32_t n, uint32_t base, void* act, void* views, int which)
  {
    if constexpr (detail::VarMsg<P>::value)
    {
      using Elem = typename P::Elem;
      if (status_ != LA3G_OK || n == 0) return;
      if (!mlen_)
      {
        alloc(&mlen_, (size_t) (dv_.nslots + 2) * 8);
        alloc(&moff_, (size_t) (dv_.nslots + 2) * 8);
        if (status_ != LA3G_OK) return;
      }
      unsigned long long* len = (unsigned long long*) mlen_;
      unsigned long long* off = (unsigned long long*) moff_;
      ck(cudaMemsetAsync(len + n, 0, 8, s_));
      detail::k_msg_len<P><<<detail::blocks_for(n), 256, 0, s_>>>(prog_, n, base, (const State*) S_,
                                                                   (const uint8_t*) act, len);
      ck(cudaGetLastError());
      size_t tb = 0;
      ck(cub::DeviceScan::ExclusiveSum(nullptr, tb, len, off, (int64_t) n + 1, s_));
      if (tb > scan_bytes_)
      {
        if (scan_tmp_) cudaFree(scan_tmp_);
        scan_tmp_ = nullptr;
        if (cudaMalloc(&scan_tmp_, tb) != cudaSuccess)
        {
          cudaGetLastError();
          fail(LA3G_ENOMEM, "message scan");
          return;
        }
        scan_bytes_ = tb;
      }
      ck(cub::DeviceScan::ExclusiveSum(scan_tmp_, tb, len, off, (int64_t) n + 1, s_));
      unsigned long long total = 0;
      ck(cudaMemcpyAsync(&total, off + n, 8, cudaMemcpyDeviceToHost, s_));
      if (sync() != LA3G_OK) return;
      if (total > arena_cap_[which])
      {
        if (arena_[which]) cudaFree(arena_[which]);
        arena_[which] = nullptr;
        arena_cap_[which] = 0;
        const size_t cap = (size_t) total + total / 2 + 16;
        if (cudaMalloc(&arena_[which], cap * sizeof(Elem)) != cudaSuccess)
        {
          cudaGetLastError();
          fail(LA3G_ENOMEM, "message arena");
          return;
        }
        arena_cap_[which] = cap;
      }
      detail::k_msg_fill<P><<<detail::blocks_for(n), 256, 0, s_>>>(prog_, n, base, (const State*) S_,
                                                                    (const uint8_t*) act, off, (Elem*) arena_[which],
                                                                    (Msg*) views);
      ck(cudaGetLastError());
    }
    else
    {
      (void) n;
      (void) base;
      (void) act;
      (void) views;
      (void) which;
    }
  }

  void make_rowset(detail::RowSet* rs, uint32_t n)
  {
    void *a = nullptr, *b = nullptr, *c = nullptr, *d = nullptr, *e = nullptr;
    alloc(&a, (size_t) (n + 1) * 4);
    alloc(&b, (size_t) (n + 1) * 4);
    const size_t nh = kAssoc ? (size_t) (n < dv_.nentries / detail::kHubDeg + 1 ? n : dv_.nentries / detail::kHubDeg + 1) : 0;
    alloc(&c, (nh + 1) * 4);
    alloc(&d, (nh + 1) * 4);
    alloc(&e, 4 * sizeof(unsigned long long));
    *rs = detail::RowSet{(uint32_t*) a, (uint32_t*) b, (uint32_t*) c, (uint32_t*) d, (unsigned long long*) e};
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
  void *xs_ = nullptr, *xsa_ = nullptr, *active_ = nullptr, *vact_ = nullptr, *ctr_ = nullptr;
  void *front_[2] = {nullptr, nullptr}, *srcs_ = nullptr, *bits_ = nullptr, *part_ = nullptr, *part_ok_ = nullptr;
  detail::RowSet sets_[3] = {};  // dense regular rows, dense sink rows, the sparse step's rows
  uint64_t nfront_ = 0, front_deg_ = 0, nsrc_act_ = 0, src_deg_ = 0;
  uint32_t sparse_steps_ = 0, dense_steps_ = 0;
  // variable-size messages: arenas (regular ping-pong, sources), lengths, offsets, scan space
  void* arena_[3] = {nullptr, nullptr, nullptr};
  size_t arena_cap_[3] = {0, 0, 0};
  void *mlen_ = nullptr, *moff_ = nullptr, *scan_tmp_ = nullptr;
  size_t scan_bytes_ = 0;
  std::vector<void*> owned_;
  int status_ = LA3G_OK;
  char msg_[160] = {0};
};

}  // namespace la3g_vp

#endif
