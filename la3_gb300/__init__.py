"""la3_gb300 — GB300-native LA3 vertex-program engine (host-side mirror).

The reference's user-facing surface is the `Graph<W>::load_*` calls
(src/matrix/graph.h:38-47) and the apps' `run()` functions (pr, bfs, sssp,
cc, tc, degree: src/apps/graph_analytics/*.cpp; bm25, lm:
src/apps/information_retrieval/*.cpp; graph simulation's input readers:
src/apps/graph_simulation/).
This module exposes the same loads and apps over the native C ABI
(include/la3g.h); every result is a numpy array indexed by vertex id with
n + 1 slots, as the reference's per-vertex states are.

Nothing here computes on the CPU: every call goes to libla3g, which runs
on the GPU, and a missing library raises at first use.
"""
from __future__ import annotations

import ctypes as C
import weakref
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _native as N
from ._native import LA3GError, Stats

DIRECTED = 1
REVERSE = 2
ACYCLIC = 4
BIPARTITE = 8
WEIGHTED = 16

SSSP_INF = 0x7FFFFFFF
BFS_INF = 255


def _ptr(a: Optional[np.ndarray], ctype):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


def _addr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


@dataclass
class Info:
    nslots: int
    nvertices: int
    nleft: int
    flags: int
    nrecords: int
    nentries: int
    nregular: int
    nsink: int
    nsource: int
    nisolated: int
    device_bytes: int


class Graph:
    """A device-resident graph (Graph<W> + its CSCMatrix2D in the reference)."""

    def __init__(self, handle: C.c_void_p, flags: int):
        self._h = handle
        self.flags = flags
        self.info = self._info()

    # -- loads (graph.hpp:224-258) ------------------------------------------
    @classmethod
    def load(cls, path: str, n: int, flags: int, nright: int = 0) -> "Graph":
        h = C.c_void_p()
        N.check(N.lib().la3g_graph_load(str(path).encode(), n, nright, flags, C.byref(h)))
        return cls(h, flags)

    @classmethod
    def load_directed(cls, path: str, n: int, reverse_edges: bool = False, remove_cycles: bool = False,
                      weighted: bool = False) -> "Graph":
        f = DIRECTED | (REVERSE if reverse_edges else 0) | (ACYCLIC if remove_cycles else 0)
        return cls.load(path, n, f | (WEIGHTED if weighted else 0))

    @classmethod
    def load_undirected(cls, path: str, n: int, weighted: bool = False) -> "Graph":
        return cls.load(path, n, WEIGHTED if weighted else 0)

    @classmethod
    def load_bipartite(cls, path: str, ndocs: int, nterms: int, directed: bool = False,
                       weighted: bool = True) -> "Graph":
        f = BIPARTITE | (DIRECTED if directed else 0) | (WEIGHTED if weighted else 0)
        return cls.load(path, ndocs, f, nright=nterms)

    @classmethod
    def from_records(cls, records: np.ndarray, n: int, flags: int, nright: int = 0) -> "Graph":
        rec = np.ascontiguousarray(records, dtype=np.uint32)
        wpr = 3 if flags & WEIGHTED else 2
        if rec.size % wpr:
            raise ValueError("records must hold whole records")
        h = C.c_void_p()
        N.check(N.lib().la3g_graph_from_records(rec.ctypes.data_as(C.c_void_p), rec.size // wpr, n, nright, flags,
                                                C.byref(h)))
        return cls(h, flags)

    @classmethod
    def from_edges(cls, edges: "EdgeList", flags: int, n: int = 0, nright: int = 0) -> "Graph":
        h = C.c_void_p()
        N.check(N.lib().la3g_graph_from_edges(C.byref(edges._e), n, nright, flags, C.byref(h)))
        return cls(h, flags)

    def _info(self) -> Info:
        gi = N.GraphInfo()
        N.check(N.lib().la3g_graph_info_get(self._h, C.byref(gi)))
        return Info(**{k: getattr(gi, k) for k, _ in gi._fields_})

    @property
    def nslots(self) -> int:
        return self.info.nslots

    def set_stream(self, cuda_stream: int | None) -> None:
        """Run subsequent calls on the given cudaStream_t (an int handle, e.g.
        torch.cuda.current_stream().cuda_stream); None = the graph's own."""
        N.check(N.lib().la3g_graph_set_stream(self._h, C.c_void_p(cuda_stream) if cuda_stream else None))

    def positions(self) -> tuple[np.ndarray, np.ndarray]:
        pos = np.empty(self.nslots, np.uint32)
        ids = np.empty(self.nslots, np.uint32)
        N.check(N.lib().la3g_graph_positions(self._h, _ptr(pos, C.c_uint32), _ptr(ids, C.c_uint32)))
        return pos, ids

    def free(self) -> None:
        # servers that hold this graph go first (they must not outlive it)
        for ref in getattr(self, "_servers", ()):
            srv = ref()
            if srv is not None:
                srv.free()
        if self._h:
            N.lib().la3g_graph_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.free()


# -- apps ------------------------------------------------------------------

def pagerank(G: Graph, iters: int, want_rank: bool = True, want_degree: bool = True):
    """pr.cpp:11-55: FP64 ranks (bit-identical to the reference) + out-degrees."""
    st = Stats()
    rank = np.empty(G.nslots, np.float64) if want_rank else None
    deg = np.empty(G.nslots, np.uint32) if want_degree else None
    N.check(N.lib().la3g_pr(G._h, iters, _ptr(rank, C.c_double), _ptr(deg, C.c_uint32), C.byref(st)))
    return rank, deg, st


def pagerank_f32(G: Graph, iters: int, tol: float = 0.0, tiled: bool = False):
    """FP32 SpMV / FP32 accumulation variant; returns (rank as f64, L1 residual, stats).
    tiled: run over the tiled DCSC copy of the matrix (la3g_pr_f32_tiled)."""
    st = Stats()
    rank = np.empty(G.nslots, np.float64)
    res = C.c_double(0.0)
    f = N.lib().la3g_pr_f32_tiled if tiled else N.lib().la3g_pr_f32
    N.check(f(G._h, iters, tol, _ptr(rank, C.c_double), C.byref(res), C.byref(st)))
    return rank, res.value, st


def bfs(G: Graph, root: int, want_hops: bool = True, want_parent: bool = True):
    """bfs.cpp:11-37: (hops uint8 with 255 = unreached, parent hashed id, stats)."""
    st = Stats()
    hops = np.empty(G.nslots, np.uint8) if want_hops else None
    parent = np.empty(G.nslots, np.uint32) if want_parent else None
    N.check(N.lib().la3g_bfs(G._h, root, _ptr(hops, C.c_uint8), _ptr(parent, C.c_uint32), C.byref(st)))
    return hops, parent, st


def sssp(G: Graph, root: int, want_dist: bool = True):
    """sssp.cpp:11-37: uint32 distances, 2147483647 = unreached."""
    st = Stats()
    dist = np.empty(G.nslots, np.uint32) if want_dist else None
    N.check(N.lib().la3g_sssp(G._h, root, _ptr(dist, C.c_uint32), C.byref(st)))
    return dist, st


def cc(G: Graph, want_labels: bool = True):
    """cc.cpp:11-31: component labels."""
    st = Stats()
    lab = np.empty(G.nslots, np.uint32) if want_labels else None
    N.check(N.lib().la3g_cc(G._h, _ptr(lab, C.c_uint32), C.byref(st)))
    return lab, st


def tc(G: Graph, want_per_vertex: bool = True):
    """tc.cpp:11-52: (total, per-vertex middle-vertex counts, stats)."""
    st = Stats()
    total = C.c_uint64(0)
    per = np.empty(G.nslots, np.uint32) if want_per_vertex else None
    N.check(N.lib().la3g_tc(G._h, C.byref(total), _ptr(per, C.c_uint32), C.byref(st)))
    return total.value, per, st


def degree(G: Graph, k: int = 3):
    """degree.cpp:16-46: in-degrees (out-degrees on a graph loaded with
    reverse_edges) by id, and the top k (degree desc, id asc)."""
    deg = np.empty(G.nslots, np.uint32)
    ids = np.empty(max(k, 1), np.uint32)
    vals = np.empty(max(k, 1), np.uint32)
    n = C.c_uint32(0)
    st = Stats()
    N.check(N.lib().la3g_degree(G._h, _ptr(deg, C.c_uint32), k, _ptr(ids, C.c_uint32), _ptr(vals, C.c_uint32),
                                C.byref(n), C.byref(st)))
    return deg, ids[:n.value].copy(), vals[:n.value].copy(), st


def topk_u32(values: np.ndarray, k: int):
    """Top k of a uint32 array on the device: (indices, values), value desc,
    index asc."""
    v = np.ascontiguousarray(np.asarray(values, np.uint32))
    ids = np.empty(max(k, 1), np.uint32)
    vals = np.empty(max(k, 1), np.uint32)
    n = C.c_uint32(0)
    N.check(N.lib().la3g_topk_u32(_ptr(v, C.c_uint32), v.size, k, _ptr(ids, C.c_uint32), _ptr(vals, C.c_uint32),
                                  C.byref(n)))
    return ids[:n.value].copy(), vals[:n.value].copy()


def _strtok(s: str, delims: str):
    """C strtok on one string: skip leading delimiters, cut at the next one;
    returns (token or None, rest)."""
    i = 0
    while i < len(s) and s[i] in delims:
        i += 1
    if i == len(s):
        return None, ""
    j = i
    while j < len(s) and s[j] not in delims:
        j += 1
    return s[i:j], s[j + 1:]


def read_graphsim_labels(path: str, nvertices: int) -> list[str]:
    """Data-graph labels (graphsim.cpp:14-40): a first line "[", then one
    line per vertex 0..nvertices-1 of the form {"key":"label"}, whose label
    is taken as C strtok takes it (the text after the first ':' minus its
    first character, up to the next '"'); a first line "null," leaves vertex
    0 without a label.  Vertex nvertices never has one."""
    labels = [""] * nvertices
    with open(path, "rb") as f:
        lines = f.read().decode("latin-1").split("\n")
    for i in range(nvertices):
        line = lines[i + 1].rstrip("\r") if i + 1 < len(lines) else ""
        line = line[:2047]
        if i == 0 and line == "null,":
            continue
        t, rest = _strtok(line, ":")
        if t is None:
            continue
        t, _ = _strtok(rest, ":")
        if t is None:
            continue
        t, _ = _strtok(t[1:], '"')
        if t is not None:
            labels[i] = t
    return labels


def read_graphsim_query(labels_path: str, mtx_path: str) -> tuple[list[str], list[tuple[int, int]]]:
    """Query graph (graphsim_query.h:17-52): labels are whitespace-separated
    tokens read with `while (!eof) { fin >> label; push }`, so a file that
    ends in whitespace, or holds no token, yields one more, empty, label; the
    matrix file holds pairs "i j" (edge i -> j), kept in file order."""
    with open(labels_path, "rb") as f:
        text = f.read().decode("latin-1")
    toks = text.split()
    labels = list(toks)
    if not toks or text[-1:].isspace():
        labels.append("")
    with open(mtx_path) as f:
        nums = [int(x) for x in f.read().split()]
    edges = [(nums[2 * k], nums[2 * k + 1]) for k in range(len(nums) // 2)]
    return labels, edges


def graphsim_label_ids(vertex_labels: Sequence[str], query_labels: Sequence[str], nslots: int):
    """Integer label ids, 0 for the empty string (no label), equal strings
    equal ids: (per-vertex ids, nslots long, and the query's ids)."""
    ids = {"": 0}
    def lid(s):
        return ids.setdefault(s, len(ids))
    v = np.zeros(nslots, np.uint32)
    for i, s in enumerate(vertex_labels):
        v[i] = lid(s)
    q = np.array([lid(s) for s in query_labels], np.uint32)
    return v, q


class BM25:
    """bm25.cpp:8-114 over a bipartite graph: prepare once, then query."""

    def __init__(self, G: Graph, want_length: bool = False):
        self.G = G
        ntok = C.c_uint64(0)
        avg = C.c_float(0)
        self.length = np.empty(G.nslots, np.float32) if want_length else None
        N.check(N.lib().la3g_bm25_prepare(G._h, C.byref(ntok), C.byref(avg), _ptr(self.length, C.c_float)))
        self.collection_ntokens = ntok.value
        self.avg_doc_length = avg.value

    def query(self, term_vids: Sequence[int], k: int = 10, full: bool = False):
        q = np.ascontiguousarray(np.asarray(term_vids, dtype=np.uint32))
        ids = np.empty(max(k, 1), np.uint32)
        scores = np.empty(max(k, 1), np.float32)
        nout = C.c_uint32(0)
        st = Stats()
        alls = np.empty(self.G.nslots, np.float32) if full else None
        act = np.empty(self.G.nslots, np.uint8) if full else None
        N.check(N.lib().la3g_bm25_query(self.G._h, _ptr(q, C.c_uint32), q.size, k, _ptr(ids, C.c_uint32),
                                        _ptr(scores, C.c_float), C.byref(nout), _ptr(alls, C.c_float),
                                        _ptr(act, C.c_uint8), C.byref(st)))
        n = nout.value
        return ids[:n].copy(), scores[:n].copy(), (alls, act), st


class LM:
    """lm.cpp:8-144 (query likelihood, Dirichlet smoothing) over a bipartite
    graph: prepare once, then query (same interface as BM25)."""

    def __init__(self, G: Graph, want_length: bool = False):
        self.G = G
        ntok = C.c_uint64(0)
        self.length = np.empty(G.nslots, np.float32) if want_length else None
        N.check(N.lib().la3g_lm_prepare(G._h, C.byref(ntok), _ptr(self.length, C.c_float)))
        self.collection_ntokens = ntok.value

    def query(self, term_vids: Sequence[int], k: int = 10, full: bool = False):
        q = np.ascontiguousarray(np.asarray(term_vids, dtype=np.uint32))
        ids = np.empty(max(k, 1), np.uint32)
        scores = np.empty(max(k, 1), np.float32)
        nout = C.c_uint32(0)
        st = Stats()
        alls = np.empty(self.G.nslots, np.float32) if full else None
        act = np.empty(self.G.nslots, np.uint8) if full else None
        N.check(N.lib().la3g_lm_query(self.G._h, _ptr(q, C.c_uint32), q.size, k, _ptr(ids, C.c_uint32),
                                      _ptr(scores, C.c_float), C.byref(nout), _ptr(alls, C.c_float),
                                      _ptr(act, C.c_uint8), C.byref(st)))
        n = nout.value
        return ids[:n].copy(), scores[:n].copy(), (alls, act), st


def read_queries(labels_path: str, queries_path: str, ndocs: int) -> list[list[int]]:
    """prepare_queries (helpers.hpp:76-123): the label on line i of the term
    labels file is term vertex ndocs + i + 1; each query line is a list of
    labels; a label that is not in the file maps to vertex 0."""
    ids = {}
    with open(labels_path) as f:
        i = 0
        for line in f:
            parts = line.split()
            if not parts:
                continue
            ids[parts[0]] = i + 1 + ndocs
            i += 1
    out = []
    with open(queries_path) as f:
        for line in f:
            toks = line.split()
            if toks:
                out.append([ids.get(t, 0) for t in toks])
    return out


QUERY_BFS, QUERY_SSSP, QUERY_BM25, QUERY_LM = 1, 2, 3, 4


class Server:
    """Serving loop over resident graphs (la3g_server_*): queries are queued
    with submit_* and collected with poll; BFS / SSSP queries of one graph
    share its engine's lanes (continuous batching), each graph runs on its
    own worker and stream."""

    def __init__(self, budget_bytes: int, bfs_lanes: int = 0, sssp_lanes: int = 0):
        h = C.c_void_p()
        N.check(N.lib().la3g_server_create(budget_bytes, bfs_lanes, sssp_lanes, C.byref(h)))
        self._h = h
        self._graphs = {}
        self._live = {}  # ticket -> output buffers (kept alive until polled)

    def add_graph(self, G: Graph) -> int:
        gid = C.c_uint32()
        N.check(N.lib().la3g_server_add_graph(self._h, G._h, C.byref(gid)))
        self._graphs[gid.value] = G
        if not hasattr(G, "_servers"):
            G._servers = []
        G._servers.append(weakref.ref(self))
        return gid.value

    def set_solo(self, bfs_depth: int, sssp_depth: int) -> None:
        """Adaptive batching depths (0, 0 = always lanes)."""
        N.check(N.lib().la3g_server_set_solo(self._h, bfs_depth, sssp_depth))

    def lanes(self, gid: int) -> int:
        n = C.c_uint32()
        N.check(N.lib().la3g_server_lanes(self._h, gid, C.byref(n)))
        return n.value

    def _submit(self, q, bufs) -> int:
        t = C.c_uint64()
        N.check(N.lib().la3g_server_submit(self._h, C.byref(q), C.byref(t)))
        self._live[t.value] = bufs
        return t.value

    def _graph(self, gid: int) -> Graph:
        G = self._graphs.get(gid)
        if G is None:
            raise LA3GError(1, f"no such graph id {gid}")
        return G

    def submit_bfs(self, gid: int, root: int, want: bool = True) -> int:
        out = np.empty(self._graph(gid).nslots, np.uint8) if want else None
        q = N.Query(kind=QUERY_BFS, graph=gid, root=root, out=_addr(out))
        return self._submit(q, (out,))

    def submit_sssp(self, gid: int, root: int, want: bool = True) -> int:
        out = np.empty(self._graph(gid).nslots, np.uint32) if want else None
        q = N.Query(kind=QUERY_SSSP, graph=gid, root=root, out=_addr(out))
        return self._submit(q, (out,))

    def submit_bm25(self, gid: int, term_vids: Sequence[int], k: int = 10, kind: int = QUERY_BM25) -> int:
        terms = np.ascontiguousarray(term_vids, dtype=np.uint32)
        ids = np.zeros(k, np.uint32)
        sc = np.zeros(k, np.float32)
        q = N.Query(kind=kind, graph=gid, k=k, terms=_ptr(terms, C.c_uint32), nterms=terms.size,
                    out=_addr(ids), scores_out=_ptr(sc, C.c_float))
        return self._submit(q, (ids, sc))

    def submit_lm(self, gid: int, term_vids: Sequence[int], k: int = 10) -> int:
        """An LM query on a served corpus (the corpus's first-query leftover
        activity is taken at add_graph, so every LM query sees the steady
        state)."""
        return self.submit_bm25(gid, term_vids, k, kind=QUERY_LM)

    def poll(self, ticket: int, timeout_ms: int = -1):
        """(result struct, outputs) when done, None while pending."""
        r = N.QueryResult()
        st = N.lib().la3g_server_poll(self._h, ticket, timeout_ms, C.byref(r))
        if st == 8:  # LA3G_EBUSY
            return None
        N.check(st)
        bufs = self._live.pop(ticket)
        if r.kind in (QUERY_BM25, QUERY_LM):
            bufs = (bufs[0][: r.nout], bufs[1][: r.nout])
        return r, bufs

    def info(self) -> dict:
        s = N.ServerStats()
        N.check(N.lib().la3g_server_info(self._h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in N.ServerStats._fields_ if f != "reserved"}

    def free(self) -> None:
        if self._h:
            N.lib().la3g_server_free(self._h)
            self._h = None
            self._live.clear()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def bfs_batch(G: Graph, roots: Sequence[int], want_hops: bool = True):
    r = np.ascontiguousarray(np.asarray(roots, dtype=np.uint32))
    st = Stats()
    hops = np.empty((r.size, G.nslots), np.uint8) if want_hops else None
    N.check(N.lib().la3g_bfs_batch(G._h, _ptr(r, C.c_uint32), r.size, _ptr(hops, C.c_uint8), C.byref(st)))
    return hops, st


def batch_autotune(G: Graph, roots: Sequence[int]) -> list:
    """Times the batched-BFS configurations on `roots`; keeps the best on G."""
    import json
    r = np.ascontiguousarray(np.asarray(roots, dtype=np.uint32))
    buf = C.create_string_buffer(1 << 14)
    N.check(N.lib().la3g_batch_autotune(G._h, _ptr(r, C.c_uint32), r.size, buf, len(buf)))
    return json.loads(buf.value.decode())


def batch_config(G: Graph, mode: int, block: int = 256, push_frac: float = 0.05) -> None:
    """mode 0: per-level CUDA graph; 1: persistent kernel."""
    N.check(N.lib().la3g_batch_config(G._h, mode, block, push_frac))


def batch_set_wait_limit(G: Graph, polls: int = -1) -> None:
    """Grid-barrier poll limit of the persistent batched-BFS kernel (< 0: the default)."""
    N.check(N.lib().la3g_batch_set_wait_limit(G._h, polls))


def batch_sssp_window(G: Graph, delta: int = 0) -> None:
    """Distance window of the batched SSSP (0: from the largest weight;
    0xFFFFFFFF: none).  Results do not depend on it."""
    N.check(N.lib().la3g_batch_sssp_window(G._h, delta))


def sssp_batch(G: Graph, roots: Sequence[int], want_dist: bool = True):
    r = np.ascontiguousarray(np.asarray(roots, dtype=np.uint32))
    st = Stats()
    dist = np.empty((r.size, G.nslots), np.uint32) if want_dist else None
    N.check(N.lib().la3g_sssp_batch(G._h, _ptr(r, C.c_uint32), r.size, _ptr(dist, C.c_uint32), C.byref(st)))
    return dist, st


# -- synthetic inputs ---------------------------------------------------------

class EdgeList:
    """A generator's edge list (host memory owned by libla3g)."""

    def __init__(self):
        self._e = N.Edges()

    @classmethod
    def rmat(cls, scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             seed: int = 1, weighted: bool = False, wseed: int = 2) -> "EdgeList":
        e = cls()
        N.check(N.lib().la3g_gen_rmat(scale, edge_factor, a, b, c, seed, int(weighted), wseed, C.byref(e._e)))
        return e

    @classmethod
    def er(cls, n: int, m: int, seed: int = 1, weighted: bool = False, wseed: int = 2) -> "EdgeList":
        e = cls()
        N.check(N.lib().la3g_gen_er(n, m, seed, int(weighted), wseed, C.byref(e._e)))
        return e

    @classmethod
    def bipartite(cls, ndocs: int, nterms: int, terms_per_doc: int = 50, zipf_s: float = 1.1, df_cap: float = 0.9,
                  seed: int = 1) -> "EdgeList":
        e = cls()
        N.check(N.lib().la3g_gen_bipartite(ndocs, nterms, terms_per_doc, zipf_s, df_cap, seed, C.byref(e._e)))
        return e

    @property
    def m(self) -> int:
        return self._e.m

    @property
    def n(self) -> int:
        return self._e.n

    @property
    def nright(self) -> int:
        return self._e.nright

    def arrays(self) -> tuple[np.ndarray, np.ndarray, Optional[np.ndarray]]:
        m = self._e.m
        src = np.ctypeslib.as_array(self._e.src, shape=(m,)).copy() if m else np.empty(0, np.uint32)
        dst = np.ctypeslib.as_array(self._e.dst, shape=(m,)).copy() if m else np.empty(0, np.uint32)
        w = None
        if self._e.weighted and m:
            w = np.ctypeslib.as_array(self._e.w, shape=(m,)).copy()
        return src, dst, w

    def write(self, path: str, header: bool = False) -> None:
        N.check(N.lib().la3g_edges_write(C.byref(self._e), str(path).encode(), int(header)))

    def free(self) -> None:
        N.lib().la3g_edges_free(C.byref(self._e))

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def profile(on: bool = True) -> None:
    N.lib().la3g_profile_enable(int(on))


def profile_reset() -> None:
    N.lib().la3g_profile_reset()


def profile_report() -> dict:
    import json
    L = N.lib()
    n = L.la3g_profile_report(None, 0)
    buf = C.create_string_buffer(n + 1)
    L.la3g_profile_report(buf, n + 1)
    return json.loads(buf.value.decode())


__all__ = ["Graph", "EdgeList", "BM25", "LA3GError", "Stats", "pagerank", "pagerank_f32", "bfs", "sssp", "cc", "tc",
           "LM", "degree", "topk_u32", "read_graphsim_labels", "read_graphsim_query", "graphsim_label_ids", "bfs_batch", "sssp_batch", "batch_autotune", "batch_config", "batch_set_wait_limit", "batch_sssp_window", "read_queries", "profile", "profile_reset", "profile_report", "DIRECTED", "REVERSE", "ACYCLIC",
           "BIPARTITE", "WEIGHTED", "SSSP_INF", "BFS_INF"]
