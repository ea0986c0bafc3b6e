"""The vertex-program API (include/la3g_vp.cuh): the reference's apps written
as device-functor programs (la3_gb300/programs/vp_apps.cu) and run by the
generic engine must give the reference's results bit for bit: the golden
cases, and seeded graphs against the oracle."""
import ctypes as C

import numpy as np
import pytest

from conftest import GOLD

DATA = GOLD / "data"
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def progs(gpu):
    import la3_gb300.build as B
    lib = C.CDLL(str(B.PROGRAMS_LIB))
    P = C.c_void_p
    u8p, u32p, f64p = C.POINTER(C.c_uint8), C.POINTER(C.c_uint32), C.POINTER(C.c_double)
    lib.la3gp_pagerank.argtypes = [P, P, C.c_uint32, f64p, u32p]
    lib.la3gp_bfs.argtypes = [P, C.c_uint32, u8p, u32p, u32p]
    lib.la3gp_sssp.argtypes = [P, C.c_uint32, u32p, u32p]
    lib.la3gp_cc.argtypes = [P, u32p, u32p]
    lib.la3gp_degree.argtypes = [P, u32p]
    lib.la3gp_graphsim.argtypes = [P, u32p, C.c_uint32, u32p, u32p, C.c_uint32, u8p, C.c_char_p, u32p, u32p]
    return lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def _pr(L, progs, path, n, iters):
    g = L.Graph.load_directed(path, n)
    gr = L.Graph.load_directed(path, n, reverse_edges=True)
    rank = np.empty(g.nslots, np.float64)
    deg = np.empty(g.nslots, np.uint32)
    assert progs.la3gp_pagerank(g._h, gr._h, iters, _p(rank, C.c_double), _p(deg, C.c_uint32)) == 0
    return rank, deg


def _bfs(L, progs, g, root):
    hops = np.empty(g.nslots, np.uint8)
    par = np.empty(g.nslots, np.uint32)
    it = C.c_uint32()
    assert progs.la3gp_bfs(g._h, root, _p(hops, C.c_uint8), _p(par, C.c_uint32), C.byref(it)) == 0
    return hops, par, it.value


def _sssp(L, progs, g, root):
    d = np.empty(g.nslots, np.uint32)
    it = C.c_uint32()
    assert progs.la3gp_sssp(g._h, root, _p(d, C.c_uint32), C.byref(it)) == 0
    return d, it.value


def _cc(L, progs, g):
    lab = np.empty(g.nslots, np.uint32)
    it = C.c_uint32()
    assert progs.la3gp_cc(g._h, _p(lab, C.c_uint32), C.byref(it)) == 0
    return lab, it.value


def _cases(golden, app):
    return sorted(k for k, v in golden.items() if v["app"] == app)


def test_programs_golden(gpu, progs, golden):
    L = gpu
    for name in _cases(golden, "pr"):
        c = golden[name]
        ref = np.load(GOLD / f"{name}.npz")
        rank, deg = _pr(L, progs, DATA / c["file"], c["n"], c["iters"])
        assert np.array_equal(deg, ref["degree"]), name
        assert np.array_equal(rank.view(np.uint64), ref["rank"].view(np.uint64)), name
    for name in _cases(golden, "bfs"):
        c = golden[name]
        ref = np.load(GOLD / f"{name}.npz")
        hops, par, _ = _bfs(L, progs, L.Graph.load_undirected(DATA / c["file"], c["n"]), c["root"])
        assert np.array_equal(hops, ref["hops"]) and np.array_equal(par, ref["parent"]), name
    for name in _cases(golden, "sssp"):
        c = golden[name]
        ref = np.load(GOLD / f"{name}.npz")
        d, _ = _sssp(L, progs, L.Graph.load_directed(DATA / c["file"], c["n"], weighted=True), c["root"])
        assert np.array_equal(d, ref["dist"]), name
    for name in _cases(golden, "cc"):
        c = golden[name]
        ref = np.load(GOLD / f"{name}.npz")
        lab, _ = _cc(L, progs, L.Graph.load_undirected(DATA / c["file"], c["n"]))
        assert np.array_equal(lab, ref["label"]), name


def test_programs_vs_oracle_rmat(gpu, progs, oracle, tmp_path):
    L = gpu
    e = L.EdgeList.rmat(13, 16, seed=41)
    ew = L.EdgeList.rmat(13, 16, seed=41, weighted=True, wseed=42)
    p, pw, n = tmp_path / "g.bin", tmp_path / "g.w.bin", 1 << 13
    e.write(p)
    ew.write(pw)
    rank, deg = _pr(L, progs, p, n, 10)
    orank, odeg = oracle.OracleGraph(p, n, oracle.DIRECTED).pagerank(10)
    assert np.array_equal(deg, odeg)
    assert np.array_equal(rank.view(np.uint64), orank.view(np.uint64))
    gu = L.Graph.load_undirected(p, n)
    ou = oracle.OracleGraph(p, n, 0)
    for r in (1, 77, 4000):
        hops, par, it = _bfs(L, progs, gu, r)
        oh, opar, oit = ou.bfs(r)
        assert np.array_equal(hops, oh) and np.array_equal(par, opar) and it == oit, r
    gw = L.Graph.load_directed(pw, n, weighted=True)
    ow = oracle.OracleGraph(pw, n, oracle.DIRECTED | oracle.WEIGHTED)
    for r in (1, 77, 4000):
        d, it = _sssp(L, progs, gw, r)
        od, oit = ow.sssp(r)
        assert np.array_equal(d, od) and it == oit, r
    lab, it = _cc(L, progs, gu)
    olab, oit = ou.cc()
    assert np.array_equal(lab, olab) and it == oit


def _graphsim(L, progs, c):
    g = L.Graph.load_directed(DATA / c["file"], c["n"], reverse_edges=True)
    vl = L.read_graphsim_labels(DATA / c["labels"], c["n"])
    ql, qe = L.read_graphsim_query(DATA / c["qlabels"], DATA / c["qmtx"])
    v, q = L.graphsim_label_ids(vl, ql, g.nslots)
    e = np.ascontiguousarray(np.asarray(qe, np.uint32).reshape(-1))
    matched = np.empty(g.nslots, np.uint8)
    res = C.create_string_buffer(g.nslots * q.size)
    nm, it = C.c_uint32(), C.c_uint32()
    assert progs.la3gp_graphsim(g._h, _p(v, C.c_uint32), q.size, _p(q, C.c_uint32), _p(e, C.c_uint32), e.size // 2,
                                _p(matched, C.c_uint8), res, C.byref(nm), C.byref(it)) == 0
    return matched, np.frombuffer(res.raw, np.uint8).reshape(g.nslots, q.size), nm.value, it.value


def test_graphsim_golden(gpu, progs, golden):
    """Graph simulation (variable-size messages bounded at 32 query vertices)
    against the reference's per-vertex results: its sample data graph and
    queries and synthetic ones (incl. the empty query label a trailing
    newline adds, a vertex 0 without a label)."""
    for name in sorted(k for k, v in golden.items() if v["app"] == "graphsim"):
        c = golden[name]
        ref = np.load(GOLD / f"{name}.npz")
        matched, res, nm, _ = _graphsim(gpu, progs, c)
        assert nm == c["nmatches"], name
        assert np.array_equal(matched, ref["matched"]), name
        assert np.array_equal(res, ref["res"]), name


def test_graphsim_vs_oracle(gpu, progs, oracle, tmp_path):
    """A larger seeded case against the oracle: R-MAT s14, 6 labels, random
    queries with cycles."""
    L = gpu
    n = 1 << 14
    p = tmp_path / "g.bin"
    L.EdgeList.rmat(14, 8, seed=23).write(p)
    rng = np.random.default_rng(29)
    labs = ["A", "B", "C", "D", "E", "F"]
    (tmp_path / "g.labels").write_text("[\n" + "".join('{"x":"%s"},\n' % labs[int(rng.integers(0, 6))]
                                                       for _ in range(n)) + "]\n")
    og = oracle.OracleGraph(p, n, oracle.DIRECTED | oracle.REVERSE)
    for qi in range(4):
        qn = int(rng.integers(3, 8))
        (tmp_path / "q.labels").write_text(" ".join(labs[int(rng.integers(0, 6))] for _ in range(qn)))
        edges = {(int(rng.integers(0, qn)), int(rng.integers(0, qn))) for _ in range(2 * qn)}
        (tmp_path / "q.mtx").write_text("".join(f"{a} {b}\n" for a, b in sorted(edges) if a != b))
        c = {"file": p, "n": n, "labels": tmp_path / "g.labels", "qlabels": tmp_path / "q.labels",
             "qmtx": tmp_path / "q.mtx"}
        matched, res, nm, it = _graphsim(L, progs, c)
        vl = L.read_graphsim_labels(c["labels"], n)
        ql, qe = L.read_graphsim_query(c["qlabels"], c["qmtx"])
        v, q = L.graphsim_label_ids(vl, ql, og.nslots)
        om, ores, onm, oit = og.graphsim(v, q, qe)
        assert nm == onm and it == oit, qi
        assert np.array_equal(matched, om) and np.array_equal(res, ores), qi


def test_graphsim_driver(gpu, golden):
    import re
    import subprocess
    import la3_gb300.build as B
    for name in sorted(k for k, v in golden.items() if v["app"] == "graphsim"):
        c = golden[name]
        out = subprocess.run([str(B.BIN / "graphsim"), str(DATA / c["labels"]), str(DATA / c["file"]), str(c["n"]),
                              str(DATA / c["qlabels"]), str(DATA / c["qmtx"])], capture_output=True, text=True,
                             check=True).stdout
        assert int(re.search(r"Num matches = (\d+)", out).group(1)) == c["nmatches"], name
        shown = {int(a): b for a, b in re.findall(r"^(\d+): (\d*)$", out, flags=re.M)}
        ref = np.load(GOLD / f"{name}.npz")["matched"]
        assert all((shown[v] == str(v)) == bool(ref[v]) for v in shown), name



def test_programs_hub_rows_vs_oracle(gpu, progs, oracle, tmp_path):
    """R-MAT s17: rows with more in-edges than the engine's hub threshold
    (4096), so associative programs (BFS, SSSP, degree) cut them into tasks
    and combine the partials; PageRank (floating-point sums, not declared
    associative) keeps the edge-by-edge order.  Every result against the
    oracle."""
    L = gpu
    n = 1 << 17
    e = L.EdgeList.rmat(17, 16, seed=43)
    ew = L.EdgeList.rmat(17, 16, seed=43, weighted=True, wseed=44)
    p, pw = tmp_path / "g.bin", tmp_path / "g.w.bin"
    e.write(p)
    ew.write(pw)
    a = np.fromfile(p, np.uint32)
    assert np.bincount(a, minlength=n + 1).max() > 2 * 4096  # hubs in both directions
    rank, deg = _pr(L, progs, p, n, 5)
    orank, odeg = oracle.OracleGraph(p, n, oracle.DIRECTED).pagerank(5)
    assert np.array_equal(deg, odeg)
    assert np.array_equal(rank.view(np.uint64), orank.view(np.uint64))
    gu = L.Graph.load_undirected(p, n)
    ou = oracle.OracleGraph(p, n, 0)
    hub = int(np.bincount(a, minlength=n + 1).argmax())
    for r in (1, hub):
        hops, par, it = _bfs(L, progs, gu, r)
        oh, opar, oit = ou.bfs(r)
        assert np.array_equal(hops, oh) and np.array_equal(par, opar) and it == oit, r
    gw = L.Graph.load_directed(pw, n, weighted=True)
    ow = oracle.OracleGraph(pw, n, oracle.DIRECTED | oracle.WEIGHTED)
    for r in (1, hub):
        d, it = _sssp(L, progs, gw, r)
        od, oit = ow.sssp(r)
        assert np.array_equal(d, od) and it == oit, r


def _order(values, ids, pos_ids, desc=True):
    """Expected top-k order: value (largest first), ties by position."""
    keyed = sorted(range(len(pos_ids)), key=lambda p: (-int(values[p]) if desc else int(values[p]), p))
    return [int(pos_ids[p]) for p in keyed], [int(values[p]) for p in keyed]


def test_engine_topk_btopk_reduce(gpu, progs, tmp_path):
    """topk / btopk / reduce of the engine (vertex_program.hpp:558-767) on the
    degree app's states: the k largest in-degrees (ties in position order),
    btopk<2> over (degree, ~degree), and the degree sum."""
    L = gpu
    n = 1 << 14
    p = tmp_path / "g.bin"
    L.EdgeList.rmat(14, 8, seed=47).write(p)
    g = L.Graph.load_directed(p, n)
    deg = np.empty(g.nslots, np.uint32)
    assert progs.la3gp_degree(g._h, _p(deg, C.c_uint32)) == 0
    _, pos_ids = g.positions()
    dpos = deg[pos_ids]  # degree at each position
    u32p, u64p = C.POINTER(C.c_uint32), C.POINTER(C.c_uint64)
    progs.la3gp_degree_topk.argtypes = [C.c_void_p, C.c_uint32, u32p, u32p, u64p, u32p, u32p]
    for k in (1, 3, 10, 100, 512):
        ids = np.empty(k, np.uint32)
        vals = np.empty(k, np.uint32)
        bids = np.empty(2 * k, np.uint32)
        bvals = np.empty(2 * k, np.uint32)
        tot = C.c_uint64()
        assert progs.la3gp_degree_topk(g._h, k, _p(ids, C.c_uint32), _p(vals, C.c_uint32), C.byref(tot),
                                       _p(bids, C.c_uint32), _p(bvals, C.c_uint32)) == 0
        eids, evals = _order(dpos, None, pos_ids)
        assert list(vals) == evals[:k] and list(ids) == eids[:k], k
        assert tot.value == int(deg.sum()) == g.info.nentries
        assert list(bids[:k]) == eids[:k] and list(bvals[:k]) == evals[:k], k
        cids, cvals = _order(~dpos, None, pos_ids)
        assert list(bids[k:]) == cids[:k] and list(bvals[k:]) == cvals[:k], k


def test_engine_topk_active_only_pads(gpu, progs, tmp_path):
    """topk(active_only) after a BFS: the vertices apply reached (not the
    root, which init activates without marking), farthest first; with fewer
    active vertices than k the list is padded with (0, 0) pairs, as one rank
    of the reference pads."""
    L = gpu
    n = 1 << 12
    p = tmp_path / "g.bin"
    e = L.EdgeList.rmat(12, 4, seed=53)
    e.write(p)
    # plus a path 4097 - 4098 - 4099 - 4100 away from the rest: a root there
    # reaches three vertices, fewer than k
    np.concatenate([np.fromfile(p, np.uint32), np.array([4097, 4098, 4098, 4099, 4099, 4100], np.uint32)]).tofile(p)
    n += 4
    g = L.Graph.load_undirected(p, n)
    _, pos_ids = g.positions()
    u32p = C.POINTER(C.c_uint32)
    progs.la3gp_bfs_topk.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, u32p, u32p]
    for root in (1, 100, 4097):
        hops, _, _ = _bfs(L, progs, g, root)
        hpos = hops[pos_ids].astype(np.int64)
        act = (hpos != 255) & (pos_ids != root)
        cand = np.nonzero(act)[0]
        ids_e, vals_e = _order(hpos[cand], None, pos_ids[cand])
        for k in (5, 512):
            ids = np.empty(k, np.uint32)
            vals = np.empty(k, np.uint32)
            assert progs.la3gp_bfs_topk(g._h, root, k, _p(ids, C.c_uint32), _p(vals, C.c_uint32)) == 0
            m = min(k, len(cand))
            assert list(vals[:m]) == vals_e[:m] and list(ids[:m]) == ids_e[:m], (root, k)
            # padding: value-initialised pairs sorted in (value 0 sorts after every reached vertex)
            assert all(v == 0 and i == 0 for i, v in zip(ids[m:], vals[m:])), (root, k)


def test_tc_through_engine_vs_oracle(gpu, progs, oracle, tmp_path):
    """TC written as the reference writes it (tc.cpp:11-52): CtVertex's
    neighbour lists are variable-size messages of any length (R-MAT hubs
    scatter lists of thousands of ids), gathered with the row's own list
    (gather_with_state); per-vertex counts and the reduce() total against
    the oracle."""
    L = gpu
    n = 1 << 15
    p = tmp_path / "t.bin"
    L.EdgeList.rmat(15, 16, seed=61).write(p)
    g = L.Graph.load_directed(p, n, remove_cycles=True)
    gr = L.Graph.load(p, n, L.DIRECTED | L.ACYCLIC | L.REVERSE)
    progs.la3gp_tc.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]
    tot = C.c_uint64()
    ntri = np.empty(g.nslots, np.uint32)
    assert progs.la3gp_tc(g._h, gr._h, C.byref(tot), _p(ntri, C.c_uint32)) == 0
    otot, oper = oracle.OracleGraph(p, n, oracle.DIRECTED | oracle.ACYCLIC).tc()
    assert tot.value == otot
    assert np.array_equal(ntri, oper)
    assert np.bincount(np.fromfile(p, np.uint32), minlength=n + 1).max() > 1000  # long messages
