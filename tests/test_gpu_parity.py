"""GPU path vs the reference: every golden case (reference outputs) and
larger seeded graphs checked against the C oracle.  Calls go through the C
ABI (la3_gb300 is a ctypes binding of libla3g)."""
import numpy as np
import pytest

from conftest import GOLD

DATA = GOLD / "data"
pytestmark = pytest.mark.gpu


def _cases(golden, app):
    return sorted(k for k, v in golden.items() if v["app"] == app)


def test_pagerank_golden(gpu, golden):
    L = gpu
    for name in _cases(golden, "pr"):
        c = golden[name]
        ref = np.load(GOLD / f"{name}.npz")
        g = L.Graph.load_directed(DATA / c["file"], c["n"])
        rank, deg, st = L.pagerank(g, c["iters"])
        assert np.array_equal(deg, ref["degree"]), name
        assert np.array_equal(rank.view(np.uint64), ref["rank"].view(np.uint64)), (
            name, float(np.abs(rank - ref["rank"]).max()))


def test_bfs_golden(gpu, golden):
    L = gpu
    for name in _cases(golden, "bfs"):
        c = golden[name]
        ref = np.load(GOLD / f"{name}.npz")
        g = L.Graph.load_undirected(DATA / c["file"], c["n"])
        hops, parent, st = L.bfs(g, c["root"])
        assert np.array_equal(hops, ref["hops"]), name
        assert np.array_equal(parent, ref["parent"]), name


def test_sssp_golden(gpu, golden):
    L = gpu
    for name in _cases(golden, "sssp"):
        c = golden[name]
        ref = np.load(GOLD / f"{name}.npz")
        g = L.Graph.load_directed(DATA / c["file"], c["n"], weighted=True)
        dist, st = L.sssp(g, c["root"])
        assert np.array_equal(dist, ref["dist"]), name


def test_cc_golden(gpu, golden):
    L = gpu
    for name in _cases(golden, "cc"):
        c = golden[name]
        ref = np.load(GOLD / f"{name}.npz")
        g = L.Graph.load_undirected(DATA / c["file"], c["n"])
        lab, st = L.cc(g)
        assert np.array_equal(lab, ref["label"]), name


def test_tc_golden(gpu, golden):
    L = gpu
    for name in _cases(golden, "tc"):
        c = golden[name]
        ref = np.load(GOLD / f"{name}.npz")
        g = L.Graph.load_directed(DATA / c["file"], c["n"], remove_cycles=True)
        total, per, st = L.tc(g)
        assert np.array_equal(per, ref["ntri"]), name
        assert total == c["triangles"], name


@pytest.fixture(scope="module")
def rmat16(gpu, tmp_path_factory):
    d = tmp_path_factory.mktemp("rmat16")
    e = gpu.EdgeList.rmat(16, 16, seed=2026)
    ew = gpu.EdgeList.rmat(16, 16, seed=2026, weighted=True, wseed=7)
    p, pw = d / "g.bin", d / "g.w.bin"
    e.write(p)
    ew.write(pw)
    return p, pw, 1 << 16


def _roots(n, k, seed):
    return [int(x) for x in np.random.default_rng(seed).integers(1, n + 1, k)]


def test_pagerank_rmat16_vs_oracle(gpu, oracle, rmat16):
    p, _, n = rmat16
    rank, deg, st = gpu.pagerank(gpu.Graph.load_directed(p, n), 20)
    orank, odeg = oracle.OracleGraph(p, n, oracle.DIRECTED).pagerank(20)
    assert np.array_equal(deg, odeg)
    assert np.array_equal(rank.view(np.uint64), orank.view(np.uint64)), float(np.abs(rank - orank).max())
    assert st.iterations == 20


def test_bfs_sssp_cc_tc_rmat16_vs_oracle(gpu, oracle, rmat16):
    p, pw, n = rmat16
    gu = gpu.Graph.load_undirected(p, n)
    ou = oracle.OracleGraph(p, n, 0)
    for r in _roots(n, 4, 1):
        h, par, st = gpu.bfs(gu, r)
        oh, op, oit = ou.bfs(r)
        assert np.array_equal(h, oh) and np.array_equal(par, op), r
        assert st.iterations == oit
    lab, _ = gpu.cc(gu)
    olab, _ = ou.cc()
    assert np.array_equal(lab, olab)
    gw = gpu.Graph.load_directed(pw, n, weighted=True)
    ow = oracle.OracleGraph(pw, n, oracle.DIRECTED | oracle.WEIGHTED)
    for r in _roots(n, 4, 2):
        d, st = gpu.sssp(gw, r)
        od, oit = ow.sssp(r)
        assert np.array_equal(d, od), r
        assert st.iterations == oit
    total, per, _ = gpu.tc(gpu.Graph.load_directed(p, n, remove_cycles=True))
    ototal, oper = oracle.OracleGraph(p, n, oracle.DIRECTED | oracle.ACYCLIC).tc()
    assert total == ototal and np.array_equal(per, oper)


def test_graph_structure_vs_oracle(gpu, oracle, rmat16):
    p, pw, n = rmat16
    for flags in (0, gpu.DIRECTED, gpu.DIRECTED | gpu.ACYCLIC, gpu.DIRECTED | gpu.REVERSE):
        g = gpu.Graph.load(p, n, flags)
        og = oracle.OracleGraph(p, n, flags)
        assert (g.info.nregular, g.info.nsink, g.info.nsource) == og.classes(), flags
        assert g.info.nentries == og.nedges
        pos, ids = g.positions()
        opos, oids = og.positions()
        assert np.array_equal(pos, opos) and np.array_equal(ids, oids)


def test_repeated_calls_are_identical(gpu, rmat16):
    p, pw, n = rmat16
    g = gpu.Graph.load_undirected(p, n)
    a = gpu.bfs(g, 11)[:2]
    b = gpu.bfs(g, 11)[:2]
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    gd = gpu.Graph.load_directed(p, n)
    r1 = gpu.pagerank(gd, 5)[0]
    r2 = gpu.pagerank(gd, 5)[0]
    assert np.array_equal(r1.view(np.uint64), r2.view(np.uint64))


def test_device_loop_matches_host_stepped(gpu, rmat16):
    """BFS and SSSP levels run as one device-driven graph; with profiling on
    the same decide kernel and bodies are stepped from the host.  Both forms
    give the same results, iteration counts, examined edges and launches."""
    p, pw, n = rmat16
    gu = gpu.Graph.load_undirected(p, n)
    gw = gpu.Graph.load_directed(pw, n, weighted=True)
    hub = int(np.bincount(np.fromfile(p, np.uint32), minlength=n + 1).argmax())
    fields = ("iterations", "pull_iterations", "edges_examined", "kernel_launches")
    try:
        for r in _roots(n, 3, 5) + [hub]:
            runs = []
            for prof in (False, True):
                gpu.profile(prof)
                h, par, st = gpu.bfs(gu, r)
                d, sst = gpu.sssp(gw, r)
                runs.append((h, par, d, [getattr(st, f) for f in fields], [getattr(sst, f) for f in fields]))
            (h0, p0, d0, s0, t0), (h1, p1, d1, s1, t1) = runs
            assert np.array_equal(h0, h1) and np.array_equal(p0, p1) and np.array_equal(d0, d1), r
            assert s0 == s1 and t0 == t1, (r, s0, s1, t0, t1)
    finally:
        gpu.profile(False)
        gpu.profile_reset()


def test_wrong_graph_kind_is_rejected(gpu, rmat16):
    p, pw, n = rmat16
    g = gpu.Graph.load_undirected(p, n)
    with pytest.raises(gpu.LA3GError):
        gpu.pagerank(g, 3)
    with pytest.raises(gpu.LA3GError):
        gpu.sssp(g, 1)
    with pytest.raises(gpu.LA3GError):
        gpu.tc(g)


def test_out_of_range_ids_rejected(gpu, tmp_path):
    p = tmp_path / "bad.bin"
    np.array([[1, 2], [3, 99]], np.uint32).tofile(p)
    with pytest.raises(gpu.LA3GError) as ei:
        gpu.Graph.load_undirected(p, 8)
    assert ei.value.status == 1


@pytest.mark.parametrize("app", ["bm25", "lm"])
def test_ir_golden(gpu, golden, app):
    L = gpu
    for name in _cases(golden, app):
        c = golden[name]
        ref = np.load(GOLD / f"{name}.npz")
        g = L.Graph.load_bipartite(DATA / c["file"], c["ndocs"], c["nterms"])
        b = L.BM25(g, want_length=True) if app == "bm25" else L.LM(g, want_length=True)
        assert b.collection_ntokens == c["collection_ntokens"], name
        assert np.array_equal(b.length.view(np.uint32), ref["length"].view(np.uint32)), name
        queries = L.read_queries(DATA / c["labels"], DATA / c["queries"], c["ndocs"])
        for qi, q in enumerate(queries):
            ids, sc, (alls, act), st = b.query(q, c["k"], full=True)
            rid, rsc = ref[f"q{qi}_ids"], ref[f"q{qi}_scores"]
            assert np.array_equal(np.flatnonzero(act), np.sort(rid)), (name, qi)
            order = np.argsort(rid)
            assert np.array_equal(alls[rid[order]].view(np.uint32), rsc[order].view(np.uint32)), (name, qi)
            # canonical top-k: score desc, id asc over the reference's scores
            want = sorted(zip(rid.tolist(), rsc.tolist()), key=lambda t: (-t[1], t[0]))[: c["k"]]
            assert ids.tolist() == [w[0] for w in want], (name, qi)
            assert np.array_equal(sc, np.array([w[1] for w in want], np.float32)), (name, qi)


def test_bm25_corpus_vs_oracle(gpu, oracle, tmp_path):
    L = gpu
    D, T = 20000, 3000
    e = L.EdgeList.bipartite(D, T, 30, seed=77)
    p = tmp_path / "c.w.bp.bin"
    e.write(p)
    g = L.Graph.load_bipartite(p, D, T)
    b = L.BM25(g, want_length=True)
    og = oracle.OracleGraph(p, D, oracle.BIPARTITE | oracle.WEIGHTED, nright=T)
    ob = oracle.OracleBM25(og)
    assert b.collection_ntokens == ob.collection_ntokens
    assert np.array_equal(b.length.view(np.uint32), ob.length.view(np.uint32))
    rng = np.random.default_rng(3)
    for qi in range(30):
        q = sorted(set(int(x) for x in rng.integers(D + 1, D + T + 1, int(rng.integers(2, 9)))))
        if qi % 5 == 4:
            q = q[::-1] + [q[0]]  # not ascending, with a repeat: the reference's pairing
        ids, sc, (alls, act), _ = b.query(q, 10, full=True)
        oids, osc, oscores, oact = ob.query(q, 10)
        assert np.array_equal(act, oact), qi
        assert np.array_equal(alls.view(np.uint32), oscores.view(np.uint32)), qi
        assert ids.tolist() == oids.tolist() and np.array_equal(sc, osc), qi


def test_lm_corpus_vs_oracle(gpu, oracle, tmp_path):
    """LM on a generated corpus against the oracle (same host libm for the
    score's log10f factor): lengths, active sets and every score bit-exact,
    including the first query's leftover term vertices."""
    L = gpu
    D, T = 20000, 3000
    e = L.EdgeList.bipartite(D, T, 30, seed=78)
    p = tmp_path / "c.w.bp.bin"
    e.write(p)
    g = L.Graph.load_bipartite(p, D, T)
    b = L.LM(g, want_length=True)
    og = oracle.OracleGraph(p, D, oracle.BIPARTITE | oracle.WEIGHTED, nright=T)
    ob = oracle.OracleLM(og)
    assert b.collection_ntokens == ob.collection_ntokens
    assert np.array_equal(b.length.view(np.uint32), ob.length.view(np.uint32))
    rng = np.random.default_rng(4)
    for qi in range(30):
        q = sorted(set(int(x) for x in rng.integers(D + 1, D + T + 1, int(rng.integers(2, 9)))))
        if qi % 5 == 4:
            q = q[::-1] + [q[0]]  # not ascending, with a repeat: the reference's pairing
        if qi == 7:
            q = [3, D + 5, 0]  # a doc vertex and vertex 0 in the list
        ids, sc, (alls, act), _ = b.query(q, 20, full=True)
        oids, osc, oscores, oact = ob.query(q, 20)
        assert np.array_equal(act, oact), qi
        assert np.array_equal(alls.view(np.uint32), oscores.view(np.uint32)), qi
        assert ids.tolist() == oids.tolist() and np.array_equal(sc, osc), qi
        if qi == 0:
            assert act[D + 1:].sum() > 0  # the TL pass's term activity in the first query

