"""Degenerate inputs through the C ABI against the oracle: an empty file,
a file of self-loops only (all dropped at load), one edge, vertex 0 with
edges, a root with no edges, a root id beyond n, n = 1, and BM25 queries
that are empty, hit no term or ask for more documents than exist."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _write(tmp_path, name, rec, cols=2):
    p = tmp_path / name
    np.asarray(rec, np.uint32).reshape(-1, cols).tofile(p)
    return p


CASES = {
    "empty": [],
    "selfloops": [[1, 1], [2, 2], [3, 3]],
    "one_edge": [[1, 2]],
    "zero_id": [[0, 1], [1, 2], [2, 0]],
    "star": [[1, k] for k in range(2, 9)],
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_graph_apps_degenerate(gpu, oracle, tmp_path, name):
    L = gpu
    rec = CASES[name]
    n = 8
    p = _write(tmp_path, "g.bin", rec)
    pw = _write(tmp_path, "g.w.bin", [r + [3 + i] for i, r in enumerate(rec)], 3)
    gu = L.Graph.load_undirected(p, n)
    ou = oracle.OracleGraph(p, n, 0)
    for root in (0, 1, 2, 5, n, n + 3):
        h, par, _ = L.bfs(gu, root)
        oh, opar, _ = ou.bfs(root)
        assert np.array_equal(h, oh) and np.array_equal(par, opar), (name, root)
    lab, _ = L.cc(gu)
    assert np.array_equal(lab, ou.cc()[0]), name
    gd = L.Graph.load_directed(p, n)
    r, d, _ = L.pagerank(gd, 5)
    orank, odeg = oracle.OracleGraph(p, n, oracle.DIRECTED).pagerank(5)
    assert np.array_equal(r.view(np.uint64), orank.view(np.uint64)) and np.array_equal(d, odeg), name
    gw = L.Graph.load_directed(pw, n, weighted=True)
    ow = oracle.OracleGraph(pw, n, oracle.DIRECTED | oracle.WEIGHTED)
    for root in (0, 1, 2, 5, n + 3):
        dist, _ = L.sssp(gw, root)
        assert np.array_equal(dist, ow.sssp(root)[0]), (name, root)
    gt = L.Graph.load_directed(p, n, remove_cycles=True)
    tot, per, _ = L.tc(gt)
    otot, oper = oracle.OracleGraph(p, n, oracle.DIRECTED | oracle.ACYCLIC).tc()
    assert tot == otot and np.array_equal(per, oper), name
    # the batched forms on the same inputs
    roots = [0, 1, 2, 5, n + 3]
    hb, _ = L.bfs_batch(gu, roots)
    for k, rt in enumerate(roots):
        assert np.array_equal(hb[k], ou.bfs(rt)[0]), (name, rt)
    db, _ = L.sssp_batch(gw, roots)
    for k, rt in enumerate(roots):
        assert np.array_equal(db[k], ow.sssp(rt)[0]), (name, rt)


def test_single_vertex(gpu, oracle, tmp_path):
    L = gpu
    p = _write(tmp_path, "g.bin", [])
    g = L.Graph.load_undirected(p, 1)
    assert g.nslots == 2
    h, _, _ = L.bfs(g, 1)
    assert h.tolist() == oracle.OracleGraph(p, 1, 0).bfs(1)[0].tolist()


def test_bm25_degenerate_queries(gpu, oracle, tmp_path):
    L = gpu
    D, T = 300, 60
    e = L.EdgeList.bipartite(D, T, 10, seed=5)
    p = tmp_path / "c.bin"
    e.write(p)
    g = L.Graph.load_bipartite(p, D, T)
    b = L.BM25(g)
    ob = oracle.OracleBM25(oracle.OracleGraph(p, D, oracle.BIPARTITE | oracle.WEIGHTED, nright=T))
    for q, k in (([], 10), ([0], 10), ([D + T + 5], 10), ([D + 1], 0), ([D + 1, D + 2], 64), ([1, D + 3], 10)):
        ids, sc, _, _ = b.query(q, k)
        oids, osc, _, _ = ob.query(q, k)
        assert ids.tolist() == oids.tolist() and np.array_equal(sc, osc), (q, k)


def test_header_format_matches_plain(gpu, tmp_path):
    """n = 0 takes the vertex count from the 16-byte header
    (graph.hpp:89-117); the graph equals the headerless one with n given."""
    L = gpu
    e = L.EdgeList.rmat(10, 8, seed=12, weighted=True, wseed=13)
    ph, pp = tmp_path / "h.bin", tmp_path / "p.bin"
    e.write(ph, header=True)
    e.write(pp, header=False)
    n = 1 << 10
    a = L.Graph.load_directed(ph, 0, weighted=True)
    b = L.Graph.load_directed(pp, n, weighted=True)
    assert a.nslots == b.nslots == n + 1
    assert a.info.nentries == b.info.nentries
    assert np.array_equal(L.sssp(a, 3)[0], L.sssp(b, 3)[0])
    au = L.Graph.load_undirected(ph, 0, weighted=True)
    bu = L.Graph.load_undirected(pp, n, weighted=True)
    assert np.array_equal(L.bfs(au, 3)[0], L.bfs(bu, 3)[0])


def test_lm_degenerate_queries(gpu, oracle, tmp_path):
    """LM on the queries BM25's edge cases use, in sequence (the first one
    also ranks the term vertices the TL pass left active), against the
    oracle."""
    L = gpu
    D, T = 300, 60
    e = L.EdgeList.bipartite(D, T, 10, seed=6)
    p = tmp_path / "c.bin"
    e.write(p)
    g = L.Graph.load_bipartite(p, D, T)
    b = L.LM(g)
    ob = oracle.OracleLM(oracle.OracleGraph(p, D, oracle.BIPARTITE | oracle.WEIGHTED, nright=T))
    for q, k in (([], 10), ([0], 10), ([D + T + 5], 10), ([D + 1], 0), ([D + 1, D + 2], 64), ([1, D + 3], 10),
                 ([D + 4, D + 4, D + 4], 5)):
        ids, sc, (alls, act), _ = b.query(q, k, full=True)
        oids, osc, oscores, oact = ob.query(q, k)
        assert ids.tolist() == oids.tolist() and np.array_equal(sc, osc), (q, k)
        assert np.array_equal(act, oact) and np.array_equal(alls.view(np.uint32), oscores.view(np.uint32)), (q, k)
