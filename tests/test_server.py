"""Serving loop (la3g_server_*): continuous batching over resident graphs.

Every served result must equal the single-query entry point's result for
the same query, whether the query ran alone or mixed with others on the
same engine (lanes joining and leaving mid-flight) and on other graphs.
"""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _graphs(L, scale=12):
    gu = L.Graph.from_edges(L.EdgeList.rmat(scale, 16, seed=5), 0)
    gw = L.Graph.from_edges(L.EdgeList.rmat(scale, 16, seed=5, weighted=True, wseed=6), L.DIRECTED | L.WEIGHTED)
    return gu, gw


def _roots(G, k, seed):
    _, ids = G.positions()
    cand = np.sort(ids[: G.info.nregular + G.info.nsink + G.info.nsource])
    return [int(x) for x in np.random.default_rng(seed).choice(cand, k)]


@pytest.fixture(params=["lanes", "adaptive"])
def servers(gpu, request):
    """Creates servers and frees them at teardown, before their graphs.  Every
    test runs twice: lanes only (every query in a lane), and with adaptive
    batching (queries arriving at an idle engine answered alone)."""
    made = []

    def make(*a, **k):
        S = gpu.Server(*a, **k)
        if request.param == "lanes":
            S.set_solo(0, 0)
        made.append(S)
        return S

    yield make
    for S in made:
        S.free()


def _wait(S, t):
    r = S.poll(t, 120000)
    assert r is not None, "query not answered within 120 s"
    res, bufs = r
    assert res.status == 0
    return res, bufs


def test_bfs_alone_and_mixed(gpu, servers):
    L = gpu
    gu, _ = _graphs(L)
    roots = _roots(gu, 300, 1)
    want = {r: L.bfs(gu, r, True, False)[0] for r in set(roots)}
    S = servers(1 << 34, bfs_lanes=128)
    gid = S.add_graph(gu)
    assert S.lanes(gid) == 128
    # alone: one query at a time
    for r in roots[:5]:
        _, (h,) = _wait(S, S.submit_bfs(gid, r))
        assert np.array_equal(h, want[r])
    # mixed: more queries than lanes, submitted at once
    ts = [(r, S.submit_bfs(gid, r)) for r in roots]
    seen_batch = 0
    for r, t in ts:
        res, (h,) = _wait(S, t)
        seen_batch = max(seen_batch, res.in_flight)
        assert np.array_equal(h, want[r]), r
    assert seen_batch > 1  # queries really shared the engine
    S.free()


def test_sssp_alone_and_mixed(gpu, servers):
    L = gpu
    _, gw = _graphs(L)
    roots = _roots(gw, 150, 2)
    want = {r: L.sssp(gw, r)[0] for r in set(roots)}
    S = servers(1 << 34, sssp_lanes=64)
    gid = S.add_graph(gw)
    for r in roots[:5]:
        _, (d,) = _wait(S, S.submit_sssp(gid, r))
        assert np.array_equal(d, want[r])
    ts = [(r, S.submit_sssp(gid, r)) for r in roots]
    for r, t in ts:
        _, (d,) = _wait(S, t)
        assert np.array_equal(d, want[r]), r
    S.free()


def test_mixed_graphs_and_threads(gpu, servers, tmp_path):
    """BFS, SSSP and BM25 queries over several resident graphs, submitted
    from two threads at once; every result equals the single-query call."""
    L = gpu
    gu, gw = _graphs(L, 12)
    gu2 = L.Graph.from_edges(L.EdgeList.rmat(14, 16, seed=9), 0)
    D, T = 5000, 800
    e = L.EdgeList.bipartite(D, T, 20, seed=4)
    p = tmp_path / "c.bin"
    e.write(p)
    gb = L.Graph.load_bipartite(p, D, T)
    b = L.BM25(gb)
    rng = np.random.default_rng(7)
    queries = [sorted(set(int(x) for x in rng.integers(D + 1, D + T + 1, int(rng.integers(2, 9))))) for _ in range(40)]
    want_b = [b.query(q, 10)[:2] for q in queries]
    lm = L.LM(gb)
    lm.query([], 0)  # the first query's leftover activity, as the server takes it
    want_l = [lm.query(q, 10)[:2] for q in queries]
    r1, r2, r3 = _roots(gu, 80, 3), _roots(gw, 60, 4), _roots(gu2, 80, 5)
    want1 = {r: L.bfs(gu, r, True, False)[0] for r in set(r1)}
    want2 = {r: L.sssp(gw, r)[0] for r in set(r2)}
    want3 = {r: L.bfs(gu2, r, True, False)[0] for r in set(r3)}
    S = servers(1 << 34, bfs_lanes=64, sssp_lanes=64)
    g1, g2, g3, g4 = S.add_graph(gu), S.add_graph(gw), S.add_graph(gu2), S.add_graph(gb)
    got = []
    lock = threading.Lock()

    def client(part):
        mine = []
        for i in range(max(len(r1), len(r2), len(r3), len(queries))):
            if part == 0 and i < len(r1):
                mine.append(("b1", r1[i], S.submit_bfs(g1, r1[i])))
            if part == 1 and i < len(r2):
                mine.append(("s", r2[i], S.submit_sssp(g2, r2[i])))
            if part == 0 and i < len(r3):
                mine.append(("b3", r3[i], S.submit_bfs(g3, r3[i])))
            if part == 1 and i < len(queries):
                mine.append(("q", i, S.submit_bm25(g4, queries[i], 10)))
            if part == 0 and i < len(queries):
                mine.append(("l", i, S.submit_lm(g4, queries[i], 10)))
        for kind, key, t in mine:
            res, bufs = _wait(S, t)
            with lock:
                got.append((kind, key, bufs))

    th = [threading.Thread(target=client, args=(k,)) for k in (0, 1)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert len(got) == len(r1) + len(r2) + len(r3) + 2 * len(queries)
    for kind, key, bufs in got:
        if kind == "b1":
            assert np.array_equal(bufs[0], want1[key])
        elif kind == "b3":
            assert np.array_equal(bufs[0], want3[key])
        elif kind == "s":
            assert np.array_equal(bufs[0], want2[key])
        else:
            want = want_b if kind == "q" else want_l
            ids, sc = bufs
            assert ids.tolist() == want[key][0].tolist()
            assert np.array_equal(sc, want[key][1])
    info = S.info()
    assert info["ngraphs"] == 4 and info["pending"] == 0
    S.free()


def test_budget_admission(gpu, servers):
    L = gpu
    gu, gw = _graphs(L, 12)
    need = gu.info.device_bytes
    # not even the graph fits
    S = servers(need // 2)
    with pytest.raises(L.LA3GError) as ex:
        S.add_graph(gu)
    assert ex.value.status == 5  # LA3G_EBUDGET
    S.free()
    # the graph fits with fewer lanes: the engine is halved to 64
    N = gu.nslots
    lane128 = N * 2 * 8 * 3 + N * 128 + N * 2 * 4 * 3 + 2 * 64 * N + 4096 + 128 * 16
    S = servers(need + lane128 - 1, bfs_lanes=128)
    gid = S.add_graph(gu)
    assert S.lanes(gid) == 64
    r = _roots(gu, 1, 9)[0]
    _, (h,) = _wait(S, S.submit_bfs(gid, r))
    assert np.array_equal(h, L.bfs(gu, r, True, False)[0])
    # nothing is left for a second graph
    with pytest.raises(L.LA3GError) as ex:
        S.add_graph(gw)
    assert ex.value.status == 5
    S.free()


def test_edge_cases(gpu, servers):
    L = gpu
    # a path of 300 vertices: lanes that would need hop 255 finish through
    # the single-root path (uint8 wrap as the reference has it)
    n = 300
    rec = np.array([[i, i + 1] for i in range(1, n)], np.uint32)
    gp = L.Graph.from_records(rec, n, 0)
    gu, gw = _graphs(L, 10)
    S = servers(1 << 34, bfs_lanes=64)
    gid, gid2, gid3 = S.add_graph(gp), S.add_graph(gu), S.add_graph(gw)
    for r in (1, 150, n):
        _, (h,) = _wait(S, S.submit_bfs(gid, r))
        assert np.array_equal(h, L.bfs(gp, r, True, False)[0]), r
    # a root with no vertex: nothing reached
    _, (h,) = _wait(S, S.submit_bfs(gid2, gu.nslots + 5))
    assert np.array_equal(h, L.bfs(gu, gu.nslots + 5, True, False)[0])
    _, (d,) = _wait(S, S.submit_sssp(gid3, gw.nslots + 5))
    assert np.array_equal(d, L.sssp(gw, gw.nslots + 5)[0])
    # sink and isolated roots of the directed graph
    _, ids = gw.positions()
    i = gw.info
    for r in (int(ids[i.nregular]), int(ids[i.nregular + i.nsink + i.nsource]) if i.nisolated else 0):
        _, (d,) = _wait(S, S.submit_sssp(gid3, r))
        assert np.array_equal(d, L.sssp(gw, r)[0]), r
    # query kind that does not match the graph
    with pytest.raises(L.LA3GError):
        S.submit_sssp(gid2, 1)
    with pytest.raises(L.LA3GError):
        S.submit_bfs(99, 1)
