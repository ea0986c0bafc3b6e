"""Batched multi-source BFS / SSSP: every root's row equals the single-root
run (la3g_bfs / la3g_sssp), for each level mode of the batched BFS."""
import numpy as np
import pytest

from conftest import GOLD

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def graphs(gpu, tmp_path_factory):
    L = gpu
    d = tmp_path_factory.mktemp("batch")
    e = L.EdgeList.rmat(14, 16, seed=77)
    p = d / "g.bin"
    e.write(p)
    ew = L.EdgeList.rmat(14, 16, seed=77, weighted=True, wseed=5)
    pw = d / "g.w.bin"
    ew.write(pw)
    er = L.EdgeList.er(1 << 14, 8 << 14, seed=9)
    pe = d / "er.bin"
    er.write(pe)
    n = 1 << 14
    return {"rmat": L.Graph.load_undirected(p, n), "er": L.Graph.load_undirected(pe, n),
            "w": L.Graph.load_directed(pw, n, weighted=True), "n": n}


def _roots(n, k, seed):
    r = np.random.default_rng(seed).integers(0, n + 1, k).astype(np.uint32)
    r[0] = r[1]            # a duplicate root
    r[2] = n + 5           # out of range: every hop stays 255
    r[3] = 0               # vertex 0 (isolated with 1-based ids)
    return r


@pytest.mark.parametrize("mode,block,push", [(0, 256, 0.0), (0, 128, 0.1), (1, 256, 0.0), (1, 512, 0.0)])
def test_bfs_batch_equals_single(gpu, graphs, mode, block, push):
    L = gpu
    for name in ("rmat", "er"):
        g = graphs[name]
        roots = _roots(graphs["n"], 100, 3)  # not a multiple of 64
        L.batch_config(g, mode, block, push)
        hops, st = L.bfs_batch(g, roots)
        for i, r in enumerate(roots):
            h1, _, _ = L.bfs(g, int(r))
            assert np.array_equal(hops[i], h1), (name, mode, i, int(r))


def test_bfs_batch_autotune_then_1024_roots(gpu, graphs):
    L = gpu
    g = graphs["rmat"]
    rep = L.batch_autotune(g, _roots(graphs["n"], 64, 4))
    assert len(rep) >= 4 and all(x["ms"] > 0 for x in rep)
    roots = _roots(graphs["n"], 1024, 5)
    hops, st = L.bfs_batch(g, roots)
    for i in range(0, 1024, 97):
        h1, _, _ = L.bfs(g, int(roots[i]))
        assert np.array_equal(hops[i], h1), i


def test_bfs_batch_deep_path_follows_single_root(gpu):
    L = gpu
    g = L.Graph.load_undirected(GOLD / "data" / "path300.bin", 300)
    ref = np.load(GOLD / "path300_bfs.npz")["hops"]
    hops, _ = L.bfs_batch(g, [1, 1])
    assert np.array_equal(hops[0], ref) and np.array_equal(hops[1], ref)


def test_sssp_batch_equals_single(gpu, graphs):
    L = gpu
    g = graphs["w"]
    roots = _roots(graphs["n"], 300, 6)  # two chunks of the 256-root pass
    dist, st = L.sssp_batch(g, roots)
    for i in list(range(0, 300, 23)) + [0, 1, 2, 3, 299]:
        d1, _ = L.sssp(g, int(roots[i]))
        assert np.array_equal(dist[i], d1), (i, int(roots[i]))


@pytest.mark.parametrize("delta", [1, 16, 128, 0xFFFFFFFF, 0])
def test_sssp_batch_window_equals_single(gpu, graphs, delta):
    """The batched SSSP's distance window (delta-stepping's buckets over all
    roots of a chunk) only reorders relaxations: for every width, on a graph
    with hubs (R-MAT) and one without (ER, where the automatic width is on),
    each root's distances equal the single-root call's."""
    L = gpu
    n = graphs["n"]
    ge = L.Graph.from_edges(L.EdgeList.er(n, 16 * n, seed=31, weighted=True, wseed=8), L.DIRECTED | L.WEIGHTED)
    for g in (graphs["w"], ge):
        L.batch_sssp_window(g, delta)
        roots = _roots(n, 130, 12)
        dist, st = L.sssp_batch(g, roots)
        for i in list(range(0, 130, 11)) + [0, 1, 2, 3, 129]:
            d1, _ = L.sssp(g, int(roots[i]))
            assert np.array_equal(dist[i], d1), (delta, i, int(roots[i]))
        L.batch_sssp_window(g, 0)
    ge.free()


def test_persistent_barrier_wait_runs_out_cleanly(gpu, graphs):
    """The persistent kernel's grid-barrier waits are bounded: with a limit
    of zero polls the first block that has to wait gives up, every block
    leaves, and the call returns LA3G_ETIMEOUT.  The device stays usable:
    with the default limit back, the same batch equals the single-root
    runs."""
    L = gpu
    g = graphs["rmat"]
    roots = _roots(graphs["n"], 96, 41)
    L.batch_config(g, 1, 256, 0.0)
    L.batch_set_wait_limit(g, 0)
    with pytest.raises(L._native.LA3GError) as ex:
        L.bfs_batch(g, roots)
    assert ex.value.status == 6  # LA3G_ETIMEOUT
    L.batch_set_wait_limit(g, -1)
    hops, _ = L.bfs_batch(g, roots)
    for i in (0, 5, 50, 95):
        assert np.array_equal(hops[i], L.bfs(g, int(roots[i]), True, False)[0]), i
