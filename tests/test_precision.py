"""PageRank precision study: FP32 SpMV with FP32 accumulation (la3g_pr_f32)
against the FP64 path, which is bit-identical to the reference (pr.cpp:11-55).

Tolerances (stated here, measured on R-MAT / ER graphs): after 20
iterations the FP32 ranks stay within 1e-5 relative L1 (sum |r32 - r64| /
sum r64) and 1e-5 relative max-abs (max |r32 - r64| / max(1, r64)) of the
FP64 ranks.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L1_REL_TOL = 1e-5
MAX_REL_TOL = 1e-5


def _errors(r32, r64):
    d = np.abs(r32 - r64)
    return d.sum() / r64.sum(), (d / np.maximum(1.0, np.abs(r64))).max(), d.max()


@pytest.mark.parametrize("kind", ["rmat", "er"])
def test_f32_vs_oracle(gpu, oracle, tmp_path, kind):
    L = gpu
    if kind == "rmat":
        e = L.EdgeList.rmat(14, 16, seed=31)
    else:
        e = L.EdgeList.er(1 << 14, 16 << 14, seed=32)
    n = e.n
    p = tmp_path / "g.bin"
    e.write(p)
    g = L.Graph.load_directed(p, n)
    r32, res, st = L.pagerank_f32(g, 20)
    assert st.iterations == 20
    orank, _ = oracle.OracleGraph(p, n, oracle.DIRECTED).pagerank(20)
    r64, _, _ = L.pagerank(g, 20)
    assert np.array_equal(r64, orank)  # the FP64 path is the oracle's
    l1, mx, _ = _errors(r32, orank)
    assert l1 < L1_REL_TOL and mx < MAX_REL_TOL, (l1, mx)
    assert res > 0.0
    # sources keep 0.15, as in the FP64 path
    pos, ids = g.positions()
    i = g.info
    src = ids[i.nregular + i.nsink: i.nregular + i.nsink + i.nsource]
    assert np.all(r32[src] == 0.15)


def test_f32_residual_and_tolerance_stop(gpu):
    L = gpu
    g = L.Graph.from_edges(L.EdgeList.rmat(13, 16, seed=33), L.DIRECTED)
    _, res5, _ = L.pagerank_f32(g, 5)
    _, res15, _ = L.pagerank_f32(g, 15)
    assert res15 < res5  # the L1 residual (FP64) shrinks with the iterations
    # stop on the residual: fewer iterations than the cap, residual below tol
    tol = res15 * 1.5
    _, res, st = L.pagerank_f32(g, 50, tol)
    assert st.iterations < 50 and res < tol
    # repeated calls give the same ranks
    a = L.pagerank_f32(g, 10)[0]
    b = L.pagerank_f32(g, 10)[0]
    assert np.array_equal(a, b)


@pytest.mark.parametrize("kind", ["rmat", "er"])
def test_f32_tiled_vs_oracle(gpu, oracle, tmp_path, kind):
    """The FP32 study over the tiled DCSC layout (la3g_pr_f32_tiled): the
    same tolerances against the FP64 oracle, and within FP32 rounding of the
    flat-CSR FP32 path (only the order of additions inside a row differs).
    2^17 vertices: eight row tiles, R-MAT hub columns above the warp
    threshold in every tile."""
    L = gpu
    if kind == "rmat":
        e = L.EdgeList.rmat(17, 16, seed=35)
    else:
        e = L.EdgeList.er(1 << 17, 16 << 17, seed=36)
    n = e.n
    p = tmp_path / "g.bin"
    e.write(p)
    g = L.Graph.load_directed(p, n)
    rt, rest, st = L.pagerank_f32(g, 20, tiled=True)
    rf, resf, _ = L.pagerank_f32(g, 20)
    assert st.iterations == 20
    orank, _ = oracle.OracleGraph(p, n, oracle.DIRECTED).pagerank(20)
    l1, mx, _ = _errors(rt, orank)
    assert l1 < L1_REL_TOL and mx < MAX_REL_TOL, (l1, mx)
    l1f, mxf, _ = _errors(rt, rf)
    assert l1f < 1e-6 and mxf < 1e-5, (l1f, mxf)
    assert abs(rest - resf) <= 1e-2 * resf
    # sinks and sources as in the flat path
    pos, ids = g.positions()
    i = g.info
    src = ids[i.nregular + i.nsink: i.nregular + i.nsink + i.nsource]
    assert np.all(rt[src] == 0.15)
    # repeated calls reuse the layout and give the same ranks up to FP32 rounding
    rt2 = L.pagerank_f32(g, 20, tiled=True)[0]
    assert np.abs(rt2 - rt).max() <= 1e-5 * max(1.0, np.abs(rt).max())
