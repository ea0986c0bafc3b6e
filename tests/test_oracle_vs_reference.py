"""The oracle against the reference itself on randomly generated inputs (CPU
only): small graphs with duplicates, self-loops, vertex 0 with edges and
isolated roots go through the reference's dump drivers (oracle/_ref, built
from its sources) and through the oracle; every app must agree bit for bit.
Skipped where the reference build is absent."""
import json
import subprocess

import numpy as np
import pytest

from conftest import ROOT

REF_BIN = ROOT / "oracle" / "_ref" / "bin"
pytestmark = pytest.mark.skipif(not (REF_BIN / "dump_pr").exists(), reason="reference build (oracle/_ref) absent")


def _dump(args):
    r = subprocess.run([str(a) for a in args], capture_output=True, text=True, check=True,
                       env={"OMP_NUM_THREADS": "2", "PATH": "/usr/bin:/bin"})
    return json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])


def _graph(rng, tmp_path, weighted):
    n = int(rng.integers(5, 300))
    m = int(rng.integers(0, 4 * n))
    rec = np.stack([rng.integers(0, n, m), rng.integers(0, n, m)], 1)
    if weighted:
        rec = np.concatenate([rec, rng.integers(1, 200, (m, 1))], 1)
    p = tmp_path / ("g.w.bin" if weighted else "g.bin")
    rec.astype(np.uint32).tofile(p)
    return p, n


@pytest.mark.parametrize("seed", range(10))
def test_graph_apps(oracle, tmp_path, seed):
    O = oracle
    rng = np.random.default_rng(1000 + seed)
    p, n = _graph(rng, tmp_path, False)
    pw, nw = _graph(rng, tmp_path, True)
    o = tmp_path / "o"
    _dump([REF_BIN / "dump_pr", p, n, 10, o])
    rank, deg = O.OracleGraph(p, n, O.DIRECTED).pagerank(10)
    assert np.array_equal(rank.view(np.uint64), np.fromfile(str(o) + ".rank.f64", np.uint64))
    assert np.array_equal(deg, np.fromfile(str(o) + ".degree.u32", np.uint32))
    for root in (0, int(rng.integers(0, n + 1)), n):
        _dump([REF_BIN / "dump_bfs", p, n, root, o])
        hops, parent, _ = O.OracleGraph(p, n, 0).bfs(root)
        assert np.array_equal(hops, np.fromfile(str(o) + ".hops.u8", np.uint8)), root
        assert np.array_equal(parent, np.fromfile(str(o) + ".parent.u32", np.uint32)), root
    for root in (0, int(rng.integers(0, nw + 1))):
        _dump([REF_BIN / "dump_sssp", pw, nw, root, o])
        dist, _ = O.OracleGraph(pw, nw, O.DIRECTED | O.WEIGHTED).sssp(root)
        assert np.array_equal(dist, np.fromfile(str(o) + ".dist.u32", np.uint32)), root
    _dump([REF_BIN / "dump_cc", p, n, o])
    assert np.array_equal(O.OracleGraph(p, n, 0).cc()[0], np.fromfile(str(o) + ".label.u32", np.uint32))
    _dump([REF_BIN / "dump_tc", p, n, o])
    assert np.array_equal(O.OracleGraph(p, n, O.DIRECTED | O.ACYCLIC).tc()[1],
                          np.fromfile(str(o) + ".ntri.u32", np.uint32))


def _queries_bin(path):
    raw = np.fromfile(path, np.uint32)
    i, out = 0, []
    while i < raw.size:
        na = int(raw[i]); i += 1
        act = raw[i:i + 2 * na].reshape(-1, 2); i += 2 * na
        nk = int(raw[i]); i += 1
        i += 2 * nk
        out.append(act)
    return out


@pytest.mark.parametrize("app", ["bm25", "lm"])
@pytest.mark.parametrize("seed", range(4))
def test_retrieval_apps(oracle, tmp_path, app, seed):
    import la3_gb300 as L
    O = oracle
    rng = np.random.default_rng(2000 + seed)
    D, T = int(rng.integers(20, 400)), int(rng.integers(5, 80))
    e = L.EdgeList.bipartite(D, T, int(rng.integers(2, 12)), seed=3000 + seed)
    p = tmp_path / "c.w.bp.bin"
    e.write(p)
    lab = tmp_path / "t.labels"
    lab.write_text("".join(f"w{i} {i}\n" for i in range(1, T + 1)))
    qs = tmp_path / "q.txt"
    lines = [" ".join(f"w{int(x)}" for x in rng.integers(1, T + 1, int(rng.integers(1, 6)))) for _ in range(8)]
    qs.write_text("\n".join(lines + ["nope w1"]) + "\n")
    o = tmp_path / "o"
    _dump([REF_BIN / f"dump_{app}", p, lab, D, T, qs, 10, o])
    g = O.OracleGraph(p, D, O.BIPARTITE | O.WEIGHTED, nright=T)
    b = O.OracleBM25(g) if app == "bm25" else O.OracleLM(g)
    assert np.array_equal(b.length.view(np.uint32), np.fromfile(str(o) + ".length.f32", np.uint32))
    want = _queries_bin(str(o) + ".queries.bin")
    queries = O.read_queries(lab, qs, D)
    assert len(queries) == len(want)
    for q, act in zip(queries, want):
        _, _, scores, active = b.query(q, 10)
        ids = act[:, 0]
        assert np.array_equal(np.flatnonzero(active), np.sort(ids))
        assert np.array_equal(scores[ids].view(np.uint32), act[:, 1])


@pytest.mark.parametrize("seed", range(6))
def test_graph_simulation(oracle, tmp_path, seed):
    import la3_gb300 as L
    O = oracle
    rng = np.random.default_rng(4000 + seed)
    p, n = _graph(rng, tmp_path, False)
    labs = ["a", "b", "c", "d"]
    lines = ["["] + [("null," if (i == 0 and seed % 2) else '{"l":"%s"},' % labs[int(rng.integers(0, 4))])
                     for i in range(n)] + ["]"]
    dl = tmp_path / "d.labels"
    dl.write_text("\n".join(lines) + "\n")
    qn = int(rng.integers(1, 6))
    ql, qm = tmp_path / "q.labels", tmp_path / "q.mtx"
    ql.write_text("\n".join(labs[int(rng.integers(0, 4))] for _ in range(qn)) + ("\n" if seed % 3 == 0 else ""))
    edges = sorted({(int(rng.integers(0, qn)), int(rng.integers(0, qn))) for _ in range(2 * qn)})
    qm.write_text("".join(f"{a} {b}\n" for a, b in edges))
    o = tmp_path / "o"
    meta = _dump([REF_BIN / "dump_graphsim", dl, p, n, ql, qm, o])
    g = O.OracleGraph(p, n, O.DIRECTED | O.REVERSE)
    labels, qedges = L.read_graphsim_query(ql, qm)
    assert len(labels) == meta["qsize"]
    v, q = L.graphsim_label_ids(L.read_graphsim_labels(dl, n), labels, g.nslots)
    matched, res, nm, _ = g.graphsim(v, q, qedges)
    assert nm == meta["nmatches"]
    assert np.array_equal(matched, np.fromfile(str(o) + ".matched.u8", np.uint8))
    assert np.array_equal(res.reshape(-1), np.fromfile(str(o) + ".res.u8", np.uint8))
