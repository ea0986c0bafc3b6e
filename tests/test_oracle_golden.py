"""The C oracle (restatement) against golden vectors produced by the
reference itself (tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

from conftest import GOLD

DATA = GOLD / "data"


def _cases(golden, app):
    return sorted(k for k, v in golden.items() if v["app"] == app)


def test_golden_manifest_complete(golden):
    apps = {v["app"] for v in golden.values()}
    assert apps == {"pr", "bfs", "sssp", "cc", "tc", "bm25", "lm", "graphsim"}
    for k in golden:
        assert (GOLD / f"{k}.npz").exists(), k


@pytest.mark.parametrize("app", ["pr", "bfs", "sssp", "cc", "tc", "bm25", "lm"])
def test_oracle_matches_reference(golden, oracle, app):
    O = oracle
    for name in _cases(golden, app):
        c = golden[name]
        ref = np.load(GOLD / f"{name}.npz")
        f = DATA / c["file"]
        if app == "pr":
            g = O.OracleGraph(f, c["n"], O.DIRECTED)
            rank, deg = g.pagerank(c["iters"])
            assert np.array_equal(rank.view(np.uint64), ref["rank"].view(np.uint64)), name  # bit-exact
            assert np.array_equal(deg, ref["degree"]), name
        elif app == "bfs":
            g = O.OracleGraph(f, c["n"], 0)
            hops, parent, _ = g.bfs(c["root"])
            assert np.array_equal(hops, ref["hops"]), name
            assert np.array_equal(parent, ref["parent"]), name
            assert int((hops.astype(np.int64) * parent).sum()) == c["checksum"], name
        elif app == "sssp":
            g = O.OracleGraph(f, c["n"], O.DIRECTED | O.WEIGHTED)
            dist, _ = g.sssp(c["root"])
            assert np.array_equal(dist, ref["dist"]), name
            assert int(dist.astype(np.int64).sum()) == c["checksum"], name
        elif app == "cc":
            g = O.OracleGraph(f, c["n"], 0)
            lab, _ = g.cc()
            assert np.array_equal(lab, ref["label"]), name
        elif app == "tc":
            g = O.OracleGraph(f, c["n"], O.DIRECTED | O.ACYCLIC)
            total, per = g.tc()
            assert np.array_equal(per, ref["ntri"]), name
            assert total == c["triangles"], name
        else:
            g = O.OracleGraph(f, c["ndocs"], O.BIPARTITE | O.WEIGHTED, nright=c["nterms"])
            b = O.OracleBM25(g) if app == "bm25" else O.OracleLM(g)
            assert b.collection_ntokens == c["collection_ntokens"], name
            assert np.array_equal(b.length.view(np.uint32), ref["length"].view(np.uint32)), name
            queries = O.read_queries(DATA / c["labels"], DATA / c["queries"], c["ndocs"])
            assert len(queries) == c["nqueries"]
            for qi, q in enumerate(queries):
                ids, sc, scores, active = b.query(q, c["k"])
                rid, rsc = ref[f"q{qi}_ids"], ref[f"q{qi}_scores"]
                assert np.array_equal(np.flatnonzero(active), np.sort(rid)), (name, qi)
                order = np.argsort(rid)
                assert np.array_equal(scores[rid[order]].view(np.uint32), rsc[order].view(np.uint32)), (name, qi)
                # the reference's top-k agrees with the canonical order up to ties
                tk = ref[f"q{qi}_topk_scores"]
                assert np.array_equal(np.sort(sc)[::-1].view(np.uint32), np.sort(tk)[::-1].view(np.uint32)), (name, qi)


def test_oracle_graphsim_matches_reference(golden, oracle):
    """Graph simulation: the reference's per-vertex result strings and match
    flags (its own sample data graph and queries, plus synthetic ones); the
    inputs are read by the package's readers, which follow the reference's
    parsing rules."""
    import la3_gb300 as L
    O = oracle
    for name in _cases(golden, "graphsim"):
        c = golden[name]
        ref = np.load(GOLD / f"{name}.npz")
        g = O.OracleGraph(DATA / c["file"], c["n"], O.DIRECTED | O.REVERSE)
        vl = L.read_graphsim_labels(DATA / c["labels"], c["n"])
        ql, qe = L.read_graphsim_query(DATA / c["qlabels"], DATA / c["qmtx"])
        assert len(ql) == c["qsize"], name
        v, q = L.graphsim_label_ids(vl, ql, g.nslots)
        matched, res, nm, _ = g.graphsim(v, q, qe)
        assert nm == c["nmatches"], name
        assert np.array_equal(matched, ref["matched"]), name
        assert np.array_equal(res, ref["res"]), name


def test_oracle_rejects_out_of_range_ids(oracle, tmp_path):
    p = tmp_path / "bad.bin"
    np.array([[1, 2], [3, 99]], np.uint32).tofile(p)
    with pytest.raises(RuntimeError, match="out of range"):
        oracle.OracleGraph(p, 8, 0)


def test_planted_mistake_is_caught(oracle, golden):
    """A deliberate error planted in the oracle's output must fail the
    comparison (the checker can see a one-ulp difference)."""
    c = golden["rmat10_pr"]
    ref = np.load(GOLD / "rmat10_pr.npz")["rank"]
    g = oracle.OracleGraph(DATA / c["file"], c["n"], oracle.DIRECTED)
    rank, _ = g.pagerank(c["iters"])
    rank[17] = np.nextafter(rank[17], 1.0)
    assert not np.array_equal(rank.view(np.uint64), ref.view(np.uint64))
