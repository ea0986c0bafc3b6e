"""The command-line drivers keep the reference apps' command lines and print
the same checksums (src/apps/graph_analytics/*.cpp, bm25.cpp): run each on
the golden inputs and compare with the reference's recorded values."""
import re
import subprocess

import numpy as np
import pytest

from conftest import GOLD

DATA = GOLD / "data"
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bins(gpu):
    import la3_gb300.build as B
    B.build()
    return B.BIN


def _run(exe, *args):
    r = subprocess.run([str(exe)] + [str(a) for a in args], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return r.stdout


def _num(out, label):
    m = re.search(re.escape(label) + r"\s*=\s*([-0-9.e+]+)", out)
    assert m, (label, out)
    return float(m.group(1))


def _cases(golden, app):
    return sorted(k for k, v in golden.items() if v["app"] == app)


def test_graph_drivers(bins, golden):
    for name in _cases(golden, "bfs"):
        c = golden[name]
        out = _run(bins / "bfs", DATA / c["file"], c["n"], c["root"])
        assert _num(out, "Reachable Vertices") == c["reachable"], name
        assert _num(out, "Checksum") == c["checksum"], name
    for name in _cases(golden, "sssp"):
        c = golden[name]
        out = _run(bins / "sssp", DATA / c["file"], c["n"], c["root"])
        assert _num(out, "Reachable Vertices") == c["reachable"], name
        assert _num(out, "Checksum") == c["checksum"], name
    for name in _cases(golden, "cc"):
        c = golden[name]
        out = _run(bins / "cc", DATA / c["file"], c["n"])
        assert _num(out, "Checksum") == c["checksum"], name
    for name in _cases(golden, "tc"):
        c = golden[name]
        out = _run(bins / "tc", DATA / c["file"], c["n"])
        assert _num(out, "Triangles") == c["triangles"], name
    for name in _cases(golden, "pr"):
        c = golden[name]
        out = _run(bins / "pr", DATA / c["file"], c["n"], c["iters"])
        assert _num(out, "Degree Checksum") == c["degree_checksum"], name
        # printed with %lf, as the reference prints it
        assert abs(_num(out, "Pagerank Checksum") - c["pr_checksum"]) <= 5e-7, name


@pytest.mark.parametrize("app", ["bm25", "lm"])
def test_ir_driver(bins, golden, app):
    for name in _cases(golden, app):
        c = golden[name]
        ref = np.load(GOLD / f"{name}.npz")
        out = _run(bins / app, DATA / c["file"], DATA / c["labels"], c["ndocs"], c["nterms"],
                   DATA / c["queries"], c["k"])
        assert _num(out, "Collection.Tokens") == c["collection_ntokens"], name
        blocks = re.split(r"^q \d+ \(", out, flags=re.M)[1:]
        assert len(blocks) == c["nqueries"], name
        for qi, b in enumerate(blocks):
            got = [(int(m.group(1)), float(m.group(2))) for m in re.finditer(r"idx (\d+): score ([-0-9.e+]+)", b)]
            # canonical top-k (score desc, id asc) over the reference's scores
            rid, rsc = ref[f"q{qi}_ids"], ref[f"q{qi}_scores"]
            want = sorted(zip(rid.tolist(), rsc.tolist()), key=lambda t: (-t[1], t[0]))[: c["k"]]
            assert [g[0] for g in got] == [w[0] for w in want], (name, qi)
            assert np.allclose([g[1] for g in got], [w[1] for w in want], rtol=0, atol=5e-7), (name, qi)


def test_driver_usage_and_errors(bins):
    r = subprocess.run([str(bins / "bfs")], capture_output=True, text=True)
    assert r.returncode == 1 and "Usage" in r.stdout
    r = subprocess.run([str(bins / "cc"), "/nonexistent.bin", "8"], capture_output=True, text=True)
    assert r.returncode == 1 and "load failed" in r.stderr
