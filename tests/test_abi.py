"""The C-ABI library loads and exports every entry point include/la3g.h
declares; host-only calls (generators, errors) work without a GPU."""
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def declared_symbols():
    text = (ROOT / "include" / "la3g.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(la3g_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    syms = declared_symbols()
    for s in ["la3g_graph_load", "la3g_pr", "la3g_bfs", "la3g_sssp", "la3g_cc", "la3g_tc", "la3g_bm25_prepare",
              "la3g_bm25_query", "la3g_lm_prepare", "la3g_lm_query", "la3g_degree", "la3g_topk_u32",
              "la3g_bfs_batch", "la3g_sssp_batch",
              "la3g_last_error_string"]:
        assert s in syms


def test_library_exports_every_declared_symbol(native):
    so = native._native.LIB_PATH
    out = subprocess.run(["nm", "-D", "--defined-only", str(so)], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (la3g_[a-z0-9_]+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    L = native._native.lib()
    for s in declared_symbols():
        assert hasattr(L, s)


def test_binding_covers_header(native):
    assert set(declared_symbols()) <= set(native._native.SIGNATURES)


def test_status_strings(native):
    L = native._native.lib()
    assert L.la3g_status_string(0) == b"ok"
    assert L.la3g_status_string(4) == b"out of memory"


def test_generator_is_deterministic(native):
    E = native.EdgeList
    a = E.rmat(9, 8, seed=3).arrays()
    b = E.rmat(9, 8, seed=3).arrays()
    c = E.rmat(9, 8, seed=4).arrays()
    assert all(np.array_equal(x, y) for x, y in zip(a[:2], b[:2]))
    assert not np.array_equal(a[1], c[1])
    src, dst, _ = a
    assert src.min() >= 1 and dst.min() >= 1 and max(src.max(), dst.max()) <= 512
    assert not np.any(src == dst)
    key = src.astype(np.uint64) << 32 | dst
    assert np.all(np.diff(key.astype(np.int64)) > 0)  # sorted, no duplicates


def test_generator_thread_count_does_not_matter(native, monkeypatch):
    E = native.EdgeList
    monkeypatch.setenv("LA3G_THREADS", "1")
    a = E.rmat(17, 2, seed=9, weighted=True).arrays()
    monkeypatch.setenv("LA3G_THREADS", "7")
    b = E.rmat(17, 2, seed=9, weighted=True).arrays()
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    w = a[2]
    assert w.min() >= 1 and w.max() <= 128


def test_bipartite_generator_caps_document_frequency(native):
    e = native.EdgeList.bipartite(3000, 500, 20, zipf_s=1.1, df_cap=0.9, seed=5)
    src, dst, w = e.arrays()
    assert src.min() >= 1 and src.max() <= 3000 and dst.min() >= 1 and dst.max() <= 500
    df = np.bincount(dst, minlength=501)
    assert df.max() < 0.9 * 3000
    assert w.min() >= 1
    pairs = src.astype(np.uint64) << 32 | dst
    assert np.unique(pairs).size == pairs.size


def test_edges_write_layout(native, tmp_path):
    e = native.EdgeList.rmat(8, 4, seed=1, weighted=True)
    p = tmp_path / "g.w.bin"
    e.write(p, header=True)
    raw = np.fromfile(p, np.uint32)
    src, dst, w = e.arrays()
    assert raw[0] == 255 and raw[1] == 255 and raw[2] == e.m and raw[3] == 0
    rec = raw[4:].reshape(-1, 3)
    assert np.array_equal(rec[:, 0], src) and np.array_equal(rec[:, 1], dst) and np.array_equal(rec[:, 2], w)


def test_load_errors_are_reported(native, tmp_path):
    G = native.Graph
    with pytest.raises(native.LA3GError) as ei:
        G.load(tmp_path / "missing.bin", 8, 0)
    assert ei.value.status == 2  # EIO before any device work
    p = tmp_path / "trunc.bin"
    p.write_bytes(b"\x01\x00\x00\x00\x02\x00\x00\x00\x03")
    with pytest.raises(native.LA3GError) as ei:
        G.load(p, 8, 0)
    assert ei.value.status == 3  # EFORMAT
    with pytest.raises(native.LA3GError) as ei:
        G.load(p, 8, native.BIPARTITE | native.ACYCLIC | native.DIRECTED)
    assert ei.value.status == 1  # EINVAL flags


def test_drivers_and_programs_are_built(native):
    """The nine command-line drivers and the vertex-program library exist;
    a driver prints its usage without touching a GPU."""
    import la3_gb300.build as B
    for d in ("pr", "bfs", "sssp", "cc", "tc", "bm25", "lm", "degree", "graphsim"):
        assert (B.BIN / d).exists(), d
    r = subprocess.run([str(B.BIN / "tc")], capture_output=True, text=True)
    assert r.returncode == 1 and "Usage" in r.stdout
    out = subprocess.run(["nm", "-D", "--defined-only", str(B.PROGRAMS_LIB)], capture_output=True, text=True,
                         check=True).stdout
    # every entry point include/la3g_programs.h declares
    hdr = (B.INCLUDE / "la3g_programs.h").read_text()
    declared = re.findall(r"^int (la3gp_\w+)\(", hdr, flags=re.M)
    assert {"la3gp_degree", "la3gp_pagerank", "la3gp_bfs", "la3gp_sssp", "la3gp_cc", "la3gp_graphsim", "la3gp_tc",
            "la3gp_degree_topk", "la3gp_bfs_topk"} <= set(declared)
    for s in declared:
        assert re.search(r"\bT " + s + r"\b", out), s


def test_new_entry_points_reject_bad_arguments(native):
    """LM, degree, top-k and graph simulation refuse bad arguments with
    LA3G_EINVAL and a message, before any device work."""
    import ctypes as C
    import la3_gb300.build as B
    L = native._native.lib()
    u32 = (C.c_uint32 * 8)()
    assert L.la3g_lm_prepare(None, None, None) == 1 and L.la3g_last_error_string()
    assert L.la3g_lm_query(None, None, 0, 10, None, None, None, None, None, None) == 1
    assert L.la3g_degree(None, None, 3, None, None, None, None) == 1
    assert L.la3g_topk_u32(None, 5, 3, None, None, None) == 1              # values missing
    assert L.la3g_topk_u32(u32, 8, 65, None, None, None) == 1              # k above 64
    assert b"64" in L.la3g_last_error_string()
    progs = C.CDLL(str(B.PROGRAMS_LIB))
    progs.la3gp_graphsim.argtypes = [C.c_void_p] + [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32,
                                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    assert progs.la3gp_graphsim(None, None, 4, None, None, 0, None, None, None, None) == 1
    # the engine-program entry points refuse a null graph before any device work
    assert progs.la3gp_tc(None, None, None, None) == 1
    progs.la3gp_degree_topk.argtypes = [C.c_void_p, C.c_uint32] + [C.c_void_p] * 5
    assert progs.la3gp_degree_topk(None, 3, None, None, None, None, None) == 1
    progs.la3gp_bfs_topk.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]
    assert progs.la3gp_bfs_topk(None, 1, 3, None, None) == 1
    # the tiled PageRank and the push view refuse a null graph
    assert L.la3g_pr_f32_tiled(None, 5, 0.0, None, None, None) == 1
    assert L.la3g_graph_push_view(None, None, None) == 1
    assert L.la3g_batch_sssp_window(None, 0) == 1
