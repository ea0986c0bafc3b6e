"""ctypes wrapper of the C oracle (oracle/la3_oracle.c).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline legs use it as the checker.  The product (la3_gb300) never
imports it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

HERE = Path(__file__).resolve().parent
SO = HERE / "_build" / "liboracle.so"
CLI = HERE / "_build" / "la3_oracle"
REF_BIN = HERE / "_ref" / "bin"

DIRECTED, REVERSE, ACYCLIC, BIPARTITE, WEIGHTED = 1, 2, 4, 8, 16

_lib = None


def build() -> None:
    """Compiles the restatement (and nothing else) with the oracle Makefile."""
    subprocess.run(["make", "-s", "-C", str(HERE), "port"], check=True)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not SO.exists():
            build()
        L = C.CDLL(str(SO))
        P = C.c_void_p
        u32p, u8p, f64p, f32p, u64p = (C.POINTER(C.c_uint32), C.POINTER(C.c_uint8), C.POINTER(C.c_double),
                                       C.POINTER(C.c_float), C.POINTER(C.c_uint64))
        sig = {
            "og_load": (C.c_int, [C.c_char_p, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(P)]),
            "og_free": (None, [P]),
            "og_nslots": (C.c_uint32, [P]),
            "og_nedges": (C.c_uint64, [P]),
            "og_classes": (None, [P, u32p, u32p, u32p]),
            "og_positions": (None, [P, u32p, u32p]),
            "og_hash": (C.c_uint32, [P, C.c_uint32]),
            "og_pagerank": (C.c_int, [P, C.c_uint32, f64p, u32p]),
            "og_bfs": (C.c_int, [P, C.c_uint32, u8p, u32p, u32p]),
            "og_sssp": (C.c_int, [P, C.c_uint32, u32p, u32p]),
            "og_cc": (C.c_int, [P, u32p, u32p]),
            "og_tc": (C.c_int, [P, u32p, u64p]),
            "og_graphsim": (C.c_int, [P, u32p, C.c_uint32, u32p, u32p, C.c_uint32, u8p, C.c_char_p, u32p, u32p]),
            "og_bm25_prepare": (C.c_int, [P, C.POINTER(P), u64p, f32p, f32p]),
            "og_bm25_query": (C.c_int, [P, u32p, C.c_uint32, C.c_uint32, f32p, u8p, u32p, f32p, u32p]),
            "og_bm25_free": (None, [P]),
            "og_lm_prepare": (C.c_int, [P, C.POINTER(P), u64p, f32p]),
            "og_lm_query": (C.c_int, [P, u32p, C.c_uint32, C.c_uint32, f32p, u8p, u32p, f32p, u32p]),
            "og_lm_free": (None, [P]),
            "og_last_error": (C.c_char_p, []),
        }
        for k, (r, a) in sig.items():
            f = getattr(L, k)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def _check(rc: int) -> None:
    if rc != 0:
        raise RuntimeError(f"oracle error {rc}: {lib().og_last_error().decode()}")


class OracleGraph:
    """og_load (graph.hpp:37-214 restated)."""

    def __init__(self, path: str, n: int, flags: int, nright: int = 0):
        self.h = C.c_void_p()
        _check(lib().og_load(str(path).encode(), n, nright, flags, C.byref(self.h)))
        self.flags = flags
        self.nslots = lib().og_nslots(self.h)
        self.nedges = lib().og_nedges(self.h)

    def classes(self) -> tuple[int, int, int]:
        a, b, c = C.c_uint32(), C.c_uint32(), C.c_uint32()
        lib().og_classes(self.h, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value

    def positions(self) -> tuple[np.ndarray, np.ndarray]:
        pos = np.empty(self.nslots, np.uint32)
        ids = np.empty(self.nslots, np.uint32)
        lib().og_positions(self.h, _p(pos, C.c_uint32), _p(ids, C.c_uint32))
        return pos, ids

    def pagerank(self, iters: int):
        r = np.empty(self.nslots, np.float64)
        d = np.empty(self.nslots, np.uint32)
        _check(lib().og_pagerank(self.h, iters, _p(r, C.c_double), _p(d, C.c_uint32)))
        return r, d

    def bfs(self, root: int):
        h = np.empty(self.nslots, np.uint8)
        p = np.empty(self.nslots, np.uint32)
        it = C.c_uint32()
        _check(lib().og_bfs(self.h, root, _p(h, C.c_uint8), _p(p, C.c_uint32), C.byref(it)))
        return h, p, it.value

    def sssp(self, root: int):
        d = np.empty(self.nslots, np.uint32)
        it = C.c_uint32()
        _check(lib().og_sssp(self.h, root, _p(d, C.c_uint32), C.byref(it)))
        return d, it.value

    def cc(self):
        lab = np.empty(self.nslots, np.uint32)
        it = C.c_uint32()
        _check(lib().og_cc(self.h, _p(lab, C.c_uint32), C.byref(it)))
        return lab, it.value

    def tc(self):
        t = np.empty(self.nslots, np.uint32)
        tot = C.c_uint64()
        _check(lib().og_tc(self.h, _p(t, C.c_uint32), C.byref(tot)))
        return tot.value, t

    def graphsim(self, vlabel, qlabel, qedges):
        """Graph simulation on a graph loaded DIRECTED | REVERSE: (matched
        flags, res as an nslots x qsize uint8 array, match count, iterations)."""
        v = np.ascontiguousarray(np.asarray(vlabel, np.uint32))
        q = np.ascontiguousarray(np.asarray(qlabel, np.uint32))
        e = np.ascontiguousarray(np.asarray(qedges, np.uint32).reshape(-1))
        matched = np.empty(self.nslots, np.uint8)
        res = C.create_string_buffer(self.nslots * q.size)
        nm, it = C.c_uint32(), C.c_uint32()
        _check(lib().og_graphsim(self.h, _p(v, C.c_uint32), q.size, _p(q, C.c_uint32), _p(e, C.c_uint32),
                                 e.size // 2, _p(matched, C.c_uint8), res, C.byref(nm), C.byref(it)))
        r = np.frombuffer(res.raw, np.uint8).reshape(self.nslots, q.size).copy()
        return matched, r, nm.value, it.value

    def __del__(self):
        try:
            if self.h:
                lib().og_free(self.h)
                self.h = None
        except Exception:
            pass


class OracleBM25:
    def __init__(self, g: OracleGraph):
        self.g = g
        self.h = C.c_void_p()
        ntok = C.c_uint64()
        avg = C.c_float()
        self.length = np.empty(g.nslots, np.float32)
        _check(lib().og_bm25_prepare(g.h, C.byref(self.h), C.byref(ntok), C.byref(avg), _p(self.length, C.c_float)))
        self.collection_ntokens = ntok.value
        self.avg_doc_length = avg.value

    def query(self, term_vids: Sequence[int], k: int):
        q = np.ascontiguousarray(np.asarray(term_vids, np.uint32))
        n = self.g.nslots
        scores = np.empty(n, np.float32)
        active = np.empty(n, np.uint8)
        ids = np.empty(max(k, 1), np.uint32)
        sc = np.empty(max(k, 1), np.float32)
        nk = C.c_uint32()
        _check(lib().og_bm25_query(self.h, _p(q, C.c_uint32), q.size, k, _p(scores, C.c_float), _p(active, C.c_uint8),
                                   _p(ids, C.c_uint32), _p(sc, C.c_float), C.byref(nk)))
        return ids[:nk.value].copy(), sc[:nk.value].copy(), scores, active

    def __del__(self):
        try:
            if self.h:
                lib().og_bm25_free(self.h)
                self.h = None
        except Exception:
            pass


class OracleLM:
    """LM (lm.cpp:8-144) on the oracle's engine: same query interface as
    OracleBM25."""

    def __init__(self, g: OracleGraph):
        self.g = g
        self.h = C.c_void_p()
        ntok = C.c_uint64()
        self.length = np.empty(g.nslots, np.float32)
        _check(lib().og_lm_prepare(g.h, C.byref(self.h), C.byref(ntok), _p(self.length, C.c_float)))
        self.collection_ntokens = ntok.value

    def query(self, term_vids: Sequence[int], k: int):
        q = np.ascontiguousarray(np.asarray(term_vids, np.uint32))
        n = self.g.nslots
        scores = np.empty(n, np.float32)
        active = np.empty(n, np.uint8)
        ids = np.empty(max(k, 1), np.uint32)
        sc = np.empty(max(k, 1), np.float32)
        nk = C.c_uint32()
        _check(lib().og_lm_query(self.h, _p(q, C.c_uint32), q.size, k, _p(scores, C.c_float), _p(active, C.c_uint8),
                                 _p(ids, C.c_uint32), _p(sc, C.c_float), C.byref(nk)))
        return ids[:nk.value].copy(), sc[:nk.value].copy(), scores, active

    def __del__(self):
        try:
            if self.h:
                lib().og_lm_free(self.h)
                self.h = None
        except Exception:
            pass


def read_queries(labels_path: str, queries_path: str, ndocs: int) -> list[list[int]]:
    """prepare_queries (helpers.hpp:76-123): label of line i -> vertex i + 1 +
    ndocs; unknown labels map to 0."""
    ids = {}
    with open(labels_path) as f:
        i = 0
        for line in f:
            parts = line.split()
            if not parts:
                continue
            ids[parts[0]] = i + 1 + ndocs
            i += 1
    out = []
    with open(queries_path) as f:
        for line in f:
            toks = line.split()
            if not toks:
                continue
            out.append([ids.get(t, 0) for t in toks])
    return out


def ref_available() -> bool:
    return (REF_BIN / "dump_pr").exists()
