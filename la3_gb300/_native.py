"""ctypes binding of libla3g (the C ABI declared in include/la3g.h).

The library is built in-tree by `la3_gb300.build`.  There is no fallback:
if the shared object is missing or does not load, importing this module
raises, so a caller can never silently run anything but the native path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libla3g.so"


class LA3GError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"la3g status {status}: {message}")
        self.status = status


class Stats(C.Structure):
    _fields_ = [
        ("device_ms", C.c_double),
        ("host_ms", C.c_double),
        ("iterations", C.c_uint32),
        ("pull_iterations", C.c_uint32),
        ("teps_edges", C.c_uint64),
        ("edges_examined", C.c_uint64),
        ("algo_bytes", C.c_uint64),
        ("kernel_launches", C.c_uint32),
        ("reserved", C.c_uint32),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class GraphInfo(C.Structure):
    _fields_ = [
        ("nslots", C.c_uint32),
        ("nvertices", C.c_uint32),
        ("nleft", C.c_uint32),
        ("flags", C.c_uint32),
        ("nrecords", C.c_uint64),
        ("nentries", C.c_uint64),
        ("nregular", C.c_uint32),
        ("nsink", C.c_uint32),
        ("nsource", C.c_uint32),
        ("nisolated", C.c_uint32),
        ("device_bytes", C.c_uint64),
    ]


class Edges(C.Structure):
    _fields_ = [
        ("src", C.POINTER(C.c_uint32)),
        ("dst", C.POINTER(C.c_uint32)),
        ("w", C.POINTER(C.c_uint32)),
        ("m", C.c_uint64),
        ("n", C.c_uint32),
        ("nright", C.c_uint32),
        ("weighted", C.c_int),
        ("reserved", C.c_int),
    ]


class Query(C.Structure):
    _fields_ = [
        ("kind", C.c_uint32),
        ("graph", C.c_uint32),
        ("root", C.c_uint32),
        ("k", C.c_uint32),
        ("terms", C.POINTER(C.c_uint32)),
        ("nterms", C.c_uint32),
        ("out", C.c_void_p),
        ("scores_out", C.POINTER(C.c_float)),
    ]


class QueryResult(C.Structure):
    _fields_ = [
        ("status", C.c_int),
        ("kind", C.c_uint32),
        ("queue_ms", C.c_double),
        ("latency_ms", C.c_double),
        ("in_flight", C.c_uint32),
        ("nout", C.c_uint32),
    ]


class ServerStats(C.Structure):
    _fields_ = [
        ("budget_bytes", C.c_uint64),
        ("used_bytes", C.c_uint64),
        ("completed", C.c_uint64),
        ("queued", C.c_uint64),
        ("pending", C.c_uint64),
        ("ngraphs", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


class DeviceGraph(C.Structure):
    _fields_ = [
        ("row_ptr", C.c_void_p),
        ("col", C.c_void_p),
        ("weight", C.c_void_p),
        ("hash_of_pos", C.c_void_p),
        ("id_of_pos", C.c_void_p),
        ("pos_of_id", C.c_void_p),
        ("nslots", C.c_uint32),
        ("nregular", C.c_uint32),
        ("nsink", C.c_uint32),
        ("nsource", C.c_uint32),
        ("flags", C.c_uint32),
        ("reserved", C.c_uint32),
        ("nentries", C.c_uint64),
        ("stream", C.c_void_p),
    ]


_P = C.c_void_p
_u32p = C.POINTER(C.c_uint32)
_u8p = C.POINTER(C.c_uint8)
_f64p = C.POINTER(C.c_double)
_f32p = C.POINTER(C.c_float)
_u64p = C.POINTER(C.c_uint64)
_statp = C.POINTER(Stats)

# name -> (restype, argtypes); every entry point the header declares.
SIGNATURES = {
    "la3g_last_error_string": (C.c_char_p, []),
    "la3g_status_string": (C.c_char_p, [C.c_int]),
    "la3g_graph_load": (C.c_int, [C.c_char_p, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(_P)]),
    "la3g_graph_from_records": (C.c_int, [_P, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(_P)]),
    "la3g_graph_from_edges": (C.c_int, [C.POINTER(Edges), C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(_P)]),
    "la3g_graph_free": (None, [_P]),
    "la3g_graph_info_get": (C.c_int, [_P, C.POINTER(GraphInfo)]),
    "la3g_graph_set_stream": (C.c_int, [_P, _P]),
    "la3g_graph_positions": (C.c_int, [_P, _u32p, _u32p]),
    "la3g_graph_device_view": (C.c_int, [_P, C.POINTER(DeviceGraph)]),
    "la3g_graph_push_view": (C.c_int, [_P, C.POINTER(_P), C.POINTER(_P)]),
    "la3g_pr": (C.c_int, [_P, C.c_uint32, _f64p, _u32p, _statp]),
    "la3g_pr_f32": (C.c_int, [_P, C.c_uint32, C.c_double, _f64p, _f64p, _statp]),
    "la3g_pr_f32_tiled": (C.c_int, [_P, C.c_uint32, C.c_double, _f64p, _f64p, _statp]),
    "la3g_bfs": (C.c_int, [_P, C.c_uint32, _u8p, _u32p, _statp]),
    "la3g_sssp": (C.c_int, [_P, C.c_uint32, _u32p, _statp]),
    "la3g_cc": (C.c_int, [_P, _u32p, _statp]),
    "la3g_tc": (C.c_int, [_P, _u64p, _u32p, _statp]),
    "la3g_bm25_prepare": (C.c_int, [_P, _u64p, _f32p, _f32p]),
    "la3g_bm25_query": (C.c_int, [_P, _u32p, C.c_uint32, C.c_uint32, _u32p, _f32p, _u32p, _f32p, _u8p, _statp]),
    "la3g_degree": (C.c_int, [_P, _u32p, C.c_uint32, _u32p, _u32p, _u32p, _statp]),
    "la3g_topk_u32": (C.c_int, [_u32p, C.c_uint32, C.c_uint32, _u32p, _u32p, _u32p]),
    "la3g_lm_prepare": (C.c_int, [_P, _u64p, _f32p]),
    "la3g_lm_query": (C.c_int, [_P, _u32p, C.c_uint32, C.c_uint32, _u32p, _f32p, _u32p, _f32p, _u8p, _statp]),
    "la3g_bfs_batch": (C.c_int, [_P, _u32p, C.c_uint32, _u8p, _statp]),
    "la3g_sssp_batch": (C.c_int, [_P, _u32p, C.c_uint32, _u32p, _statp]),
    "la3g_bfs_noalloc": (C.c_int, [_P, _P, _P, C.c_uint32, C.c_uint32, _P, _P, _P, _statp]),
    "la3g_batch_autotune": (C.c_int, [_P, _u32p, C.c_uint32, C.c_char_p, C.c_size_t]),
    "la3g_batch_config": (C.c_int, [_P, C.c_int, C.c_int, C.c_double]),
    "la3g_batch_set_wait_limit": (C.c_int, [_P, C.c_longlong]),
    "la3g_batch_sssp_window": (C.c_int, [_P, C.c_uint32]),
    "la3g_gen_rmat": (C.c_int, [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_uint64, C.c_int,
                                C.c_uint64, C.POINTER(Edges)]),
    "la3g_gen_er": (C.c_int, [C.c_uint32, C.c_uint64, C.c_uint64, C.c_int, C.c_uint64, C.POINTER(Edges)]),
    "la3g_gen_bipartite": (C.c_int, [C.c_uint32, C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_uint64,
                                     C.POINTER(Edges)]),
    "la3g_edges_write": (C.c_int, [C.POINTER(Edges), C.c_char_p, C.c_int]),
    "la3g_edges_free": (None, [C.POINTER(Edges)]),
    "la3g_server_create": (C.c_int, [C.c_uint64, C.c_uint32, C.c_uint32, C.POINTER(_P)]),
    "la3g_server_add_graph": (C.c_int, [_P, _P, _u32p]),
    "la3g_server_submit": (C.c_int, [_P, C.POINTER(Query), _u64p]),
    "la3g_server_poll": (C.c_int, [_P, C.c_uint64, C.c_int, C.POINTER(QueryResult)]),
    "la3g_server_info": (C.c_int, [_P, C.POINTER(ServerStats)]),
    "la3g_server_lanes": (C.c_int, [_P, C.c_uint32, _u32p]),
    "la3g_server_set_solo": (C.c_int, [_P, C.c_uint32, C.c_uint32]),
    "la3g_server_free": (None, [_P]),
    "la3g_profile_enable": (None, [C.c_int]),
    "la3g_profile_reset": (None, []),
    "la3g_profile_report": (C.c_size_t, [C.c_char_p, C.c_size_t]),
}

_lib = None


def lib() -> C.CDLL:
    """Loads libla3g (once).  Raises if it is missing: there is no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing; build it with `python -m la3_gb300.build`")
    L = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status: int) -> None:
    if status != 0:
        msg = lib().la3g_last_error_string()
        raise LA3GError(status, msg.decode() if msg else "")
