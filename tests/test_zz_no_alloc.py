"""la3g_bfs_noalloc: BFS for callers that cannot allocate device memory at
call time (a memory manager owns every byte, or the caller's latency path
must not take cudaMalloc/cudaFree's device-wide synchronisation).  The
caller passes its graph (a CSR in device memory) and the output arrays; the
library's temporaries live in one fixed device array.  These tests check, on
two calls in a row, that its output equals la3g_bfs's for the same graph
(also at the largest size the array allows, from a root without edges and
from a root outside the graph), and that sizes beyond the fixed array are
refused.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_VERTICES = 1 << 20


def bucket_hash(ids: np.ndarray, nvertices: int) -> np.ndarray:
    """The reference's SimpleBucketHasher at one rank (hashers.h:39-68)."""
    height = nvertices // 128
    max_range = height * 128
    ids = ids.astype(np.int64)
    h = ids // 128 + (ids % 128) * height
    return np.where(ids >= max_range, ids, h).astype(np.uint32)


def csr_by_key(src, dst, nslots, key):
    """Symmetric CSR over ids 0..nslots-1 without self-loops or duplicates,
    each row sorted by ascending key of the neighbour."""
    keep = src != dst
    a = np.concatenate([src[keep], dst[keep]]).astype(np.int64)
    b = np.concatenate([dst[keep], src[keep]]).astype(np.int64)
    pairs = np.unique(a * nslots + b)
    rows, cols = pairs // nslots, pairs % nslots
    order = np.lexsort((key[cols], rows))
    rows, cols = rows[order], cols[order]
    ptr = np.zeros(nslots + 1, np.uint32)
    np.add.at(ptr, rows + 1, 1)
    return np.cumsum(ptr, dtype=np.uint64).astype(np.uint32), cols.astype(np.uint32)


def test_bfs_noalloc_matches_bfs_on_two_calls(gpu):
    import torch
    L = gpu
    lib = L._native.lib()
    n = 1 << 12
    e = L.EdgeList.rmat(12, 8, seed=321)
    g = L.Graph.from_edges(e, 0)
    nslots = g.nslots
    src, dst, _ = e.arrays()
    key = bucket_hash(np.arange(nslots), n)
    ptr, col = csr_by_key(src, dst, nslots, key)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(a.view(np.int32)).to(dev)
    d_ptr, d_col, d_key = t(ptr), t(col), t(key)
    d_hops = torch.empty(nslots, dtype=torch.uint8, device=dev)
    d_parent = torch.empty(nslots, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for root in (5, 1234):  # two calls in a row share the fixed scratch
        hops, parent, _ = L.bfs(g, root)
        st = L.Stats()
        rc = lib.la3g_bfs_noalloc(d_ptr.data_ptr(), d_col.data_ptr(), d_key.data_ptr(), nslots, root,
                                  d_hops.data_ptr(), d_parent.data_ptr(), C.c_void_p(stream), C.byref(st))
        assert rc == 0, lib.la3g_last_error_string()
        torch.cuda.synchronize()
        assert np.array_equal(d_hops.cpu().numpy(), hops), root
        assert np.array_equal(d_parent.cpu().numpy().view(np.uint32), parent), root
        assert st.iterations >= 1


def _noalloc(lib, d_ptr, d_col, d_key, nslots, root, d_hops, d_parent, stream):
    import torch
    st = gpu_stats()
    rc = lib.la3g_bfs_noalloc(d_ptr.data_ptr(), d_col.data_ptr(), d_key.data_ptr(), nslots, root,
                              d_hops.data_ptr(), d_parent.data_ptr(), C.c_void_p(stream), C.byref(st))
    assert rc == 0, lib.la3g_last_error_string()
    torch.cuda.synchronize()
    return d_hops.cpu().numpy(), d_parent.cpu().numpy().view(np.uint32), st


def gpu_stats():
    import la3_gb300 as L
    return L.Stats()


def test_bfs_noalloc_at_its_size_limit_and_odd_roots(gpu, tmp_path):
    """A graph of exactly 2^20 vertex slots (ids 0 .. 2^20 - 1), a random
    root, a root with no edges and a root outside the graph, in a row."""
    import torch
    L = gpu
    lib = L._native.lib()
    nslots = MAX_VERTICES
    n = nslots - 1
    rng = np.random.default_rng(11)
    src = rng.integers(1, n + 1, 3 << 20, dtype=np.uint32)
    dst = rng.integers(1, n + 1, 3 << 20, dtype=np.uint32)
    recs = np.stack([src, dst], 1).astype(np.uint32)
    (tmp_path / "g.bin").write_bytes(recs.tobytes())
    g = L.Graph.load_undirected(tmp_path / "g.bin", n)
    assert g.nslots == nslots
    key = bucket_hash(np.arange(nslots), n)
    ptr, col = csr_by_key(src, dst, nslots, key)
    present = np.zeros(nslots, bool)
    present[src] = present[dst] = True
    isolated = int(np.nonzero(~present[1:])[0][0]) + 1
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(a.view(np.int32)).to(dev)
    d_ptr, d_col, d_key = t(ptr), t(col), t(key)
    d_hops = torch.empty(nslots, dtype=torch.uint8, device=dev)
    d_parent = torch.empty(nslots, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for root in (int(src[0]), isolated, nslots + 5):
        hops, parent, _ = L.bfs(g, root)
        h, p, st = _noalloc(lib, d_ptr, d_col, d_key, nslots, root, d_hops, d_parent, stream)
        assert np.array_equal(h, hops), root
        assert np.array_equal(p, parent), root
    assert np.all(h == 255)  # the root outside the graph reaches nothing
    g.free()


def test_bfs_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    lib = gpu._native.lib()
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.la3g_bfs_noalloc(dummy, dummy, dummy, MAX_VERTICES + 1, 0, dummy, dummy, None, None)
    assert rc == 1  # LA3G_EINVAL
    assert b"1048576" in lib.la3g_last_error_string()
    rc = lib.la3g_bfs_noalloc(dummy, dummy, dummy, 0, 0, dummy, dummy, None, None)
    assert rc == 1
