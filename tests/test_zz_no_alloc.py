"""fc_stcon_batch_noalloc: s-t queries for callers that cannot allocate
device memory (for example a service whose device memory is all reserved by
its own pool, or a plug-in inside a framework that owns the device memory).

The entry point works in a fixed device array inside the library instead of
allocating.  These tests call it through the C ABI with device arrays and
check its answers against the regular (allocating) batch entry point, on two
calls in a row (the second call must not be disturbed by what the first one
left in the shared array).  Answers are integers: they must be identical.
This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

from fastcon import graphs

pytestmark = pytest.mark.gpu

MAX_NV = 1 << 20


def _entry(fc):
    return fc.lib().fc_stcon_batch_noalloc


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).cuda()


def _reverse_csr(nv, rp, col):
    rows = np.repeat(np.arange(nv, dtype=np.int64), np.diff(rp))
    o = np.lexsort((rows, col))
    rrp = np.zeros(nv + 1, np.int64)
    np.add.at(rrp, col.astype(np.int64) + 1, 1)
    return np.cumsum(rrp).astype(np.int32), rows[o].astype(np.int32)


def _compare(torch, fc, G, s, t, sched, directed=False, bad=()):
    """Two calls in a row of the no-alloc entry point against fc_stcon_batch;
    queries listed in `bad` hold out-of-range ids (connected 0, hops -2)."""
    fn = _entry(fc)
    nv = G.nv
    rp, col = G.csr()
    ok = np.setdiff1d(np.arange(len(s)), np.asarray(bad, np.int64))
    want_c = np.zeros(len(s), np.int32)
    want_h = np.full(len(s), -2, np.int32)
    c, h = fc.stcon_batch(G, s[ok], t[ok], opts=fc.make_opts(sched=sched))
    want_c[ok] = c
    want_h[ok] = h
    d_rp, d_col, d_s, d_t = _dev(torch, rp), _dev(torch, col), _dev(torch, s), _dev(torch, t)
    d_rrp = d_rcol = None
    if directed:
        rrp, rcol = _reverse_csr(nv, rp, col)
        d_rrp, d_rcol = _dev(torch, rrp), _dev(torch, rcol)
    nq = len(s)
    d_c = torch.empty(nq, dtype=torch.int32, device="cuda")
    d_h = torch.empty(nq, dtype=torch.int32, device="cuda")
    for call in range(2):
        d_c.fill_(-7)
        d_h.fill_(-7)
        torch.cuda.synchronize()
        rc = fn(d_rp.data_ptr(), d_col.data_ptr(), nv, len(col),
                d_rrp.data_ptr() if directed else None, d_rcol.data_ptr() if directed else None,
                d_s.data_ptr(), d_t.data_ptr(), nq, d_c.data_ptr(), d_h.data_ptr(), sched, None)
        assert rc == fc.OK, fc.lib().fc_last_error_message()
        torch.cuda.synchronize()
        assert (d_h.cpu().numpy() == want_h).all(), (sched, call)
        assert (d_c.cpu().numpy() == want_c).all(), (sched, call)


def test_noalloc_matches_allocating_entry_point(fastcon_lib):
    torch = pytest.importorskip("torch")
    fc = fastcon_lib
    scale = 15
    u, v = graphs.rmat_edges(scale, 8 << scale, seed=41, perm_seed=42)
    nv = 1 << scale
    G = fc.Graph.from_edges(u, v, nv)
    rp, _ = G.csr()
    s, t = graphs.pairs_with_degree(np.diff(rp), 700, seed=43)
    s = np.concatenate([s, [5, 7]]).astype(np.int32)  # plus an s == t pair
    t = np.concatenate([t, [5, np.flatnonzero(np.diff(rp) == 0)[0]]]).astype(np.int32)
    for sched in (fc.SCHED_HEURISTIC, fc.SCHED_PLAIN):
        _compare(torch, fc, G, s, t, sched)


def test_noalloc_directed_graph_and_bad_ids(fastcon_lib):
    """A directed graph passed with its reverse CSR (the t side walks it),
    and queries whose ids are out of range."""
    torch = pytest.importorskip("torch")
    fc = fastcon_lib
    scale = 14
    nv = 1 << scale
    u, v = graphs.rmat_edges(scale, 8 << scale, seed=44, perm_seed=45)
    G = fc.Graph.from_edges(u, v, nv, flags=fc.INGEST_DIRECTED)
    s, t = graphs.uniform_pairs(nv, 500, seed=46)
    s[[3, 77]] = [-1, nv]
    t[[120]] = [nv + 5]
    _compare(torch, fc, G, s, t, fc.SCHED_HEURISTIC, directed=True, bad=(3, 77, 120))


def test_noalloc_at_its_vertex_limit_with_hubs(fastcon_lib):
    """Graphs of 2^20 vertices (the limit) and 2^20 - 3 (not a multiple of the
    16-byte initialisation stores), each with hub rows of 50,000 and 20,000
    entries next to R-MAT edges."""
    torch = pytest.importorskip("torch")
    fc = fastcon_lib
    for nv in (MAX_NV, MAX_NV - 3):
        u, v = graphs.rmat_edges(20, 4 << 20, seed=47, perm_seed=48)
        keep = (u < nv) & (v < nv)
        u, v = u[keep], v[keep]
        hub_u = np.concatenate([np.full(50000, nv - 1), np.full(20000, 17)]).astype(np.int32)
        hub_v = np.concatenate([np.arange(0, 50000), np.arange(nv - 20001, nv - 1)]).astype(np.int32)
        G = fc.Graph.from_edges(np.concatenate([u, hub_u]), np.concatenate([v, hub_v]), nv)
        rp, _ = G.csr()
        s, t = graphs.pairs_with_degree(np.diff(rp), 300, seed=49)
        s = np.concatenate([s, [nv - 1, 17]]).astype(np.int32)
        t = np.concatenate([t, [17, nv - 2]]).astype(np.int32)
        _compare(torch, fc, G, s, t, fc.SCHED_HEURISTIC)
        G.free()


def test_noalloc_rejects_graphs_over_its_limit(fastcon_lib):
    fc = fastcon_lib
    fn = _entry(fc)
    dummy = ctypes.c_void_p(1)  # never dereferenced: the argument checks come first
    rc = fn(dummy, dummy, MAX_NV + 1, 10, None, None, dummy, dummy, 1, dummy, dummy, 1, None)
    assert rc == fc.ERR_INVALID
    assert b"1048576" in fc.lib().fc_last_error_message()
    rc = fn(dummy, dummy, 100, 10, None, None, dummy, dummy, 1, dummy, dummy, 7, None)
    assert rc == fc.ERR_INVALID  # not an FC_SCHED_* value
    assert b"sched" in fc.lib().fc_last_error_message()
