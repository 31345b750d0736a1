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


def test_noalloc_matches_allocating_entry_point(fastcon_lib):
    torch = pytest.importorskip("torch")
    fc = fastcon_lib
    fn = _entry(fc)
    scale = 15
    u, v = graphs.rmat_edges(scale, 8 << scale, seed=41, perm_seed=42)
    nv = 1 << scale
    G = fc.Graph.from_edges(u, v, nv)
    rp, col = G.csr()
    s, t = graphs.pairs_with_degree(np.diff(rp), 700, seed=43)
    s = np.concatenate([s, [5, 7]]).astype(np.int32)  # plus an s == t pair
    t = np.concatenate([t, [5, np.flatnonzero(np.diff(rp) == 0)[0]]]).astype(np.int32)
    nq = len(s)
    for sched in (fc.SCHED_HEURISTIC, fc.SCHED_PLAIN):
        want_c, want_h = fc.stcon_batch(G, s, t, opts=fc.make_opts(sched=sched))
        d_rp, d_col, d_s, d_t = _dev(torch, rp), _dev(torch, col), _dev(torch, s), _dev(torch, t)
        d_c = torch.empty(nq, dtype=torch.int32, device="cuda")
        d_h = torch.empty(nq, dtype=torch.int32, device="cuda")
        for call in range(2):
            d_c.fill_(-7)
            d_h.fill_(-7)
            torch.cuda.synchronize()
            rc = fn(d_rp.data_ptr(), d_col.data_ptr(), nv, len(col), None, None, d_s.data_ptr(),
                    d_t.data_ptr(), nq, d_c.data_ptr(), d_h.data_ptr(), sched, None)
            assert rc == fc.OK, fc.lib().fc_last_error_message()
            torch.cuda.synchronize()
            assert (d_h.cpu().numpy() == want_h).all(), (sched, call)
            assert (d_c.cpu().numpy() == want_c).all(), (sched, call)


def test_noalloc_rejects_graphs_over_its_limit(fastcon_lib):
    fc = fastcon_lib
    fn = _entry(fc)
    dummy = ctypes.c_void_p(1)  # never dereferenced: the size check comes first
    rc = fn(dummy, dummy, MAX_NV + 1, 10, None, None, dummy, dummy, 1, dummy, dummy, 1, None)
    assert rc == fc.ERR_INVALID
    assert b"1048576" in fc.lib().fc_last_error_message()
