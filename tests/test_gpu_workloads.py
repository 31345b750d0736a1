"""Every answer of the benchmark workloads at their full sizes against the
oracle (the reference's CPU path, Graph::bfs K/src/host/graph.cpp:83-97,
restated in oracle/fc_oracle.c), each on a CSR the oracle builds itself from
the same generator, so the device ingest is checked at full size as well.

* grid 4096 x 4096 (5% of edges deleted, seed 5; 0.01% n shortcuts, seed 6),
  256 pairs at Manhattan distance >= 2,000 (seed 7): every pair;
* 512 R-MAT graphs of scale 12-20 (seeds 100-611), 8 pairs each: every one
  of the 4,096 queries;
* R-MAT scale 24 (seed 3, ids permuted), 1,024 pairs (seed 4): every pair
  against the oracle's bidirectional search, a sample against Graph::bfs;
* the learned schedule's held-out sets, R-MAT scale 24 (seed 9) with 4,096
  pairs and the grid with 4,096 pairs (seed 17): every R-MAT answer against
  the bidirectional search, samples against Graph::bfs.

The bidirectional search (oracle_stcon_bidir_batch) is pinned to the
Graph::bfs restatement by tests/test_oracle.py; it is used where one full BFS
per query would take many minutes on the host (R-MAT 24 at ~6 queries/s on
16 cores).
"""
import os

import numpy as np
import pytest

from fastcon import graphs

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 4


def _csr_equal(G, rp, col):
    grp, gcol = G.csr()
    return len(grp) == len(rp) and (grp == rp).all() and len(gcol) == len(col) and (gcol == col).all()


def _schedules(fc):
    from fastcon import learn
    out = [fc.SCHED_HEURISTIC]
    if os.path.exists(learn.WEIGHTS_PATH):
        learn.load_default_weights()
        out.append(fc.SCHED_LEARNED)
    return out


def test_c3_grid_every_pair(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    w = h = 4096
    n = w * h
    k = graphs.grid_shortcut_count(n)
    G = fc.Graph.grid(w, h, p_del=0.05, del_seed=5, shortcuts=k, sc_seed=6)
    u, v = graphs.grid_edges(w, h, 0.05, 5, k, 6)
    rp, col = oracle_mod.build_csr(n, u, v, nthreads=NT)
    del u, v
    assert _csr_equal(G, rp, col)
    s, t = graphs.grid_pairs(w, h, 256, 7, 2000)
    want_c, want_h, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=NT)
    for sch in _schedules(fc) + [fc.SCHED_PLAIN]:
        conn, hops = fc.stcon_batch(G, s, t, opts=fc.make_opts(sched=sch,
                                                                engine=fc.ENGINE_BATCHED))
        assert (hops == want_h).all() and (conn == want_c).all(), sch
    G.free()


def test_c4_batched512_every_query(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    scales = graphs.batched_scales(512, 100)
    Gs, ss, ts, gi = [], [], [], []
    want_c, want_h = [], []
    for k, sc in enumerate(scales):
        seed = 100 + k
        G = fc.Graph.rmat(sc, 8 << sc, seed=seed, perm_seed=seed)
        u, v = oracle_mod.gen_rmat(sc, 8 << sc, seed=seed, perm_seed=seed, nthreads=NT)
        rp, col = oracle_mod.build_csr(1 << sc, u, v, nthreads=NT)
        assert _csr_equal(G, rp, col), k
        s, t = graphs.pairs_with_degree(np.diff(rp), 8, seed=seed)
        c, hh, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=NT)
        Gs.append(G)
        ss.append(s)
        ts.append(t)
        gi.append(np.full(8, k, np.int32))
        want_c.append(c)
        want_h.append(hh)
    s, t, gi = np.concatenate(ss), np.concatenate(ts), np.concatenate(gi)
    want_c, want_h = np.concatenate(want_c), np.concatenate(want_h)
    assert len(s) == 4096
    for sch in _schedules(fc):
        o = fc.make_opts(sched=sch, engine=fc.ENGINE_BATCHED, use_graph=1)
        conn, hops = fc.stcon_batch(Gs, s, t, graph_idx=gi, opts=o)
        assert (hops == want_h).all() and (conn == want_c).all(), sch
    for G in Gs:
        G.free()


def _rmat24(fc, oracle_mod, seed):
    G = fc.Graph.rmat(24, 8 << 24, seed=seed, perm_seed=seed)
    u, v = oracle_mod.gen_rmat(24, 8 << 24, seed=seed, perm_seed=seed, nthreads=NT)
    rp, col = oracle_mod.build_csr(1 << 24, u, v, nthreads=NT)
    del u, v
    assert _csr_equal(G, rp, col)
    return G, rp, col


def _check_rmat(fc, oracle_mod, G, rp, col, s, t, sample):
    want_c, want_h, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=NT, bidir=True)
    idx = np.arange(0, len(s), max(1, len(s) // sample))
    full_c, full_h, _ = oracle_mod.stcon_batch(rp, col, s[idx], t[idx], nthreads=NT)
    assert (full_h == want_h[idx]).all() and (full_c == want_c[idx]).all()
    for sch in _schedules(fc) + [fc.SCHED_PLAIN]:
        o = fc.make_opts(sched=sch, engine=fc.ENGINE_BATCHED, use_graph=1)
        conn, hops = fc.stcon_batch(G, s, t, opts=o)
        assert (hops == want_h).all() and (conn == want_c).all(), sch


def test_c2_rmat24_every_pair(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    G, rp, col = _rmat24(fc, oracle_mod, 3)
    s, t = graphs.pairs_with_degree(np.diff(rp), 1024, seed=4)
    _check_rmat(fc, oracle_mod, G, rp, col, s, t, sample=64)
    G.free()


def test_c5_learned_heldout_rmat24_every_pair(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    G, rp, col = _rmat24(fc, oracle_mod, 9)
    s, t = graphs.pairs_with_degree(np.diff(rp), 4096, seed=9)
    _check_rmat(fc, oracle_mod, G, rp, col, s, t, sample=48)
    G.free()


def test_c5_learned_heldout_grid(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    w = h = 4096
    n = w * h
    k = graphs.grid_shortcut_count(n)
    G = fc.Graph.grid(w, h, p_del=0.05, del_seed=5, shortcuts=k, sc_seed=6)
    u, v = graphs.grid_edges(w, h, 0.05, 5, k, 6)
    rp, col = oracle_mod.build_csr(n, u, v, nthreads=NT)
    del u, v
    s, t = graphs.grid_pairs(w, h, 4096, 17, 2000)
    idx = np.arange(0, 4096, 16)  # 256 pairs: one full grid BFS each on the host
    want_c, want_h, _ = oracle_mod.stcon_batch(rp, col, s[idx], t[idx], nthreads=NT)
    res = {}
    for sch in _schedules(fc):
        o = fc.make_opts(sched=sch, engine=fc.ENGINE_BATCHED, use_graph=1)
        conn, hops = fc.stcon_batch(G, s, t, opts=o)
        assert (hops[idx] == want_h).all() and (conn[idx] == want_c).all(), sch
        res[sch] = hops
    # every schedule gives the same 4,096 answers
    vals = list(res.values())
    assert all((x == vals[0]).all() for x in vals)
    G.free()
