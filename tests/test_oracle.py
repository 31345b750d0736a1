"""The CPU oracle pinned against the reference's own outputs (CPU only).

Pins: the reference's Graph::bfs (BFS-4K/src/host/graph.cpp:83-97) outputs
committed under tests/golden/ by make_golden.py, and the reference's logged
ST-CON run st_stats_20200418_140644 (100 rows, DEPTH = ceil(d/2)).
"""
import hashlib
import os
import tempfile

import numpy as np
import pytest
from conftest import known_answer_graph

from fastcon import graphs


def sha_levels(lev):
    return hashlib.sha256(np.ascontiguousarray(lev, dtype="<i4").tobytes()).hexdigest()


def sha_csr(rp, col):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(rp, dtype="<i4").tobytes())
    h.update(np.ascontiguousarray(col, dtype="<i4").tobytes())
    return h.hexdigest()


def test_tiny_graphs_match_reference_levels(oracle_mod, tiny_golden):
    for g in tiny_golden:
        es = np.array(g["edges"], dtype=np.int32).reshape(-1, 2)
        rp, col = oracle_mod.build_csr(g["nv"], es[:, 0], es[:, 1])
        assert rp.tolist() == g["row_ptr"], g["name"]
        assert col.tolist() == g["col"], g["name"]
        for i, s in enumerate(g["sources"]):
            lev, _ = oracle_mod.bfs_levels(rp, col, s)
            assert lev.tolist() == g["levels"][i], (g["name"], s)


def test_er_workload_matches_reference(oracle_mod, er_golden):
    gi = er_golden["graph"]
    u, v = graphs.er_edges(gi["n"], gi["m"], seed=gi["seed"])
    rp, col = oracle_mod.build_csr(gi["n"], u, v)
    assert len(col) == gi["directed_entries"]
    assert sha_csr(rp, col) == gi["csr_sha256"]
    s, t = graphs.uniform_pairs(gi["n"], 64, seed=er_golden["pairs_seed"])
    assert s.tolist() == er_golden["s"] and t.tolist() == er_golden["t"]
    for i in range(len(s)):
        lev, _ = oracle_mod.bfs_levels(rp, col, s[i])
        assert sha_levels(lev) == er_golden["levels_sha256"][i]
        assert lev[t[i]] == er_golden["hops"][i]
    conn, hops, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=4)
    assert hops.tolist() == er_golden["hops"]
    assert conn.tolist() == [int(h >= 0) for h in er_golden["hops"]]


def test_known_answer_depths(oracle_mod, ka):
    nv, u, v = known_answer_graph()
    rp, col = oracle_mod.build_csr(nv, u, v)
    assert len(col) == ka["graph"]["directed_entries"] == 1831864
    assert sha_csr(rp, col) == ka["graph"]["csr_sha256"]
    red = np.array([r["red"] for r in ka["rows"]], np.int32)
    blue = np.array([r["blue"] for r in ka["rows"]], np.int32)
    conn, hops, _ = oracle_mod.stcon_batch(rp, col, red, blue, nthreads=4)
    assert conn.all()
    # the reference's DEPTH is the number of two-sided rounds: ceil(d/2)
    assert ((hops + 1) // 2).tolist() == [r["depth"] for r in ka["rows"]]
    assert hops.tolist() == ka["ref_bfs_hops"]
    for i in range(0, 100, 9):
        lev, _ = oracle_mod.bfs_levels(rp, col, red[i])
        assert sha_levels(lev) == ka["ref_bfs_levels_sha256"][i]


def test_bidirectional_baseline_agrees(oracle_mod):
    u, v = graphs.rmat_edges(12, 8 << 12, seed=11, perm_seed=12)
    rp, col = oracle_mod.build_csr(1 << 12, u, v)
    s, t = graphs.uniform_pairs(1 << 12, 300, seed=13)
    c1, h1, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=2)
    c2, h2, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=3, bidir=True)
    assert (c1 == c2).all() and (h1 == h2).all()
    assert (c1 == 0).any() and (c1 == 1).any()


def test_canonical_csr_matches_numpy(oracle_mod):
    rng = np.random.default_rng(5)
    for nv, n in [(1, 0), (5, 20), (100, 1000), (3000, 20000)]:
        u = rng.integers(0, nv, n).astype(np.int32)
        v = rng.integers(0, nv, n).astype(np.int32)
        rp, col = oracle_mod.build_csr(nv, u, v)
        rp2, col2 = graphs.csr_from_edges(nv, u, v)
        assert (rp == rp2).all() and (col == col2).all()


def test_oracle_rejects_bad_ids(oracle_mod):
    with pytest.raises(ValueError):
        oracle_mod.build_csr(4, np.array([0, 5], np.int32), np.array([1, 1], np.int32))
    rp, col = oracle_mod.build_csr(3, np.array([0], np.int32), np.array([1], np.int32))
    with pytest.raises(ValueError):
        oracle_mod.stcon_batch(rp, col, np.array([0], np.int32), np.array([3], np.int32))


@pytest.mark.skipif(not __import__("oracle").ref_available(), reason="reference BFS not built here")
def test_oracle_matches_compiled_reference_directly(oracle_mod):
    for seed, scale in [(21, 10), (22, 13)]:
        u, v = graphs.rmat_edges(scale, 6 << scale, seed=seed, perm_seed=seed + 1)
        rp, col = oracle_mod.build_csr(1 << scale, u, v)
        srcs = graphs.uniform_pairs(1 << scale, 16, seed=seed + 2)[0]
        ref, _ = oracle_mod.ref_bfs_levels(rp, col, srcs)
        for i, s in enumerate(srcs):
            lev, _ = oracle_mod.bfs_levels(rp, col, s)
            assert (lev == ref[i]).all()


def _write(td, name, text):
    p = os.path.join(td, name)
    with open(p, "w") as f:
        f.write(text)
    return p


def test_edgelist_reader_formats(oracle_mod):
    with tempfile.TemporaryDirectory() as td:
        snap = _write(td, "g.txt", "# Undirected graph: test\n# Nodes: 6 Edges: 4\n"
                                   "# FromNodeId\tToNodeId\n0\t1\n1\t2\n5\t3\n3\t4\n")
        nv, s, d, fd = oracle_mod.read_edgelist(snap)
        assert nv == 6 and s.tolist() == [0, 1, 5, 3] and d.tolist() == [1, 2, 3, 4] and fd == 0
        nv, s, d, _ = oracle_mod.read_edgelist(snap, relabel=True)
        assert nv == 6 and s.tolist() == [0, 1, 3, 4] and d.tolist() == [1, 2, 4, 5]
        mm = _write(td, "g.mtx", "%%MatrixMarket matrix coordinate pattern symmetric\n% c\n"
                                 "4 4 3\n2 1\n3 2\n4 1\n")
        nv, s, d, fd = oracle_mod.read_edgelist(mm)
        assert nv == 4 and s.tolist() == [1, 2, 3] and d.tolist() == [0, 1, 0] and fd == 0
        d9 = _write(td, "g.gr", "c test\np sp 3 2\na 1 2 7\na 2 3 9\n")
        nv, s, d, _ = oracle_mod.read_edgelist(d9)
        assert nv == 3 and s.tolist() == [0, 1] and d.tolist() == [1, 2]
        d10 = _write(td, "g.graph", "% metis\n3 2\n2\n1 3\n2\n")
        nv, s, d, fd = oracle_mod.read_edgelist(d10)
        assert nv == 3 and s.tolist() == [0, 1, 1, 2] and d.tolist() == [1, 0, 2, 1] and fd == 0
        bad = _write(td, "bad.txt", "hello world\n")
        with pytest.raises(ValueError):
            oracle_mod.read_edgelist(bad)


def _tree_case(oracle_mod):
    rng = np.random.default_rng(41)
    nv = 400
    u = rng.integers(0, nv, 1500).astype(np.int32)
    v = rng.integers(0, nv, 1500).astype(np.int32)
    rp, col = oracle_mod.build_csr(nv, u, v)
    lev, _ = oracle_mod.bfs_levels(rp, col, 3)
    return rp, col, lev


def test_parents_and_validation_restatement(oracle_mod):
    """The tree rule (smallest-id parent one level closer) and the Graph500
    validation counters; mistakes are planted in host arrays."""
    rp, col, lev = _tree_case(oracle_mod)
    par = oracle_mod.bfs_parents(rp, col, lev, 3)
    nv = len(rp) - 1
    reached = lev >= 0
    assert par[3] == 3 and (par[~reached] == -1).all()
    for x in np.flatnonzero(reached & (lev > 0)):
        nb = col[rp[x]:rp[x + 1]]
        assert par[x] == nb[lev[nb] == lev[x] - 1].min()
    e = oracle_mod.validate_bfs(rp, col, rp, col, par, 3)
    assert e[:6] == [0] * 6 and e[6] == int(reached.sum())
    # planted mistakes, one rule each
    bad = par.copy(); bad[3] = 7
    assert oracle_mod.validate_bfs(rp, col, rp, col, bad, 3)[0] == 1
    x = int(np.flatnonzero(reached & (lev > 1))[0])
    bad = par.copy(); bad[x] = x
    assert oracle_mod.validate_bfs(rp, col, rp, col, bad, 3)[1] == 1
    nonnb = int(np.setdiff1d(np.flatnonzero(reached), np.append(col[rp[x]:rp[x + 1]], x))[0])
    bad = par.copy(); bad[x] = nonnb
    assert oracle_mod.validate_bfs(rp, col, rp, col, bad, 3)[2] >= 1
    y = int(par[x])
    bad = par.copy(); bad[y] = x  # a two-cycle x <-> y cut off from the root
    e = oracle_mod.validate_bfs(rp, col, rp, col, bad, 3)
    assert e[3] >= 2
    unreached = np.flatnonzero(~reached)
    if len(unreached):
        bad = par.copy(); bad[x] = -1  # x left out of the tree: its edges leave it
        e = oracle_mod.validate_bfs(rp, col, rp, col, bad, 3)
        assert e[4] >= 1
    assert nv == len(par)
