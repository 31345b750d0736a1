"""GPU parity: the CUDA path (through the C ABI) against the oracle and the
reference's golden outputs.  All answers are integers and must match exactly.
"""
import hashlib

import numpy as np
import pytest
from conftest import known_answer_graph

from fastcon import graphs

pytestmark = pytest.mark.gpu

ENGINES_SINGLE = ["hostloop", "persistent", "batched"]
ENGINES_BATCH = ["batched", "persistent", "hostloop"]
SCHEDS = ["plain", "heuristic", "learned"]


def sha_levels(lev):
    return hashlib.sha256(np.ascontiguousarray(lev, dtype="<i4").tobytes()).hexdigest()


def sha_csr(rp, col):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(rp, dtype="<i4").tobytes())
    h.update(np.ascontiguousarray(col, dtype="<i4").tobytes())
    return h.hexdigest()


def opts(fc, engine="persistent", sched="heuristic"):
    e = {"auto": fc.ENGINE_AUTO, "hostloop": fc.ENGINE_HOSTLOOP,
         "persistent": fc.ENGINE_PERSISTENT, "batched": fc.ENGINE_BATCHED}[engine]
    s = {"plain": fc.SCHED_PLAIN, "heuristic": fc.SCHED_HEURISTIC,
         "learned": fc.SCHED_LEARNED}[sched]
    return fc.make_opts(sched=s, engine=e)


# --------------------------------------------------------------------------
# tiny edge-case graphs: full level arrays from the reference
# --------------------------------------------------------------------------
def test_tiny_graphs_bfs_levels(fastcon_lib, tiny_golden):
    fc = fastcon_lib
    for g in tiny_golden:
        es = np.array(g["edges"], dtype=np.int32).reshape(-1, 2)
        G = fc.Graph.from_edges(es[:, 0], es[:, 1], g["nv"])
        rp, col = G.csr()
        assert rp.tolist() == g["row_ptr"] and col.tolist() == g["col"], g["name"]
        G2 = fc.Graph.from_csr(np.array(g["row_ptr"]), np.array(g["col"]))
        for eng in ENGINES_SINGLE:
            for sch in ("plain", "heuristic"):
                o = opts(fc, eng, sch)
                for i, s in enumerate(g["sources"]):
                    assert G.bfs_levels(s, o).tolist() == g["levels"][i], (g["name"], eng, sch, s)
                    assert G2.bfs_levels(s, o).tolist() == g["levels"][i]
        # the plain BFS engine, in the graph's numbering and degree-ordered
        for order in (fc.ORDER_GIVEN, fc.ORDER_DEGREE):
            o = fc.make_opts(sched=fc.SCHED_PLAIN, vertex_order=order)
            for i, s in enumerate(g["sources"]):
                assert G.bfs_levels(s, o).tolist() == g["levels"][i], (g["name"], order, s)


def test_tiny_graphs_stcon_all_pairs(fastcon_lib, tiny_golden):
    fc = fastcon_lib
    for g in tiny_golden:
        es = np.array(g["edges"], dtype=np.int32).reshape(-1, 2)
        G = fc.Graph.from_edges(es[:, 0], es[:, 1], g["nv"])
        srcs = g["sources"]
        ss, tt, want = [], [], []
        for i, s in enumerate(srcs):
            for t in range(g["nv"]):
                ss.append(s)
                tt.append(t)
                want.append(g["levels"][i][t])
        ss, tt, want = np.array(ss), np.array(tt), np.array(want)
        for eng in ENGINES_SINGLE:
            for sch in SCHEDS:
                o = opts(fc, eng, sch)
                for k in range(0, len(ss), max(1, len(ss) // 40)):
                    c, h = G.stcon(ss[k], tt[k], o)
                    assert (c, h) == (want[k] >= 0, want[k]), (g["name"], eng, sch, ss[k], tt[k])
        for eng in ENGINES_BATCH:
            for sch in SCHEDS:
                conn, hops = fc.stcon_batch(G, ss, tt, opts=opts(fc, eng, sch))
                assert (hops == want).all(), (g["name"], eng, sch)
                assert (conn == (want >= 0)).all()


# --------------------------------------------------------------------------
# ER workload: 65,536 vertices, 524,288 edges (seed 1), 64 pairs (seed 2)
# --------------------------------------------------------------------------
@pytest.fixture(scope="module")
def er_graph(fastcon_lib, er_golden):
    gi = er_golden["graph"]
    u, v = graphs.er_edges(gi["n"], gi["m"], seed=gi["seed"])
    return fastcon_lib.Graph.from_edges(u, v, gi["n"])


def test_er_device_ingest_is_canonical(er_graph, er_golden):
    rp, col = er_graph.csr()
    assert er_graph.ne == er_golden["graph"]["directed_entries"]
    assert sha_csr(rp, col) == er_golden["graph"]["csr_sha256"]
    assert rp.ctypes.data % 4 == 0


@pytest.mark.parametrize("engine,sched", [("hostloop", "plain"), ("persistent", "plain"),
                                          ("persistent", "heuristic"), ("hostloop", "heuristic"),
                                          ("batched", "plain"), ("batched", "heuristic"),
                                          ("auto", "plain")])
def test_er_bfs_levels_match_reference(fastcon_lib, er_graph, er_golden, engine, sched):
    o = opts(fastcon_lib, engine, sched)
    if engine == "auto":  # the plain BFS engine, degree-ordered copy
        o = fastcon_lib.make_opts(sched=fastcon_lib.SCHED_PLAIN,
                                  vertex_order=fastcon_lib.ORDER_DEGREE)
    bu = 0
    for i, s in enumerate(er_golden["s"]):
        lev, st = er_graph.bfs_levels(s, o, stats=True)
        assert sha_levels(lev) == er_golden["levels_sha256"][i], (engine, sched, s)
        bu += st["bottom_up_steps"]
    if sched == "heuristic":
        assert bu > 0  # the direction switch was exercised


@pytest.mark.parametrize("engine", ENGINES_BATCH)
@pytest.mark.parametrize("sched", SCHEDS)
def test_er_stcon_matches_reference(fastcon_lib, er_graph, er_golden, engine, sched):
    s, t = np.array(er_golden["s"]), np.array(er_golden["t"])
    want = np.array(er_golden["hops"])
    conn, hops = fastcon_lib.stcon_batch(er_graph, s, t, opts=opts(fastcon_lib, engine, sched))
    assert (hops == want).all() and (conn == (want >= 0)).all()
    if engine != "batched":
        o = opts(fastcon_lib, engine, sched)
        for k in range(0, 64, 7):
            assert er_graph.stcon(s[k], t[k], o) == (want[k] >= 0, want[k])


def test_batched_graph_replay(fastcon_lib, er_graph, er_golden):
    """use_graph captures the batched launch once and replays it for the next
    batch of the same size; the replay reads the new queries."""
    fc = fastcon_lib
    s, t = np.array(er_golden["s"]), np.array(er_golden["t"])
    want = np.array(er_golden["hops"])
    o = fc.make_opts(sched=fc.SCHED_HEURISTIC, engine=fc.ENGINE_BATCHED, use_graph=1)
    conn, hops, st = fc.stcon_batch(er_graph, s, t, opts=o, stats=True)
    assert (hops == want).all() and st["graph"] in (1, 2)
    # reversed pairs: same distances on an undirected graph, replayed graph
    conn, hops, st = fc.stcon_batch(er_graph, t, s, opts=o, stats=True)
    assert (hops == want).all() and st["graph"] == 1
    assert st["edges_inspected"] > 0 and st["kernel_ms"][0] > 0
    # another size captures again; without use_graph nothing is captured
    conn, hops, st = fc.stcon_batch(er_graph, s[:40], t[:40], opts=o, stats=True)
    assert (hops == want[:40]).all() and st["graph"] == 2
    o0 = fc.make_opts(sched=fc.SCHED_HEURISTIC, engine=fc.ENGINE_BATCHED)
    conn, hops, st = fc.stcon_batch(er_graph, s, t, opts=o0, stats=True)
    assert (hops == want).all() and st["graph"] == 0


@pytest.mark.parametrize("engine", ENGINES_BATCH)
def test_batch_into_caller_arrays_without_stats(fastcon_lib, er_graph, er_golden, engine):
    """Host-array batches without statistics wait once for the answers and the
    engine's error words together; answers land in the caller's arrays."""
    import torch
    fc = fastcon_lib
    s, t = np.array(er_golden["s"]), np.array(er_golden["t"])
    want = np.array(er_golden["hops"])
    hc = torch.full((len(s) + 3,), -7, dtype=torch.int32).pin_memory().numpy()
    hh = torch.full((len(s) + 3,), -7, dtype=torch.int32).pin_memory().numpy()
    o = opts(fc, engine, "heuristic")
    for _ in range(2):  # the second call reuses the staging (and a captured graph)
        conn, hops = fc.stcon_batch(er_graph, s, t, opts=o, out=(hc, hh))
        assert conn is hc and hops is hh
        assert (hh[:len(s)] == want).all() and (hc[:len(s)] == (want >= 0)).all()
        assert (hh[len(s):] == -7).all()  # nothing written past the batch
    with pytest.raises(ValueError):
        fc.stcon_batch(er_graph, s, t, opts=o, out=(hc[:10], hh))


# --------------------------------------------------------------------------
# the reference's known-answer run (Graph500 R-MAT scale 16)
# --------------------------------------------------------------------------
def test_known_answer_run(fastcon_lib, ka):
    fc = fastcon_lib
    nv, u, v = known_answer_graph()
    G = fc.Graph.from_edges(u, v, nv)
    rp, col = G.csr()
    assert sha_csr(rp, col) == ka["graph"]["csr_sha256"]
    red = np.array([r["red"] for r in ka["rows"]])
    blue = np.array([r["blue"] for r in ka["rows"]])
    depth = [r["depth"] for r in ka["rows"]]
    for k in range(0, 100, 5):
        assert G.stcon_depth(red[k], blue[k]) == depth[k]
    for eng in ENGINES_BATCH:
        for sch in SCHEDS:
            conn, hops = fc.stcon_batch(G, red, blue, opts=opts(fc, eng, sch))
            assert conn.all()
            assert hops.tolist() == ka["ref_bfs_hops"]
            assert ((hops + 1) // 2).tolist() == depth
    for k in range(0, 100, 11):
        assert sha_levels(G.bfs_levels(red[k])) == ka["ref_bfs_levels_sha256"][k]


# --------------------------------------------------------------------------
# device ingest and generators against the CPU canonical CSR
# --------------------------------------------------------------------------
def test_ingest_matches_oracle_csr(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    rng = np.random.default_rng(17)
    cases = []
    for nv, n in [(1, 0), (2, 1), (7, 40), (300, 5000), (5000, 60000)]:
        cases.append((nv, rng.integers(0, nv, n), rng.integers(0, nv, n)))
    # rows in every sort class: a 20,000-leaf star (large), 3,000 (medium),
    # with duplicates and loops mixed in
    hub = np.concatenate([np.zeros(20000), np.full(3000, 1), rng.integers(0, 30000, 3000)])
    leaf = np.concatenate([rng.permutation(np.arange(2, 20002)), rng.integers(2, 30000, 3000),
                           rng.integers(0, 30000, 3000)])
    cases.append((30000, hub, leaf))
    flagsets = [(0, oracle_mod.CANONICAL),
                (fc.INGEST_DIRECTED, oracle_mod.DROP_LOOPS | oracle_mod.DEDUPE),
                (fc.INGEST_KEEP_LOOPS, oracle_mod.SYMMETRIZE | oracle_mod.DEDUPE),
                (fc.INGEST_KEEP_DUPS, oracle_mod.SYMMETRIZE | oracle_mod.DROP_LOOPS)]
    for nv, u, v in cases:
        u = u.astype(np.int32)
        v = v.astype(np.int32)
        for ff, of in flagsets:
            G = fc.Graph.from_edges(u, v, nv, flags=ff)
            rp, col = G.csr()
            rp2, col2 = oracle_mod.build_csr(nv, u, v, flags=of)
            if ff == fc.INGEST_KEEP_DUPS:
                # duplicates kept: rows must be sorted and equal as multisets
                assert (rp == rp2).all()
                for r in range(0, nv, max(1, nv // 200)):
                    a = col[rp[r]:rp[r + 1]]
                    assert (np.diff(a) >= 0).all()
                    assert (a == np.sort(col2[rp2[r]:rp2[r + 1]])).all()
            else:
                assert (rp == rp2).all() and (col == col2).all(), (nv, ff)


def test_ingest_rejects_bad_ids(fastcon_lib):
    fc = fastcon_lib
    with pytest.raises(fc.FastconError) as e:
        fc.Graph.from_edges(np.array([0, 9]), np.array([1, 1]), 4)
    assert e.value.code == fc.ERR_INVALID


def test_rmat_generator_matches_numpy(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    for scale, ne, seed, perm in [(10, 9000, 3, 4), (12, 8 << 12, 7, -1)]:
        G = fc.Graph.rmat(scale, ne, seed=seed, perm_seed=perm)
        u, v = graphs.rmat_edges(scale, ne, seed=seed, perm_seed=None if perm < 0 else perm)
        rp2, col2 = oracle_mod.build_csr(1 << scale, u, v)
        rp, col = G.csr()
        assert (rp == rp2).all() and (col == col2).all()


def test_grid_generator_matches_numpy(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    w, h, k = 64, 48, 7
    G = fc.Graph.grid(w, h, p_del=0.05, del_seed=5, shortcuts=k, sc_seed=6)
    u, v = graphs.grid_edges(w, h, 0.05, 5, k, 6)
    rp2, col2 = oracle_mod.build_csr(w * h, u, v)
    rp, col = G.csr()
    assert (rp == rp2).all() and (col == col2).all()


# --------------------------------------------------------------------------
# directed graphs: the t side walks the reverse CSR
# --------------------------------------------------------------------------
def test_directed_graphs(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    rng = np.random.default_rng(3)
    nv, n = 2000, 5000
    u = rng.integers(0, nv, n).astype(np.int32)
    v = rng.integers(0, nv, n).astype(np.int32)
    G = fc.Graph.from_edges(u, v, nv, flags=fc.INGEST_DIRECTED)
    assert G.directed
    rp, col = oracle_mod.build_csr(nv, u, v, flags=oracle_mod.DROP_LOOPS | oracle_mod.DEDUPE)
    s, t = graphs.uniform_pairs(nv, 200, seed=9)
    conn, hops, _ = oracle_mod.stcon_batch(rp, col, s, t)
    for eng in ENGINES_BATCH:
        for sch in ("plain", "heuristic"):
            c2, h2 = fc.stcon_batch(G, s, t, opts=opts(fc, eng, sch))
            assert (h2 == hops).all() and (c2 == conn).all(), (eng, sch)
    for k in range(0, 200, 20):
        lev, _ = oracle_mod.bfs_levels(rp, col, s[k])
        assert (G.bfs_levels(s[k], opts(fc, "persistent", "heuristic")) == lev).all()


# --------------------------------------------------------------------------
# edge cases
# --------------------------------------------------------------------------
def test_edge_cases(fastcon_lib):
    fc = fastcon_lib
    G = fc.Graph.from_edges(np.array([0, 1, 3]), np.array([1, 2, 4]), 6)
    assert G.stcon(2, 2) == (True, 0)
    assert G.stcon(5, 5) == (True, 0)  # isolated vertex, s == t
    assert G.stcon(0, 5) == (False, -1)  # isolated target
    assert G.stcon(5, 0) == (False, -1)  # isolated source
    assert G.stcon(0, 4) == (False, -1)
    assert G.stcon(0, 2) == (True, 2)
    assert G.stcon_depth(0, 2) == 1 and G.stcon_depth(0, 4) == -1 and G.stcon_depth(1, 1) == 0
    assert G.bfs_levels(5).tolist() == [-1, -1, -1, -1, -1, 0]
    for bad in [(-1, 0), (0, 6), (6, 6)]:
        with pytest.raises(fc.FastconError) as e:
            G.stcon(*bad)
        assert e.value.code == fc.ERR_INVALID
    with pytest.raises(fc.FastconError):
        G.bfs_levels(6)
    with pytest.raises(fc.FastconError):
        fc.stcon_batch(G, np.array([0, 1]), np.array([1, 7]))
    conn, hops = fc.stcon_batch(G, np.zeros(0), np.zeros(0))
    assert len(conn) == 0 and len(hops) == 0
    # empty graph (no edges)
    E = fc.Graph.from_edges(np.zeros(0), np.zeros(0), 3)
    assert E.ne == 0 and E.stcon(0, 2) == (False, -1) and E.bfs_levels(1).tolist() == [-1, 0, -1]


def test_multi_graph_batch(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    Gs, csrs = [], []
    for k, scale in enumerate([8, 11, 13, 9]):
        u, v = graphs.rmat_edges(scale, 16 << scale, seed=100 + k, perm_seed=200 + k)
        Gs.append(fc.Graph.from_edges(u, v, 1 << scale))
        csrs.append(oracle_mod.build_csr(1 << scale, u, v))
    rng = np.random.default_rng(1)
    gi = rng.integers(0, 4, 800).astype(np.int32)
    s = np.array([rng.integers(0, Gs[g].nv) for g in gi], np.int32)
    t = np.array([rng.integers(0, Gs[g].nv) for g in gi], np.int32)
    want = np.zeros(800, np.int32)
    for g in range(4):
        m = gi == g
        _, h, _ = oracle_mod.stcon_batch(*csrs[g], s[m], t[m], nthreads=4)
        want[m] = h
    for eng in ENGINES_BATCH:
        conn, hops = fc.stcon_batch(Gs, s, t, graph_idx=gi, opts=opts(fc, eng, "heuristic"))
        assert (hops == want).all(), eng


def test_batched_many_queries_rmat(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    scale = 16
    u, v = graphs.rmat_edges(scale, 8 << scale, seed=31, perm_seed=32)
    G = fc.Graph.from_edges(u, v, 1 << scale)
    rp, col = G.csr()
    s, t = graphs.pairs_with_degree(np.diff(rp), 3000, seed=33)
    _, want, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=16)
    for eng in ("batched", "persistent"):
        for sch in SCHEDS:
            conn, hops, st = fc.stcon_batch(G, s, t, opts=opts(fc, eng, sch), stats=True)
            assert (hops == want).all(), (eng, sch)
            assert st["edges_inspected"] > 0


# --------------------------------------------------------------------------
# every expansion variant, forced, on every engine (answers never change)
# --------------------------------------------------------------------------
@pytest.mark.parametrize("variant", [1, 2, 3])
def test_forced_variants(fastcon_lib, oracle_mod, variant):
    fc = fastcon_lib
    cases = []
    u, v = graphs.rmat_edges(14, 8 << 14, seed=51, perm_seed=52)
    cases.append((1 << 14, u, v))
    u, v = graphs.grid_edges(90, 70, 0.05, 5, 4, 6)
    cases.append((90 * 70, u, v))
    nv = 40000  # a 20,000-leaf hub next to random edges
    rng = np.random.default_rng(4)
    u = np.concatenate([np.zeros(20000), rng.integers(0, nv, 30000)]).astype(np.int32)
    v = np.concatenate([np.arange(1, 20001), rng.integers(0, nv, 30000)]).astype(np.int32)
    cases.append((nv, u, v))
    for nv, u, v in cases:
        G = fc.Graph.from_edges(u, v, nv)
        rp, col = oracle_mod.build_csr(nv, u, v)
        s, t = graphs.uniform_pairs(nv, 150, seed=53)
        _, want, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=4)
        for eng in ENGINES_BATCH:
            for work_k in (0, -1):
                o = fc.make_opts(sched=fc.SCHED_HEURISTIC, engine=opts(fc, eng).engine,
                                 cta_work_k=work_k, variant=variant)
                conn, hops = fc.stcon_batch(G, s, t, opts=o)
                assert (hops == want).all(), (nv, eng, work_k)
        for eng in ENGINES_SINGLE:
            o = fc.make_opts(sched=fc.SCHED_HEURISTIC, engine=opts(fc, eng).engine, variant=variant)
            for k in range(0, 150, 29):
                assert G.stcon(s[k], t[k], o) == (want[k] >= 0, want[k]), (nv, eng)
            lev, _ = oracle_mod.bfs_levels(rp, col, s[0])
            assert (G.bfs_levels(s[0], o) == lev).all(), (nv, eng)


# --------------------------------------------------------------------------
# deep graphs: both sides grow past 127 levels (status bytes clamp the level)
# --------------------------------------------------------------------------
def test_deep_levels_path_and_grid(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    n = 700
    P = fc.Graph.from_edges(np.arange(n - 1), np.arange(1, n), n)
    for eng in ENGINES_SINGLE:
        for sch in SCHEDS:
            o = opts(fc, eng, sch)
            assert P.stcon(0, n - 1, o) == (True, n - 1), (eng, sch)
            assert P.stcon(350, 3, o) == (True, 347), (eng, sch)
            assert P.bfs_levels(0, o).tolist() == list(range(n)), (eng, sch)
    w = h = 220
    u, v = graphs.grid_edges(w, h, 0.05, 5, 3, 6)
    G = fc.Graph.from_edges(u, v, w * h)
    rp, col = oracle_mod.build_csr(w * h, u, v)
    s, t = graphs.grid_pairs(w, h, 60, 7, 200)
    _, want, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=4)
    assert want.max() > 260
    for eng in ENGINES_BATCH:
        for sch in SCHEDS:
            conn, hops = fc.stcon_batch(G, s, t, opts=opts(fc, eng, sch))
            assert (hops == want).all(), (eng, sch)
    for k in range(0, 60, 13):
        for eng in ENGINES_SINGLE:
            assert G.stcon(s[k], t[k], opts(fc, eng, "heuristic")) == (want[k] >= 0, want[k])


# --------------------------------------------------------------------------
# the work-sharing engine with every step shared: tiles, row jobs for hub
# rows longer than 8,192 entries, shared status resets
# --------------------------------------------------------------------------
def test_shared_steps_and_row_jobs(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    rng = np.random.default_rng(8)
    nv = 70000
    # two hubs of 30,000 and 12,000 leaves, a long path, random extra edges
    u = np.concatenate([np.zeros(30000), np.full(12000, 1), np.arange(50000, 69999),
                        rng.integers(0, nv, 20000)]).astype(np.int32)
    v = np.concatenate([np.arange(2, 30002), np.arange(30002, 42002), np.arange(50001, 70000),
                        rng.integers(0, nv, 20000)]).astype(np.int32)
    G = fc.Graph.from_edges(u, v, nv)
    rp, col = oracle_mod.build_csr(nv, u, v)
    s, t = graphs.uniform_pairs(nv, 300, seed=21)
    s[:4] = [0, 1, 50000, 0]
    t[:4] = [1, 69999, 2, 60000]
    _, want, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=4)
    for work_k in (-1, 1, 0):
        for sch in SCHEDS:
            o = fc.make_opts(sched={"plain": 0, "heuristic": 1, "learned": 2}[sch],
                             engine=fc.ENGINE_BATCHED, cta_work_k=work_k)
            conn, hops = fc.stcon_batch(G, s, t, opts=o)
            assert (hops == want).all(), (work_k, sch)
            for k in range(0, 300, 37):
                assert G.stcon(s[k], t[k], o) == (want[k] >= 0, want[k])
            for src in (0, 1, 50000, 7):
                lev, _ = oracle_mod.bfs_levels(rp, col, src)
                assert (G.bfs_levels(src, o) == lev).all(), (work_k, sch, src)
    # small tiles and the shortest row jobs, every variant
    for te, je in ((1024, 1024), (4096, 2048)):
        for var in (0, 1, 2, 3):
            o = fc.make_opts(sched=fc.SCHED_HEURISTIC, engine=fc.ENGINE_BATCHED, cta_work_k=-1,
                             tile_entries=te, job_entries=je, variant=var)
            conn, hops = fc.stcon_batch(G, s, t, opts=o)
            assert (hops == want).all(), (te, je, var)
            lev, _ = oracle_mod.bfs_levels(rp, col, 0)
            assert (G.bfs_levels(0, o) == lev).all(), (te, je, var)
    # hub rows (30,000 and 12,000 entries) as team row jobs of the host-loop
    # and grid engines, in every variant and schedule
    for eng in (fc.ENGINE_HOSTLOOP, fc.ENGINE_PERSISTENT):
        for sch in (fc.SCHED_PLAIN, fc.SCHED_HEURISTIC):
            for var in (0, 1, 2, 3):
                o = fc.make_opts(sched=sch, engine=eng, variant=var)
                for src in (0, 1, 2, 50000):
                    lev, _ = oracle_mod.bfs_levels(rp, col, src)
                    assert (G.bfs_levels(src, o) == lev).all(), (eng, sch, var, src)
                conn, hops = fc.stcon_batch(G, s[:60], t[:60], opts=o)
                assert (hops == want[:60]).all(), (eng, sch, var)


# --------------------------------------------------------------------------
# the first batch on a graph bigger than any before it: the workspaces are
# reallocated and initialised, and must be ready before the kernels run
# --------------------------------------------------------------------------
def test_first_call_after_workspace_growth(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    scale = 20
    u, v = graphs.rmat_edges(scale, 8 << scale, seed=81, perm_seed=82)
    G = fc.Graph.from_edges(u, v, 1 << scale)
    rp, col = G.csr()
    s, t = graphs.pairs_with_degree(np.diff(rp), 2000, seed=83)
    conn, hops = fc.stcon_batch(G, s, t, opts=opts(fc, "batched", "plain"))
    samp = np.arange(0, 2000, 7)
    _, want, _ = oracle_mod.stcon_batch(rp, col, s[samp], t[samp], nthreads=16)
    assert (hops[samp] == want).all()
    conn2, hops2 = fc.stcon_batch(G, s, t, opts=opts(fc, "batched", "heuristic"))
    assert (hops2 == hops).all()


# --------------------------------------------------------------------------
# autotuner: picks one of its candidate settings; answers stay exact
# --------------------------------------------------------------------------
def test_autotune_batch(fastcon_lib, oracle_mod):
    import torch
    fc = fastcon_lib
    u, v = graphs.rmat_edges(15, 8 << 15, seed=95, perm_seed=96)
    G = fc.Graph.from_edges(u, v, 1 << 15)
    rp, col = oracle_mod.build_csr(1 << 15, u, v)
    s, t = graphs.pairs_with_degree(np.diff(rp), 300, seed=97)
    _, want, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=4)
    ds = torch.from_numpy(s).cuda()
    dt = torch.from_numpy(t).cuda()
    o, ms = fc.autotune_batch(G, ds.data_ptr(), dt.data_ptr(), len(s), reps=1)
    assert ms > 0 and o.engine == fc.ENGINE_BATCHED
    assert o.ctas_per_sm in (2, 3, 4) and o.cta_work_k in (2, 4, 8)
    assert o.tile_entries in (4096, 8192, 16384)
    conn, hops = fc.stcon_batch(G, s, t, opts=o)
    assert (hops == want).all()


# --------------------------------------------------------------------------
# the statistics count adjacency entries actually read: a plain top-down BFS
# expands every reached vertex once, so it reads exactly their degree sum
# --------------------------------------------------------------------------
def test_entries_read_accounting(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    u, v = graphs.rmat_edges(15, 8 << 15, seed=111, perm_seed=112)
    G = fc.Graph.from_edges(u, v, 1 << 15)
    rp, col = oracle_mod.build_csr(1 << 15, u, v)
    deg = np.diff(rp)
    for src in (0, 77, 4096):
        lev, _ = oracle_mod.bfs_levels(rp, col, src)
        want = int(deg[lev >= 0].sum())
        for eng in ("hostloop", "persistent", "batched"):
            o = opts(fc, eng, "plain")
            got, st = G.bfs_levels(src, o, stats=True)
            assert (got == lev).all()
            assert st["edges_inspected"] == want, (eng, src, st["edges_inspected"], want)


# --------------------------------------------------------------------------
# the plain BFS engine (visited bitmap, degree-ordered copy): levels against
# the oracle on hub graphs, directed graphs, deep paths, grids, isolated
# vertices; statistics follow the algorithmic-byte rule
# --------------------------------------------------------------------------
def test_plain_bfs_engine(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    cases = []
    u, v = graphs.rmat_edges(16, 8 << 16, seed=81, perm_seed=82)
    cases.append(("rmat16", 1 << 16, u, v, 0))
    cases.append(("rmat15_directed", 1 << 15, *graphs.rmat_edges(15, 8 << 15, seed=83, perm_seed=84),
                  fc.INGEST_DIRECTED))
    nv = 90001  # a 60,000-leaf hub (row jobs), a path, random edges; nv not a multiple of 32
    rng = np.random.default_rng(85)
    u = np.concatenate([np.zeros(60000), np.arange(60001, 90000),
                        rng.integers(0, nv, 5000)]).astype(np.int32)
    v = np.concatenate([np.arange(1, 60001), np.arange(60002, 90001),
                        rng.integers(0, nv, 5000)]).astype(np.int32)
    cases.append(("hub_path", nv, u, v, 0))
    cases.append(("path700", 700, np.arange(699), np.arange(1, 700), 0))
    u, v = graphs.grid_edges(300, 200, 0.05, 5, 7, 6)
    cases.append(("grid300x200", 60000, u, v, 0))
    u = rng.integers(0, 50000, 40000).astype(np.int32)  # many isolated vertices
    v = rng.integers(0, 50000, 40000).astype(np.int32)
    cases.append(("sparse", 50003, u, v, 0))
    for name, nv, u, v, flags in cases:
        G = fc.Graph.from_edges(u, v, nv, flags=flags)
        rp, col = G.csr()
        deg = np.diff(rp)
        srcs = [int(np.argmax(deg)), 0, nv - 1, int(np.argsort(deg)[3 * nv // 4])]
        for order in (fc.ORDER_AUTO, fc.ORDER_GIVEN, fc.ORDER_DEGREE):
            o = fc.make_opts(sched=fc.SCHED_PLAIN, vertex_order=order)
            for src in srcs:
                want, _ = oracle_mod.bfs_levels(rp, col, src)
                lev, st = G.bfs_levels(src, o, stats=True)
                assert (lev == want).all(), (name, order, src)
                reached = int((want >= 0).sum())
                assert st["visited"] == reached and st["steps"] == int(want.max()) + 1
                assert st["edges_inspected"] == int(deg[want >= 0].sum()), (name, order, src)
                assert st["alg_bytes"] == 20 * reached - 8 + 8 * st["edges_inspected"]
        G.free()


# --------------------------------------------------------------------------
# s-t searches run on the degree-ordered copy of an undirected graph with
# hubs unless the caller keeps its numbering: every engine and order gives
# the oracle's answers, single queries and batches, on graphs with and
# without hubs (the copy is built only when there are hubs, or when asked)
# --------------------------------------------------------------------------
def test_stcon_vertex_order(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    cases = []
    u, v = graphs.rmat_edges(16, 8 << 16, seed=61, perm_seed=62)
    cases.append(("rmat16", 1 << 16, u, v))
    rng = np.random.default_rng(64)
    u = rng.integers(0, 30000, 90000).astype(np.int32)  # no vertex of degree 256
    v = rng.integers(0, 30000, 90000).astype(np.int32)
    cases.append(("er", 30001, u, v))
    for name, nv, u, v in cases:
        G = fc.Graph.from_edges(u, v, nv)
        rp, col = G.csr()
        deg = np.diff(rp)
        s, t = graphs.pairs_with_degree(deg, 1200, seed=63)
        s[1] = t[1] = int(np.argmax(deg))  # s == t on a hub
        isolated = np.where(deg == 0)[0]
        s[2] = int(isolated[0]) if len(isolated) else s[2]
        _, want, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=16)
        for order in (fc.ORDER_AUTO, fc.ORDER_GIVEN, fc.ORDER_DEGREE):
            for eng in (fc.ENGINE_AUTO, fc.ENGINE_BATCHED, fc.ENGINE_PERSISTENT):
                for sch in (fc.SCHED_PLAIN, fc.SCHED_HEURISTIC):
                    o = fc.make_opts(sched=sch, engine=eng, vertex_order=order)
                    conn, hops = fc.stcon_batch(G, s, t, opts=o)
                    assert (hops == want).all(), (name, order, eng, sch)
                    assert (conn == (want >= 0)).all()
                    for k in (0, 1, 2, 3, 500, 1199):
                        assert G.stcon(s[k], t[k], o) == (want[k] >= 0, want[k]), (name, k)
            # the batch's device form (the benchmark's call) with a replayed graph
            o = fc.make_opts(sched=fc.SCHED_LEARNED, engine=fc.ENGINE_BATCHED, use_graph=1,
                             vertex_order=order)
            for _ in range(2):
                conn, hops = fc.stcon_batch(G, s, t, opts=o)
                assert (hops == want).all(), (name, order, "graph replay")
        # the levels of a full BFS are indexed by the caller's ids whatever the order
        lev, _ = oracle_mod.bfs_levels(rp, col, int(s[0]))
        assert (G.bfs_levels(int(s[0])) == lev).all()
        G.free()


# --------------------------------------------------------------------------
# host-array batches from page-locked memory: the engine copies the queries
# in and the answers out with its kernels, inside the captured CUDA graph
# when one is used; new contents of the same arrays are read on replay
# --------------------------------------------------------------------------
def test_batch_page_locked_host_arrays(fastcon_lib, oracle_mod):
    import torch
    fc = fastcon_lib
    gs, csrs = [], []
    for k, sc in enumerate((12, 14)):
        u, v = graphs.rmat_edges(sc, 8 << sc, seed=90 + k, perm_seed=91 + k)
        G = fc.Graph.from_edges(u, v, 1 << sc)
        gs.append(G)
        csrs.append(G.csr())
    nq = 700
    rng = np.random.default_rng(92)

    def pinned(a):
        return torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).pin_memory().numpy()

    hs, ht, hg = pinned(np.zeros(nq)), pinned(np.zeros(nq)), pinned(np.zeros(nq))
    hc, hh = pinned(np.full(nq, -7)), pinned(np.full(nq, -7))
    for use_graph in (1, 0):
        for sch in (fc.SCHED_HEURISTIC, fc.SCHED_LEARNED):
            o = fc.make_opts(sched=sch, engine=fc.ENGINE_BATCHED, use_graph=use_graph)
            for rep in range(3):  # new queries in the same arrays each call
                hg[:] = rng.integers(0, 2, nq)
                for j in range(nq):
                    n = 1 << (12 if hg[j] == 0 else 14)
                    hs[j], ht[j] = rng.integers(0, n, 2)
                want = np.empty(nq, np.int32)
                for gi in (0, 1):
                    idx = np.where(hg == gi)[0]
                    rp, col = csrs[gi]
                    _, w, _ = oracle_mod.stcon_batch(rp, col, hs[idx].copy(), ht[idx].copy(),
                                                     nthreads=8)
                    want[idx] = w
                stats = rep == 2
                r = fc.stcon_batch(gs, hs, ht, graph_idx=hg, opts=o, out=(hc, hh), stats=stats)
                assert r[0] is hc and r[1] is hh
                assert (hh == want).all(), (use_graph, sch, rep)
                assert (hc == (want >= 0)).all()
                if stats:
                    assert r[2]["graph"] == (2 if use_graph else 0)  # captured with the copies
    # pageable arrays take the copies outside the engine: same answers
    o = fc.make_opts(sched=fc.SCHED_HEURISTIC, engine=fc.ENGINE_BATCHED, use_graph=1)
    c2, h2 = fc.stcon_batch(gs, np.array(hs), np.array(ht), graph_idx=np.array(hg), opts=o)
    assert (h2 == hh).all()
    for G in gs:
        G.free()


# --------------------------------------------------------------------------
# the spill pass: with small query-slot logs, queries whose claims could
# outgrow their slot are finished by the whole grid after the batch, on the
# degree-ordered copy and in the caller's numbering, with and without a
# captured graph
# --------------------------------------------------------------------------
def test_batch_spill_pass(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    u, v = graphs.rmat_edges(16, 8 << 16, seed=71, perm_seed=72)
    G = fc.Graph.from_edges(u, v, 1 << 16)
    rp, col = G.csr()
    s, t = graphs.pairs_with_degree(np.diff(rp), 600, seed=73)
    _, want, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=16)
    for order in (fc.ORDER_AUTO, fc.ORDER_GIVEN):
        for sch in (fc.SCHED_PLAIN, fc.SCHED_HEURISTIC):
            for ug in (0, 1):
                o = fc.make_opts(sched=sch, engine=fc.ENGINE_BATCHED, slot_log_cap=1024,
                                 vertex_order=order, use_graph=ug)
                conn, hops, st = fc.stcon_batch(G, s, t, opts=o, stats=True)
                assert (hops == want).all(), (order, sch, ug)
                assert (conn == (want >= 0)).all()
                assert st["escalated"] > 0, (order, sch, ug)  # the pass did run
    # the default (full-size logs) spills nothing
    conn, hops, st = fc.stcon_batch(G, s, t, opts=fc.make_opts(engine=fc.ENGINE_BATCHED), stats=True)
    assert (hops == want).all() and st["escalated"] == 0
    G.free()
