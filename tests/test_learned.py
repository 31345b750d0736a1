"""Learned schedule: the CUDA training kernels against a float64 CPU
restatement (gradient check), training convergence, trace/script hooks, and
exact answers under the learned schedule."""
import json
import os

import numpy as np
import pytest

from fastcon import graphs

pytestmark = pytest.mark.gpu


def unpack(w):
    w = np.asarray(w, np.float64)
    return (w[0:384].reshape(32, 12), w[384:416], w[416:1440].reshape(32, 32), w[1440:1472],
            w[1472:1696].reshape(7, 32), w[1696:1703])


def loss_grad_np(X, Y, w, SW=None):
    """Mean (weighted) softmax cross-entropy over labelled heads and its
    gradient, float64."""
    W1, b1, W2, b2, W3, b3 = unpack(w)
    X = np.asarray(X, np.float64)
    n = len(X)
    a1 = X @ W1.T + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0)
    z = h2 @ W3.T + b3
    dz = np.zeros_like(z)
    loss = 0.0
    for col, (lo, k) in enumerate(((0, 2), (2, 2), (4, 3))):
        zz = z[:, lo:lo + k]
        mx = zz.max(axis=1, keepdims=True)
        e = np.exp(zz - mx)
        p = e / e.sum(axis=1, keepdims=True)
        lab = Y[:, col]
        m = lab >= 0
        wgt = np.ones(n) if SW is None else np.asarray(SW, np.float64)[:, col]
        loss += (wgt[m] * (np.log(e.sum(axis=1))[m] + mx[m, 0] - zz[m, lab[m]])).sum()
        g = p.copy()
        g[m, lab[m]] -= 1.0
        g[~m] = 0.0
        dz[:, lo:lo + k] = g * wgt[:, None]
    dz /= n
    gW3 = dz.T @ h2
    gb3 = dz.sum(0)
    dh2 = dz @ W3
    da2 = dh2 * (a2 > 0)
    gW2 = da2.T @ h1
    gb2 = da2.sum(0)
    dh1 = da2 @ W2
    da1 = dh1 * (a1 > 0)
    gW1 = da1.T @ X
    gb1 = da1.sum(0)
    grad = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss / n, grad


def random_set(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.uniform(0, 1, size=(n, 12)).astype(np.float32)
    Y = np.stack([rng.integers(-1, 2, n), rng.integers(-1, 2, n), rng.integers(-1, 3, n)], 1)
    return X, Y.astype(np.int32)


def test_restatement_matches_finite_differences():
    from fastcon import learn
    X, Y = random_set(16, 1)
    w = learn.init_weights(3).astype(np.float64) * 0.7 + 0.01
    _, g = loss_grad_np(X, Y, w)
    rng = np.random.default_rng(2)
    for i in rng.choice(1703, 40, replace=False):
        e = np.zeros(1703)
        e[i] = 1e-6
        num = (loss_grad_np(X, Y, w + e)[0] - loss_grad_np(X, Y, w - e)[0]) / 2e-6
        assert abs(num - g[i]) <= 1e-6 + 1e-4 * abs(g[i]), i


def test_gpu_gradient_matches_float64(fastcon_lib):
    from fastcon import learn
    for seed in (5, 6, 7):
        X, Y = random_set(300, seed)
        w = learn.init_weights(seed)
        SW = None if seed == 5 else np.random.default_rng(seed).uniform(0.02, 4, (300, 3))
        loss, g = learn.loss_grad(X, Y, w, SW)
        loss_ref, g_ref = loss_grad_np(X, Y, w, SW)
        assert abs(loss - loss_ref) <= 1e-4 * max(1.0, abs(loss_ref))
        # float32 accumulation vs float64: compare relative to the gradient norm
        err = np.abs(g - g_ref).max() / max(np.abs(g_ref).max(), 1e-12)
        assert err < 2e-3, err


def test_training_reduces_loss(fastcon_lib):
    from fastcon import learn
    rng = np.random.default_rng(11)
    X = rng.uniform(0, 1, size=(4000, 12)).astype(np.float32)
    Y = np.stack([(X[:, 0] > X[:, 1]).astype(int), (X[:, 4] > 0.5).astype(int),
                  np.digitize(X[:, 6], [0.33, 0.66])], 1).astype(np.int32)
    w0 = learn.init_weights(0)
    l0, _ = learn.loss_grad(X, Y, w0)
    w, curve = learn.train(X, Y, epochs=30, batch=128, lr=3e-3, w0=w0)
    l1, _ = learn.loss_grad(X, Y, w)
    assert curve[-1] < curve[0] and l1 < 0.5 * l0
    acc = learn.head_accuracy(X, Y, w)
    assert acc["side"] > 0.9 and acc["direction"] > 0.9


def test_traces_and_scripts(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    from fastcon import learn
    u, v = graphs.rmat_edges(14, 8 << 14, seed=61, perm_seed=62)
    G = fc.Graph.from_edges(u, v, 1 << 14)
    rp, col = oracle_mod.build_csr(1 << 14, u, v)
    s, t = graphs.pairs_with_degree(np.diff(rp), 400, seed=63)
    _, want, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=4)
    hops, ins, rec = learn.run_scripted(G, s, t, sched=fc.SCHED_PLAIN, trace=True)
    assert (hops == want).all()
    tr = learn.decode(rec)
    # the steps of each query add up to its total
    tot = np.zeros(len(s), np.int64)
    np.add.at(tot, tr["q"], tr["cost"])
    assert (tot == ins).all()
    assert np.isfinite(tr["feat"]).all() and (tr["feat"] >= 0).all() and (tr["feat"] <= 1.5).all()
    # plain alternates sides: side = step parity
    assert (tr["side"] == tr["step"] % 2).all()
    # a script that forces every step to side 1 top-down still gives exact answers
    script = np.full((len(s), 3), learn.action_byte(1, 0), np.uint8)
    hops2, _, rec2 = learn.run_scripted(G, s, t, script, sched=fc.SCHED_HEURISTIC, trace=True)
    assert (hops2 == want).all()
    tr2 = learn.decode(rec2)
    first = tr2["step"] < 3
    assert (tr2["side"][first] == 1).all()


def test_learned_schedule_is_exact(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    from fastcon import learn
    learn.set_weights(learn.init_weights(21))  # arbitrary weights: answers must not change
    cases = []
    u, v = graphs.rmat_edges(15, 8 << 15, seed=71, perm_seed=72)
    cases.append((1 << 15, u, v))
    u, v = graphs.grid_edges(120, 90, 0.05, 5, 3, 6)
    cases.append((120 * 90, u, v))
    for nv, u, v in cases:
        G = fc.Graph.from_edges(u, v, nv)
        rp, col = oracle_mod.build_csr(nv, u, v)
        s, t = graphs.uniform_pairs(nv, 300, seed=73)
        _, want, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=4)
        for eng in (fc.ENGINE_BATCHED, fc.ENGINE_PERSISTENT, fc.ENGINE_HOSTLOOP):
            o = fc.make_opts(sched=fc.SCHED_LEARNED, engine=eng)
            conn, hops = fc.stcon_batch(G, s, t, opts=o)
            assert (hops == want).all(), (nv, eng)
            lev, _ = oracle_mod.bfs_levels(rp, col, s[0])
            assert (G.bfs_levels(s[0], o) == lev).all()


def test_trained_weights_beat_plain(fastcon_lib, oracle_mod):
    """The committed trained network reads fewer adjacency entries than the
    plain alternating schedule on a held-out graph, with identical answers."""
    fc = fastcon_lib
    from fastcon import learn
    if not os.path.exists(learn.WEIGHTS_PATH):
        pytest.skip("no trained weights committed")
    learn.load_default_weights()
    u, v = graphs.rmat_edges(17, 8 << 17, seed=9, perm_seed=9)
    G = fc.Graph.from_edges(u, v, 1 << 17)
    rp, col = oracle_mod.build_csr(1 << 17, u, v)
    s, t = graphs.pairs_with_degree(np.diff(rp), 1000, seed=19)
    _, want, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=8)
    res = learn.evaluate(G, s, t, want, reps=1)
    assert res["learned"]["exact"] and res["plain"]["exact"] and res["heuristic"]["exact"]
    assert res["learned"]["edges_inspected"] < res["plain"]["edges_inspected"]


def test_box_gate_and_margin(fastcon_lib, oracle_mod):
    """The network steers only inside its feature box and only with a clear
    logit margin; otherwise every decision is the heuristic's."""
    fc = fastcon_lib
    from fastcon import learn
    u, v = graphs.rmat_edges(14, 8 << 14, seed=91, perm_seed=92)
    G = fc.Graph.from_edges(u, v, 1 << 14)
    rp, col = oracle_mod.build_csr(1 << 14, u, v)
    s, t = graphs.pairs_with_degree(np.diff(rp), 300, seed=93)
    _, want, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=4)

    def trace(sched):
        hops, _, rec = learn.run_scripted(G, s, t, sched=sched, trace=True)
        assert (hops == want).all()
        d = learn.decode(rec)
        order = np.lexsort((d["step"], d["q"]))
        return (d["q"][order], d["step"][order], d["side"][order], d["dir"][order],
                d["cost"][order])

    heur = trace(fc.SCHED_HEURISTIC)
    w = np.zeros(1703, np.float32)
    w[1696 + 1] = 10.0  # side-1 logit: always expand t's side, with a clear margin
    full = (np.full(12, -1e9), np.full(12, 1e9))
    learn.set_weights(w, full)
    q, step, side, _, cost = trace(fc.SCHED_LEARNED)
    two = s[q] != t[q]
    # the network moves steps to side 1 where the size gate (1024+ entries)
    # and the trust region let it: more side-1 steps than the heuristic takes
    hq, _, hside, _, _ = heur
    htwo = s[hq] != t[hq]
    assert two.any() and (side[two] == 1).sum() > (hside[htwo] == 1).sum()
    # an empty box: the heuristic decides every step
    learn.set_weights(w, (np.ones(12), np.zeros(12)))
    got = trace(fc.SCHED_LEARNED)
    for a, b in zip(got[:4], heur[:4]):
        assert (a == b).all()
    # a margin below ln 3: the heuristic decides as well
    w[1696 + 1] = 0.5
    learn.set_weights(w, full)
    got = trace(fc.SCHED_LEARNED)
    for a, b in zip(got[:4], heur[:4]):
        assert (a == b).all()
