"""Multi-seed s~t connectivity (region growth + device union-find) against
the oracle's connectivity; exact yes/no on graphs with several components."""
import numpy as np
import pytest

from fastcon import graphs

pytestmark = pytest.mark.gpu


def test_multiseed_connectivity_matches_oracle(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    rng = np.random.default_rng(61)
    cases = []
    u, v = graphs.rmat_edges(14, 4 << 14, seed=62, perm_seed=63)   # isolated vertices
    cases.append((1 << 14, u, v))
    u, v = graphs.grid_edges(80, 60, 0.35, 64, 0, 65)               # many grid components
    cases.append((80 * 60, u, v))
    nv = 5000                                                        # sparse random: components
    cases.append((nv, rng.integers(0, nv, 2600).astype(np.int32),
                  rng.integers(0, nv, 2600).astype(np.int32)))
    for nv, u, v in cases:
        G = fc.Graph.from_edges(u, v, nv)
        rp, col = oracle_mod.build_csr(nv, u, v)
        s, t = graphs.uniform_pairs(nv, 120, seed=66)
        s[:3] = [5, 5, 0]
        t[:3] = [5, 6, nv - 1]
        conn, _, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=4)
        assert conn.any() and not conn.all()
        for nseeds in (2, 17, 320, 4096):
            for k in range(0, 120, 7 if nseeds != 320 else 1):
                got, st = G.stcon_multiseed(int(s[k]), int(t[k]), nseeds=nseeds, seed=k + 1,
                                            stats=True)
                assert got == bool(conn[k]), (nv, nseeds, k)
                assert st["visited"] >= 1


def test_multiseed_rejects_directed_and_bad_sizes(fastcon_lib):
    fc = fastcon_lib
    u = np.array([0, 1, 2], np.int32)
    v = np.array([1, 2, 3], np.int32)
    D = fc.Graph.from_edges(u, v, 4, flags=fc.INGEST_DIRECTED)
    with pytest.raises(fc.FastconError):
        D.stcon_multiseed(0, 3)
    G = fc.Graph.from_edges(u, v, 4)
    assert G.stcon_multiseed(0, 3, nseeds=2)
    with pytest.raises(fc.FastconError):
        G.stcon_multiseed(0, 3, nseeds=1)
    with pytest.raises(fc.FastconError):
        G.stcon_multiseed(0, 3, nseeds=5000)
