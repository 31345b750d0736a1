"""BFS trees, shortest paths and predecessor-map validation on the GPU,
against the oracle's restatements (exact integers)."""
import numpy as np
import pytest

from fastcon import graphs

pytestmark = pytest.mark.gpu


def _cases(fc):
    rng = np.random.default_rng(51)
    out = []
    u, v = graphs.rmat_edges(14, 8 << 14, seed=52, perm_seed=53)
    out.append(("rmat14", fc.Graph.from_edges(u, v, 1 << 14), 1 << 14, u, v, False))
    u, v = graphs.grid_edges(60, 50, 0.05, 5, 2, 6)
    out.append(("grid", fc.Graph.from_edges(u, v, 3000), 3000, u, v, False))
    nv = 2000
    u = rng.integers(0, nv, 9000).astype(np.int32)
    v = rng.integers(0, nv, 9000).astype(np.int32)
    out.append(("directed", fc.Graph.from_edges(u, v, nv, flags=fc.INGEST_DIRECTED), nv, u, v, True))
    return out


def _csr_pair(oracle_mod, nv, u, v, directed):
    if not directed:
        rp, col = oracle_mod.build_csr(nv, u, v)
        return rp, col, rp, col
    f = oracle_mod.DROP_LOOPS | oracle_mod.DEDUPE
    rp, col = oracle_mod.build_csr(nv, u, v, flags=f)
    irp, icol = oracle_mod.build_csr(nv, v, u, flags=f)
    return rp, col, irp, icol


def test_parents_paths_and_validation(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    for name, G, nv, u, v, directed in _cases(fc):
        rp, col, irp, icol = _csr_pair(oracle_mod, nv, u, v, directed)
        for s in (0, 7, nv // 2):
            lev_ref, _ = oracle_mod.bfs_levels(rp, col, s)
            par, lev = G.bfs_parents(s, with_levels=True)
            assert (lev == lev_ref).all(), (name, s)
            want = oracle_mod.bfs_parents(irp, icol, lev_ref, s)
            assert (par == want).all(), (name, s)
            e = G.validate_bfs(s, par)
            assert e[:6].tolist() == [0] * 6 and e[6] == int((lev_ref >= 0).sum()), (name, s, e)
            assert e.tolist()[:7] == oracle_mod.validate_bfs(rp, col, irp, icol, par, s, directed)[:7]
            # paths to a few targets: the parent chain, hops + 1 vertices
            for t in np.flatnonzero(lev_ref >= 0)[::97][:6]:
                p = G.stcon_path(s, int(t))
                assert len(p) == lev_ref[t] + 1 and p[0] == s and p[-1] == t
                chain = [int(t)]
                while chain[-1] != s:
                    chain.append(int(want[chain[-1]]))
                assert p.tolist() == chain[::-1]
            unreached = np.flatnonzero(lev_ref < 0)
            if len(unreached):
                assert len(G.stcon_path(s, int(unreached[0]))) == 0


def test_validation_catches_planted_mistakes(fastcon_lib, oracle_mod):
    """Mistakes planted in host predecessor arrays: the GPU counters equal the
    oracle's for every rule."""
    fc = fastcon_lib
    for name, G, nv, u, v, directed in _cases(fc):
        rp, col, irp, icol = _csr_pair(oracle_mod, nv, u, v, directed)
        s = 7
        lev, _ = oracle_mod.bfs_levels(rp, col, s)
        par = oracle_mod.bfs_parents(irp, icol, lev, s)
        deep = np.flatnonzero(lev > 1)
        x = int(deep[0])
        y = int(par[x])
        nonnb = int(np.setdiff1d(np.flatnonzero(lev >= 0), np.append(icol[irp[x]:irp[x + 1]], x))[0])
        plants = []
        b = par.copy(); b[s] = y; plants.append(b)                  # root's parent
        b = par.copy(); b[x] = x; plants.append(b)                  # self parent
        b = par.copy(); b[x] = nv + 5; plants.append(b)             # out of range
        b = par.copy(); b[x] = nonnb; plants.append(b)              # no edge to parent
        b = par.copy(); b[y] = x; plants.append(b)                  # cycle cut off from the root
        b = par.copy(); b[x] = -1; plants.append(b)                 # x dropped from the tree
        b = par.copy(); b[deep[-1]] = s if deep[-1] != s else b[deep[-1]]; plants.append(b)
        for k, b in enumerate(plants):
            got = G.validate_bfs(s, b).tolist()[:7]
            want = oracle_mod.validate_bfs(rp, col, irp, icol, b, s, directed)[:7]
            assert got == want, (name, k, got, want)
            assert any(got[:6]), (name, k)
