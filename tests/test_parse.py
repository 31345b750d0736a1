"""Host edge-list parser (fc_parse_edgelist) against the oracle's sequential
reader: every format, comments inside the body, first-appearance
renumbering, and files large enough to be cut into many thread chunks.  No
GPU needed."""
import os
import tempfile

import numpy as np
import pytest


def _write(td, name, text):
    p = os.path.join(td, name)
    with open(p, "w") as f:
        f.write(text)
    return p


def _same(fc, oracle_mod, path, relabel=False):
    want = oracle_mod.read_edgelist(path, relabel=relabel)
    for nt in (1, 3, 8):
        nv, s, d, fd = fc.parse_edgelist(path, relabel=relabel, nthreads=nt)
        assert nv == want[0] and (s == want[1]).all() and (d == want[2]).all(), (path, nt)
        assert fd == want[3], (path, nt, fd, want[3])
    return want


def test_small_files_every_format(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    with tempfile.TemporaryDirectory() as td:
        snap = _write(td, "g.txt", "# Undirected graph: test\n# Nodes: 6 Edges: 4\n"
                                   "# FromNodeId\tToNodeId\n0\t1\n1\t2\n5\t3\n3\t4\n")
        assert _same(fc, oracle_mod, snap)[0] == 6
        nv, s, d, _ = _same(fc, oracle_mod, snap, relabel=True)
        assert s.tolist() == [0, 1, 3, 4] and d.tolist() == [1, 2, 4, 5]
        _same(fc, oracle_mod, _write(td, "g.mtx", "%%MatrixMarket matrix coordinate pattern "
                                                  "symmetric\n% c\n4 4 3\n2 1\n3 2\n4 1\n"))
        _same(fc, oracle_mod, _write(td, "g.gr", "c test\np sp 3 2\na 1 2 7\na 2 3 9\n"))
        # METIS: an empty line is a vertex without neighbours
        # (readGraphDimacs10, K/Util/readGraphSTD.cpp:101-125, reads one line per vertex)
        d10 = _write(td, "g.graph", "% metis\n4 2\n2\n1\n\n\n")
        nv, s, d, fd = _same(fc, oracle_mod, d10)
        assert nv == 4 and s.tolist() == [0, 1] and d.tolist() == [1, 0]
        d10 = _write(td, "h.graph", "% metis\n4 2\n\n3\n2\n\n")
        nv, s, d, _ = _same(fc, oracle_mod, d10)
        assert s.tolist() == [1, 2] and d.tolist() == [2, 1]
        bad = _write(td, "bad.txt", "hello world\n")
        with pytest.raises(fc.FastconError):
            fc.parse_edgelist(bad)


def test_large_files_many_chunks(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    rng = np.random.default_rng(5)
    with tempfile.TemporaryDirectory() as td:
        # SNAP, 300k lines with comments mid-body and big sparse raw ids
        m = 300000
        u = rng.integers(0, 1 << 30, m)
        v = rng.integers(0, 1 << 30, m)
        lines = ["# Directed graph", "# Nodes: 5 Edges: 9"]
        for i in range(m):
            if i % 50000 == 7:
                lines.append("# a comment inside the body")
            lines.append(f"{u[i]}\t{v[i]}")
        snap = _write(td, "big.txt", "\n".join(lines) + "\n")
        assert os.path.getsize(snap) > (4 << 20)
        _same(fc, oracle_mod, snap, relabel=True)
        small = _write(td, "small_ids.txt", "# Nodes: 10\n" + "".join(
            f"{a} {b}\n" for a, b in zip(rng.integers(0, 90000, m), rng.integers(0, 90000, m))))
        _same(fc, oracle_mod, small)
        _same(fc, oracle_mod, small, relabel=True)
        # METIS with isolated vertices (empty lines) and body comments
        n = 200000
        rows = []
        for i in range(n):
            k = int(rng.integers(0, 6)) if i % 7 else 0
            rows.append(" ".join(str(x) for x in rng.integers(1, n + 1, k)))
            if i % 40000 == 3:
                rows.append("% comment")
        d10 = _write(td, "big.graph", f"% big\n{n} 0\n" + "\n".join(rows) + "\n")
        _same(fc, oracle_mod, d10)
        # DIMACS9 and MatrixMarket
        arcs = "".join(f"a {a} {b} 1\n" for a, b in zip(rng.integers(1, 5000, m), rng.integers(1, 5000, m)))
        _same(fc, oracle_mod, _write(td, "big.gr", "c x\np sp 5000 %d\n" % m + arcs))
        mm = "".join(f"{a} {b}\n" for a, b in zip(rng.integers(1, 7000, m), rng.integers(1, 7000, m)))
        _same(fc, oracle_mod, _write(td, "big.mtx", "%%MatrixMarket matrix coordinate pattern "
                                                    "general\n7000 7000 %d\n" % m + mm))
