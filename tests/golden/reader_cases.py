"""Edge-list files whose parse is pinned to the reference's own readers.

Each case is (name, file text, which readers apply).  The texts are
deterministic functions of fixed seeds, so ``make_golden.py`` (which runs the
reference readers compiled into ``oracle/_ref``) and the tests (which run the
oracle's and the product's readers) see byte-identical files.

Readers:

* ``bfs4k`` -- ``readGraph::readGraphHeader`` + ``readSTD`` + ``Graph::ToCSR``
  (BFS-4K/Util/readGraphHeader.cpp:14-61, BFS-4K/Util/readGraphSTD.cpp:14-145,
  BFS-4K/src/host/graph.cpp:19-42): SNAP ids renumbered by first appearance,
  1-based MatrixMarket / DIMACS9 / DIMACS10 ids shifted to 0-based.
* ``bernaschi`` -- ``load_graph`` (bernaschi/ST_CONN_ONE_ATOMIC/current-st/
  st-conn/load_graph.c:20-104): SNAP only, raw ids, node count from the
  ``# Nodes:`` header.

The files are well formed: the reference readers stop the process on a
malformed file (``error()`` / ``MPI_Abort``), so malformed input is covered
against the oracle only.
"""
from __future__ import annotations

import numpy as np


def _snap(rng, n_nodes, m, directed, raw_span):
    ids = rng.permutation(raw_span)[:n_nodes]  # raw ids, not contiguous
    u = ids[rng.integers(0, n_nodes, m)]
    v = ids[rng.integers(0, n_nodes, m)]
    kind = "Directed" if directed else "Undirected"
    lines = [f"# {kind} graph (each unordered pair of nodes is saved once): sample.txt",
             "# a synthetic graph",
             f"# Nodes: {n_nodes} Edges: {m}",
             "# FromNodeId\tToNodeId"]
    lines += [f"{a}\t{b}" for a, b in zip(u, v)]
    return "\n".join(lines) + "\n"


def _mm(rng, n, m, symmetric):
    u = rng.integers(1, n + 1, m)
    v = rng.integers(1, n + 1, m)
    if symmetric:  # lower triangle, as symmetric MatrixMarket files store it
        u, v = np.maximum(u, v), np.minimum(u, v)
    kind = "symmetric" if symmetric else "general"
    lines = [f"%%MatrixMarket matrix coordinate pattern {kind}", "% synthetic", "%",
             f"{n} {n} {m}"]
    lines += [f"{a} {b}" for a, b in zip(u, v)]
    return "\n".join(lines) + "\n"


def _dimacs9(rng, n, m):
    u = rng.integers(1, n + 1, m)
    v = rng.integers(1, n + 1, m)
    w = rng.integers(1, 1000, m)
    lines = ["c 9th DIMACS challenge format", "c synthetic", f"p sp {n} {m}"]
    lines += [f"a {a} {b} {c}" for a, b, c in zip(u, v, w)]
    return "\n".join(lines) + "\n"


def _dimacs10(rng, n, max_deg):
    rows = []
    nent = 0
    for i in range(n):
        k = int(rng.integers(0, max_deg + 1)) if i % 5 else 0  # every 5th vertex isolated
        nb = rng.integers(1, n + 1, k)
        nent += k
        rows.append(" ".join(str(x) for x in nb))
    # the reader sizes its edge array from the header (2 x edges): round up
    return "% METIS adjacency lines\n" + f"{n} {(nent + 1) // 2}\n" + "\n".join(rows) + "\n"


def cases():
    rng = np.random.default_rng(20240611)
    out = []
    out.append(("snap_undirected_small",
                "# Undirected graph: tiny.txt\n# Nodes: 7 Edges: 6\n# FromNodeId\tToNodeId\n"
                "10\t4\n4\t3\n3\t10\n42\t7\n7\t0\n0\t42\n", ("bfs4k",)))
    out.append(("snap_directed_small",
                "# Directed graph: tiny.txt\n# Nodes: 6 Edges: 5\n# FromNodeId\tToNodeId\n"
                "0\t1\n1\t2\n5\t3\n3\t4\n4\t5\n", ("bfs4k", "bernaschi")))
    out.append(("snap_undirected_5k", _snap(rng, 1500, 5000, False, 1 << 20), ("bfs4k",)))
    out.append(("snap_directed_5k", _snap(rng, 1500, 5000, True, 1 << 20), ("bfs4k",)))
    # raw ids below the header's node count (bernaschi keeps raw ids)
    out.append(("snap_raw_ids_5k", _snap(rng, 2000, 5000, False, 2000), ("bfs4k", "bernaschi")))
    out.append(("mm_symmetric_small", "%%MatrixMarket matrix coordinate pattern symmetric\n"
                "% c\n4 4 3\n2 1\n3 2\n4 1\n", ("bfs4k",)))
    out.append(("mm_symmetric_5k", _mm(rng, 1200, 5000, True), ("bfs4k",)))
    out.append(("mm_general_5k", _mm(rng, 1200, 5000, False), ("bfs4k",)))
    out.append(("dimacs9_small", "c test\np sp 3 2\na 1 2 7\na 2 3 9\n", ("bfs4k",)))
    out.append(("dimacs9_5k", _dimacs9(rng, 900, 5000), ("bfs4k",)))
    out.append(("dimacs10_small", "% metis\n4 2\n2\n1 3\n2\n\n", ("bfs4k",)))
    out.append(("dimacs10_1k", _dimacs10(rng, 1000, 9), ("bfs4k",)))
    return out
