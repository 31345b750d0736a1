"""Regenerates the golden fixtures in this folder from the reference itself.

Run in a checkout that has the reference tree (read-only) available:

    python tests/golden/make_golden.py --ref /path/to/reference

What it writes (all small, all committed):

* ``stcon_known_answer.json`` -- the 100 (RED-V, BLUE-V, DEPTH) rows and the
  graph header of the reference's logged ST-CON run
  ``bernaschi/ST_CONN_ONE_ATOMIC/current-st/st-conn/data/st_stats_20200418_140644``
  (Graph500 R-MAT, SCALE 16, edgefactor 16, seeds 670021781 / 1422323141).
* ``rmat16_graph500_edges.npz`` -- that graph's edge list, produced by the
  reference's vendored Graph500 generator (compiled by ``oracle/Makefile``
  into ``oracle/_ref/graph500_gen``), symmetrised, loop-free and deduped,
  stored as the sorted upper triangle (u < v): ``du`` = deltas of u, ``v``.
* ``ref_readers.json`` -- what the reference's own edge-list readers make of
  the files of ``reader_cases.py``: BFS-4K's ``readGraphHeader`` +
  ``readSTD`` + ``Graph::ToCSR`` (compiled into ``oracle/_ref/libref_read.so``)
  and bernaschi's ``load_graph`` (``oracle/_ref/libref_loadgraph.so``):
  vertex count, direction, the COO list in the reader's order and the CSR,
  as SHA-256 digests plus the full arrays of the small files.
* ``ref_graph500.json`` -- the reference's Graph500 generator (make_graph,
  ``oracle/_ref/graph500_gen``) at a few sizes and seeds: its raw edge list
  (both ends, smaller first, self-loops and repeats kept) sorted, and the
  canonical CSR built from it, as SHA-256 digests and counts.
* ``ref_bfs_*.json`` -- outputs of the reference's own CPU BFS
  (``Graph::bfs``, BFS-4K/src/host/graph.cpp:83-97, compiled into
  ``oracle/_ref/libref_bfs.so``) on the ER workload (65,536 vertices,
  524,288 edges, seed 1; 64 pairs, seed 2), on the known-answer graph, and
  on a set of tiny edge-case graphs (full level arrays for the tiny ones,
  SHA-256 of the int32 level arrays for the large ones).
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "fast-con_gb300"))

import oracle  # noqa: E402
from fastcon import graphs  # noqa: E402

STATS = "bernaschi/ST_CONN_ONE_ATOMIC/current-st/st-conn/data/st_stats_20200418_140644"


def sha_levels(lev: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(lev, dtype="<i4").tobytes()).hexdigest()


def sha_csr(rp, col) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(rp, dtype="<i4").tobytes())
    h.update(np.ascontiguousarray(col, dtype="<i4").tobytes())
    return h.hexdigest()


def tiny_graphs():
    """Edge-case graphs: (name, nv, edges)."""
    g = []
    g.append(("single_vertex", 1, []))
    g.append(("two_isolated", 2, []))
    g.append(("one_edge", 2, [(0, 1)]))
    g.append(("path10", 10, [(i, i + 1) for i in range(9)]))
    g.append(("star9", 9, [(0, i) for i in range(1, 9)]))
    g.append(("two_components", 8, [(0, 1), (1, 2), (2, 3), (4, 5), (5, 6), (6, 7), (7, 4)]))
    g.append(("loops_and_dups", 6, [(0, 0), (0, 1), (1, 0), (0, 1), (1, 2), (2, 2), (2, 3),
                                    (3, 4), (4, 3), (5, 5)]))
    g.append(("cycle7", 7, [(i, (i + 1) % 7) for i in range(7)]))
    g.append(("complete6", 6, [(i, j) for i in range(6) for j in range(i + 1, 6)]))
    # 8x8 grid with a few edges removed
    es = []
    for r in range(8):
        for c in range(8):
            v = r * 8 + c
            if c < 7 and (r * 7 + c) % 5 != 3:
                es.append((v, v + 1))
            if r < 7 and (r * 8 + c) % 7 != 2:
                es.append((v, v + 8))
    g.append(("grid8_holes", 64, es))
    # hub with a long tail: high degree next to a path
    es = [(0, i) for i in range(1, 200)] + [(199 + i, 200 + i) for i in range(60)]
    g.append(("hub_tail", 260, es))
    return g


def sha_i32(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()


def reader_fixtures():
    """ref_readers.json from the reference readers run on reader_cases.py."""
    sys.path.insert(0, HERE)
    import reader_cases
    out = []
    with tempfile.TemporaryDirectory() as td:
        for name, text, readers in reader_cases.cases():
            p = os.path.join(td, name)
            with open(p, "w") as f:
                f.write(text)
            rec = {"name": name, "readers": list(readers)}
            r = oracle.ref_read_graph(p)
            small = len(r["coo"]) <= 64
            rec["bfs4k"] = {"V": r["V"], "direction": r["direction"],
                            "coo_n": int(len(r["coo"])), "coo_sha256": sha_i32(r["coo"]),
                            "row_ptr_sha256": sha_i32(r["row_ptr"]),
                            "col_sha256": sha_i32(r["col"])}
            if small:
                rec["bfs4k"].update(coo=r["coo"].tolist(), row_ptr=r["row_ptr"].tolist(),
                                    col=r["col"].tolist())
            if "bernaschi" in readers:
                nv, pairs = oracle.ref_load_graph(p)
                rec["bernaschi"] = {"nverts": nv, "n": int(len(pairs)),
                                    "pairs_sha256": sha_i32(pairs)}
                if small:
                    rec["bernaschi"]["pairs"] = pairs.tolist()
            out.append(rec)
    json.dump(out, open(os.path.join(HERE, "ref_readers.json"), "w"), indent=1)


GRAPH500_CASES = [(8, 16, 1, 2), (10, 16, 1, 2), (12, 16, 77, 991), (14, 8, 5, 6),
                  (16, 16, 670021781, 1422323141)]


def graph500_fixtures():
    """ref_graph500.json from the reference generator."""
    out = []
    with tempfile.TemporaryDirectory() as td:
        for scale, ef, s1, s2 in GRAPH500_CASES:
            path = os.path.join(td, "e.bin")
            subprocess.run([oracle.REF_GEN_PATH, str(scale), str(ef), str(s1), str(s2), path],
                           check=True, stdout=subprocess.DEVNULL)
            e = np.fromfile(path, dtype=np.int64).reshape(-1, 2)
            lo = np.minimum(e[:, 0], e[:, 1]).astype(np.int32)
            hi = np.maximum(e[:, 0], e[:, 1]).astype(np.int32)
            o = np.lexsort((hi, lo))
            pairs = np.stack([lo[o], hi[o]], 1)
            nv = 1 << scale
            rp, col = oracle.build_csr(nv, lo, hi)
            out.append({"scale": scale, "edgefactor": ef, "seed1": s1, "seed2": s2,
                        "nedges": int(len(e)), "self_loops": int((lo == hi).sum()),
                        "sorted_edges_sha256": sha_levels(pairs.reshape(-1)),
                        "directed_entries": int(len(col)), "csr_sha256": sha_csr(rp, col)})
    json.dump(out, open(os.path.join(HERE, "ref_graph500.json"), "w"), indent=1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("FASTCON_REFERENCE", ""),
                    help="root of the reference tree")
    ap.add_argument("--only", default=None, choices=["readers", "graph500"],
                    help="write only this fixture")
    args = ap.parse_args()
    if not args.ref or not os.path.isdir(args.ref):
        sys.exit("reference tree not found; pass --ref")
    oracle.build(args.ref)
    if args.only == "readers":
        reader_fixtures()
        return
    if args.only == "graph500":
        graph500_fixtures()
        return

    # 1. known-answer rows
    lines = open(os.path.join(args.ref, STATS)).read().splitlines()
    hdr = {}
    for ln in lines[:7]:
        k, v = re.split(r"[ =]", ln.strip(), maxsplit=1)
        hdr[k] = v.strip()
    rows = []
    for ln in lines:
        p = ln.split()
        if len(p) == 7 and p[0].isdigit():
            rows.append({"run": int(p[0]), "red": int(p[1]), "blue": int(p[2]),
                         "depth": int(p[3]), "mn_found": int(p[4])})
    assert len(rows) == 100, len(rows)
    scale = int(hdr["SCALE"])
    ef = float(hdr["Edgefactor"])
    seed1, seed2 = int(hdr["Seed1"]), int(hdr["Seed2"])

    # 2. the graph, from the reference's generator
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "edges.bin")
        subprocess.run([oracle.REF_GEN_PATH, str(scale), str(ef), str(seed1), str(seed2), out],
                       check=True, stdout=subprocess.DEVNULL)
        e = np.fromfile(out, dtype=np.int64).reshape(-1, 2)
    n_generated = len(e)
    e = e[e[:, 0] >= 0]
    nv = 1 << scale
    u = np.minimum(e[:, 0], e[:, 1])
    v = np.maximum(e[:, 0], e[:, 1])
    ok = u != v
    key = np.unique(u[ok] * nv + v[ok])
    uu = (key // nv).astype(np.int64)
    vv = (key % nv).astype(np.int64)
    du = np.diff(np.concatenate([[0], uu])).astype(np.uint16)
    assert int(np.abs(np.diff(np.concatenate([[0], uu]))).max()) < 65536
    np.savez_compressed(os.path.join(HERE, "rmat16_graph500_edges.npz"),
                        du=du, v=vv.astype(np.uint16))
    rp, col = oracle.build_csr(nv, uu.astype(np.int32), vv.astype(np.int32))

    red = np.array([r["red"] for r in rows], np.int32)
    blue = np.array([r["blue"] for r in rows], np.int32)
    dist, vis = oracle.ref_bfs_levels(rp, col, red)
    ka = {
        "source": STATS,
        "header": hdr,
        "graph": {"scale": scale, "edgefactor": ef, "seed1": seed1, "seed2": seed2,
                  "initiator": [0.57, 0.19, 0.19, 0.05], "generated_edges": int(n_generated),
                  "undirected_unique": int(len(key)), "directed_entries": int(len(col)),
                  "csr_sha256": sha_csr(rp, col)},
        "rows": rows,
        "ref_bfs_hops": [int(dist[i, blue[i]]) for i in range(len(rows))],
        "ref_bfs_levels_sha256": [sha_levels(dist[i]) for i in range(len(rows))],
        "ref_bfs_visited": [int(x) for x in vis],
    }
    json.dump(ka, open(os.path.join(HERE, "stcon_known_answer.json"), "w"), indent=1)

    # 3. ER workload: 65,536 vertices, 524,288 edges, seed 1; pairs seed 2
    n, m = 65536, 524288
    eu, ev = graphs.er_edges(n, m, seed=1)
    rp, col = oracle.build_csr(n, eu, ev)
    s, t = graphs.uniform_pairs(n, 64, seed=2)
    dist, vis = oracle.ref_bfs_levels(rp, col, s)
    er = {
        "graph": {"kind": "er", "n": n, "m": m, "seed": 1, "directed_entries": int(len(col)),
                  "csr_sha256": sha_csr(rp, col)},
        "pairs_seed": 2,
        "s": [int(x) for x in s], "t": [int(x) for x in t],
        "hops": [int(dist[i, t[i]]) for i in range(len(s))],
        "levels_sha256": [sha_levels(dist[i]) for i in range(len(s))],
        "visited": [int(x) for x in vis],
        "max_level": [int(dist[i].max()) for i in range(len(s))],
    }
    json.dump(er, open(os.path.join(HERE, "ref_bfs_er65536.json"), "w"), indent=1)

    # 4. tiny edge cases: full level arrays from every source
    tiny = []
    for name, nvt, es in tiny_graphs():
        a = np.array([x[0] for x in es], np.int32)
        b = np.array([x[1] for x in es], np.int32)
        rp, col = oracle.build_csr(nvt, a, b)
        srcs = np.arange(nvt, dtype=np.int32) if nvt <= 64 else \
            np.unique(np.concatenate([np.arange(8), np.arange(0, nvt, 23), [nvt - 1]])).astype(np.int32)
        dist, _ = oracle.ref_bfs_levels(rp, col, srcs)
        tiny.append({"name": name, "nv": nvt, "edges": [list(x) for x in es],
                     "row_ptr": [int(x) for x in rp], "col": [int(x) for x in col],
                     "sources": [int(x) for x in srcs], "levels": dist.tolist()})
    json.dump(tiny, open(os.path.join(HERE, "ref_bfs_tiny.json"), "w"))

    # 5. the edge-list readers
    reader_fixtures()
    # 6. the Graph500 generator
    graph500_fixtures()
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
