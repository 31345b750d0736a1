"""ctypes binding of the CPU oracle (oracle/liboracle.so) and of the
reference's own CPU BFS compiled into oracle/_ref/libref_bfs.so.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, always as the checker.  The product library
never loads it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_BFS_PATH = os.path.join(HERE, "_ref", "libref_bfs.so")
REF_GEN_PATH = os.path.join(HERE, "_ref", "graph500_gen")
REF_READ_PATH = os.path.join(HERE, "_ref", "libref_read.so")
REF_LOADGRAPH_PATH = os.path.join(HERE, "_ref", "libref_loadgraph.so")

SYMMETRIZE, DROP_LOOPS, DEDUPE = 1, 2, 4
CANONICAL = SYMMETRIZE | DROP_LOOPS | DEDUPE

_lib = None
_ref = None


def build(ref_root: str | None = None) -> None:
    """Compile liboracle.so; also oracle/_ref when the reference sources are
    present at ref_root."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if ref_root and os.path.isdir(ref_root):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_root}"], check=True)


def _P(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.oracle_bfs_levels.restype = ctypes.c_int32
        L.oracle_bfs_levels.argtypes = [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p]
        for fn in (L.oracle_stcon_batch, L.oracle_stcon_bidir_batch):
            fn.restype = ctypes.c_int
            fn.argtypes = [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                           ctypes.c_void_p, ctypes.c_int]
        L.oracle_build_csr.restype = ctypes.c_int64
        L.oracle_build_csr.argtypes = [ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_void_p]
        L.oracle_build_csr_mt.restype = ctypes.c_int64
        L.oracle_build_csr_mt.argtypes = [ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_int]
        L.oracle_gen_rmat.restype = None
        L.oracle_gen_rmat.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                      ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_int]
        L.oracle_count_visited_edges.restype = ctypes.c_int64
        L.oracle_count_visited_edges.argtypes = [ctypes.c_int32, ctypes.c_void_p,
                                                 ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_read_edgelist.restype = ctypes.c_int
        L.oracle_read_edgelist.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p]
        _lib = L
    return _lib


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def bfs_levels(row_ptr, col, src):
    """Levels from src (-1 unreachable) and edges inspected."""
    row_ptr, col = _i32(row_ptr), _i32(col)
    nv = len(row_ptr) - 1
    lev = np.empty(nv, np.int32)
    q = np.empty(nv, np.int32)
    ins = np.zeros(1, np.int64)
    lib().oracle_bfs_levels(nv, _P(row_ptr), _P(col), int(src), _P(lev), _P(q), _P(ins))
    return lev, int(ins[0])


def stcon_batch(row_ptr, col, s, t, nthreads=1, bidir=False):
    """(connected int32[nq], hops int32[nq], edges_inspected int64[nq])."""
    row_ptr, col, s, t = _i32(row_ptr), _i32(col), _i32(s), _i32(t)
    nv = len(row_ptr) - 1
    nq = len(s)
    conn = np.zeros(nq, np.int32)
    hops = np.zeros(nq, np.int32)
    ins = np.zeros(nq, np.int64)
    fn = lib().oracle_stcon_bidir_batch if bidir else lib().oracle_stcon_batch
    rc = fn(nv, _P(row_ptr), _P(col), nq, _P(s), _P(t), _P(conn), _P(hops), _P(ins),
            int(nthreads))
    if rc != 0:
        raise ValueError("oracle_stcon_batch: vertex id out of range")
    return conn, hops, ins


def build_csr(nv, src, dst, flags=CANONICAL, nthreads=1):
    src, dst = _i32(src), _i32(dst)
    rp = np.zeros(nv + 1, np.int32)
    cap = 2 * len(src) if flags & SYMMETRIZE else len(src)
    col = np.zeros(max(1, cap), np.int32)
    ne = lib().oracle_build_csr_mt(int(nv), len(src), _P(src), _P(dst), int(flags), _P(rp),
                                   _P(col), int(nthreads))
    if ne < 0:
        raise ValueError("oracle_build_csr: bad edge list")
    return rp, (col[:ne].copy() if ne < len(col) // 2 else col[:ne])


def gen_rmat(scale, nedges, a=0.57, b=0.19, c=0.19, seed=3, perm_seed=-1, nthreads=1):
    """R-MAT samples (same hash stream as fastcon/graphs.py and the GPU)."""
    src = np.empty(max(1, nedges), np.int32)
    dst = np.empty(max(1, nedges), np.int32)
    lib().oracle_gen_rmat(int(scale), int(nedges), float(a), float(b), float(c), int(seed),
                          int(perm_seed), _P(src), _P(dst), int(nthreads))
    return src[:nedges], dst[:nedges]


def count_visited_edges(row_ptr, col, levels):
    row_ptr, col, levels = _i32(row_ptr), _i32(col), _i32(levels)
    return int(lib().oracle_count_visited_edges(len(row_ptr) - 1, _P(row_ptr), _P(col),
                                                _P(levels)))


def bfs_parents(in_row_ptr, in_col, levels, s):
    """Deterministic BFS tree from a level array: parent(v) = the smallest
    in-neighbour one level closer to s; parent(s) = s; -1 where unreached."""
    rp, col, lev = (np.asarray(x, np.int64) for x in (in_row_ptr, in_col, levels))
    nv = len(rp) - 1
    rows = np.repeat(np.arange(nv), np.diff(rp))
    ok = (lev[rows] > 0) & (lev[col] == lev[rows] - 1)
    par = np.full(nv, np.iinfo(np.int64).max)
    np.minimum.at(par, rows[ok], col[ok])
    par[par == np.iinfo(np.int64).max] = -1
    par[lev <= 0] = -1
    par[s] = s
    return par.astype(np.int32)


def validate_bfs(row_ptr, col, in_row_ptr, in_col, parents, root, directed=False):
    """validate_bfs_result (S/reference_functions.c:99-434) restated for one
    process with the same seven counters as fc_validate_bfs: [0] root's
    parent wrong, [1] self parent or out of range, [2] no edge parent -> v,
    [3] chain does not reach the root, [4] edge from the tree to outside,
    [5] depth gap over an edge, [6] vertices in the tree."""
    rp, cl, irp, icl = (np.asarray(x, np.int64) for x in (row_ptr, col, in_row_ptr, in_col))
    par = np.asarray(parents, np.int64)
    nv = len(rp) - 1
    e = [0] * 8
    e[0] = int(par[root] != root)
    v = np.arange(nv)
    bad = (v != root) & (par != -1) & ((par < 0) | (par >= nv) | (par == v))
    e[1] = int(bad.sum())
    e[6] = int(((par != -1) | (v == root)).sum())
    good = (v != root) & (par >= 0) & (par < nv) & (par != v)
    miss = 0
    for x in np.flatnonzero(good):
        row = icl[irp[x]:irp[x + 1]]
        k = np.searchsorted(row, par[x])
        miss += int(k >= len(row) or row[k] != par[x])
    e[2] = miss
    depth = np.full(nv, -1, np.int64)
    depth[root] = 0
    for x in np.flatnonzero(good | bad):
        if depth[x] >= 0:
            continue
        chain, y = [], x
        while 0 <= y < nv and depth[y] == -1 and y != root and len(chain) <= nv and par[y] != -1:
            chain.append(y)
            if (par[y] < 0 or par[y] >= nv or par[y] == y):
                y = -1
                break
            y = par[y]
        d = depth[y] if 0 <= y < nv and depth[y] >= 0 else None
        if d is None:
            for c in chain:
                depth[c] = -2
        else:
            for c in reversed(chain):
                d += 1
                depth[c] = d
    e[3] = int(((good | bad) & (depth < 0)).sum())
    d = np.where(depth >= 0, depth, -1)
    rows = np.repeat(np.arange(nv), np.diff(rp))
    du, dv = d[rows], d[cl]
    tree = du >= 0
    e[4] = int((tree & (dv < 0)).sum())
    both = tree & (dv >= 0)
    gap = (dv - du > 1) if directed else (np.abs(dv - du) > 1)
    e[5] = int((both & gap).sum())
    return e


def read_edgelist(path, relabel=False):
    """(nv, src int32, dst int32, file_directed)."""
    nv = np.zeros(1, np.int32)
    n = np.zeros(1, np.int64)
    fd = np.zeros(1, np.int32)
    rc = lib().oracle_read_edgelist(path.encode(), int(relabel), _P(nv), _P(n), _P(fd), None, None)
    if rc != 0:
        raise ValueError(f"oracle_read_edgelist: cannot parse {path}")
    src = np.zeros(max(1, int(n[0])), np.int32)
    dst = np.zeros(max(1, int(n[0])), np.int32)
    rc = lib().oracle_read_edgelist(path.encode(), int(relabel), _P(nv), _P(n), _P(fd),
                                    _P(src), _P(dst))
    if rc != 0:
        raise ValueError(f"oracle_read_edgelist: cannot parse {path}")
    return int(nv[0]), src[: int(n[0])], dst[: int(n[0])], int(fd[0])


# ---------------------------------------------------------------------------
# The reference's own CPU BFS (compiled from its sources; present only where
# the reference tree was available at build time).
# ---------------------------------------------------------------------------
def ref_available() -> bool:
    return os.path.exists(REF_BFS_PATH)


def ref():
    global _ref
    if _ref is None:
        R = ctypes.CDLL(REF_BFS_PATH)
        R.ref_bfs_many.restype = ctypes.c_int
        R.ref_bfs_many.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p]
        R.ref_inf.restype = ctypes.c_int
        _ref = R
    return _ref


def ref_bfs_levels(row_ptr, col, sources):
    """Reference Graph::bfs distances, INF mapped to -1: int32[len(sources), nv]."""
    row_ptr, col = _i32(row_ptr), _i32(col)
    src = _i32(sources)
    nv = len(row_ptr) - 1
    dist = np.zeros((len(src), nv), np.int32)
    vis = np.zeros(len(src), np.int32)
    ref().ref_bfs_many(nv, len(col), _P(row_ptr), _P(col), len(src), _P(src), _P(dist), _P(vis))
    inf = ref().ref_inf()
    dist[dist == inf] = -1
    return dist, vis


# ---------------------------------------------------------------------------
# The reference's own edge-list readers (compiled from its sources into
# oracle/_ref/ where the reference tree was available; used only to write the
# reader fixtures of tests/golden/).
# ---------------------------------------------------------------------------
def ref_read_graph(path: str, user_dir: int = 2):
    """BFS-4K readGraphHeader + readSTD + ToCSR on `path` (user_dir 0
    directed, 1 undirected, 2 as the file says): dict with V, E, direction
    (0/1), coo int32[n, 2] in the reader's order, row_ptr, col."""
    R = ctypes.CDLL(REF_READ_PATH)
    R.ref_read_graph.restype = ctypes.c_int
    IP = ctypes.POINTER(ctypes.c_int)
    R.ref_read_graph.argtypes = [ctypes.c_char_p, ctypes.c_int, IP, IP, IP, IP,
                                 ctypes.POINTER(IP), ctypes.POINTER(IP), ctypes.POINTER(IP)]
    R.ref_read_free.argtypes = [ctypes.c_void_p]
    V, E, d, n = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    coo, rp, col = IP(), IP(), IP()
    R.ref_read_graph(path.encode(), int(user_dir), ctypes.byref(V), ctypes.byref(E),
                     ctypes.byref(d), ctypes.byref(n), ctypes.byref(coo), ctypes.byref(rp),
                     ctypes.byref(col))
    out = {"V": V.value, "E": E.value, "direction": d.value,
           "coo": np.ctypeslib.as_array(coo, shape=(max(1, 2 * n.value),))[: 2 * n.value]
           .reshape(-1, 2).copy(),
           "row_ptr": np.ctypeslib.as_array(rp, shape=(V.value + 1,)).copy()}
    ne = int(out["row_ptr"][-1])
    out["col"] = np.ctypeslib.as_array(col, shape=(max(1, ne),))[:ne].copy()
    for p in (coo, rp, col):
        R.ref_read_free(ctypes.cast(p, ctypes.c_void_p))
    return out


def ref_load_graph(path: str):
    """bernaschi load_graph on `path` (one rank): (nverts, int64[n, 2] raw
    (u, v) pairs in file order)."""
    R = ctypes.CDLL(REF_LOADGRAPH_PATH)
    R.ref_load_graph.restype = ctypes.c_int
    LP = ctypes.POINTER(ctypes.c_int64)
    R.ref_load_graph.argtypes = [ctypes.c_char_p, LP, ctypes.POINTER(LP), LP]
    R.ref_free.argtypes = [ctypes.c_void_p]
    n, nv, e = ctypes.c_int64(), ctypes.c_int64(), LP()
    R.ref_load_graph(path.encode(), ctypes.byref(n), ctypes.byref(e), ctypes.byref(nv))
    pairs = np.ctypeslib.as_array(e, shape=(max(1, 2 * n.value),))[: 2 * n.value].reshape(-1, 2).copy()
    R.ref_free(ctypes.cast(e, ctypes.c_void_p))
    return int(nv.value), pairs
