"""Python binding of libfastcon.so (the C ABI in include/fastcon.h).

Thin ctypes layer used by the tests and the benchmark.  Every call goes to the
CUDA library; there is no CPU path here.  Loading fails loudly when the
library has not been built (``python fast-con_gb300/build.py``).

Names follow the reference's host entry points:

* ``Graph.load_edgelist``  -- load_graph + run_make_struct (S/load_graph.c:20,
  S/make_struct.c:39) / readGraph::readSTD (K/Util/readGraphSTD.cpp:14)
* ``Graph.bfs_levels``     -- cudaGraph::Reset + cudaBFS4K (K/src/device/
  BFS_WorkEfficient.cu:81-133): level array, -1 where the reference has INF
* ``Graph.stcon``          -- make_stcon (S/make_stcon.c:730) with the exact
  hop distance; ``Graph.stcon_depth`` returns make_stcon's DEPTH = ceil(d/2)
* ``stcon_batch``          -- the query loop of run_make_stcon
  (S/make_stcon.c:416-576) as one call
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfastcon.so")

OK, ERR_INVALID, ERR_CUDA, ERR_OOM, ERR_IO, ERR_FORMAT, ERR_TIMEOUT, ERR_OVERFLOW, \
    ERR_NO_DEVICE, ERR_UNSUPPORTED = range(10)
INGEST_DIRECTED, INGEST_KEEP_LOOPS, INGEST_KEEP_DUPS = 1, 2, 4
SCHED_PLAIN, SCHED_HEURISTIC, SCHED_LEARNED = 0, 1, 2
ENGINE_AUTO, ENGINE_HOSTLOOP, ENGINE_PERSISTENT, ENGINE_BATCHED = 0, 1, 2, 3
ORDER_AUTO, ORDER_GIVEN, ORDER_DEGREE = 0, 1, 2

# Every symbol include/fastcon.h declares.
EXPORTS = [
    "fc_opts_init", "fc_graph_load_edgelist", "fc_graph_from_csr", "fc_graph_from_edges",
    "fc_graph_from_device_edges", "fc_graph_generate_rmat", "fc_graph_generate_grid",
    "fc_graph_info", "fc_graph_get_csr", "fc_graph_free", "fc_bfs_levels", "fc_bfs_levels_ex",
    "fc_bfs_trace", "fc_graph_generate_graph500", "fc_graph_generate_graph500_edges",
    "fc_selftest_primitives",
    "fc_stcon", "fc_stcon_ex", "fc_stcon_depth", "fc_stcon_batch", "fc_stcon_batch_device",
    "fc_stcon_batch_noalloc", "fc_sched_set_weights", "fc_sched_get_weights",
    "fc_mlp_loss_grad", "fc_mlp_train", "fc_stcon_batch_scripted", "fc_selftest_wait",
    "fc_bfs_parents", "fc_stcon_path", "fc_validate_bfs", "fc_parse_edgelist",
    "fc_stcon_multiseed", "fc_autotune_batch",
    "fc_strerror", "fc_last_error_message", "fc_device_info", "fc_version",
]


class FastconError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{msg} (code {code})")
        self.code = code


class Opts(ctypes.Structure):
    _fields_ = [("sched", ctypes.c_int32), ("engine", ctypes.c_int32), ("block", ctypes.c_int32),
                ("ctas_per_sm", ctypes.c_int32), ("use_graph", ctypes.c_int32),
                ("max_slots", ctypes.c_int32), ("stream", ctypes.c_void_p),
                ("cta_work_k", ctypes.c_int32), ("variant", ctypes.c_int32),
                ("tile_entries", ctypes.c_int32), ("job_entries", ctypes.c_int32),
                ("private_variant", ctypes.c_int32), ("vertex_order", ctypes.c_int32),
                ("slot_log_cap", ctypes.c_int32), ("reserved", ctypes.c_int32 * 1)]


class Stats(ctypes.Structure):
    _fields_ = [("edges_inspected", ctypes.c_int64), ("visited", ctypes.c_int64),
                ("steps", ctypes.c_int32), ("bottom_up_steps", ctypes.c_int32),
                ("gpu_ms", ctypes.c_double), ("alg_bytes", ctypes.c_int64),
                ("escalated", ctypes.c_int32), ("launches", ctypes.c_int32),
                ("kernel_ms", ctypes.c_double * 2), ("kernel_alg_bytes", ctypes.c_int64 * 2),
                ("graph", ctypes.c_int32), ("pad_", ctypes.c_int32),
                ("visited_adjacency", ctypes.c_int64)]

    def as_dict(self):
        d = {}
        for k, _ in self._fields_:
            v = getattr(self, k)
            d[k] = list(v) if isinstance(v, ctypes.Array) else v
        return d


_lib = None
_VP = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FastconError(ERR_UNSUPPORTED,
                               f"{LIB_PATH} not built; run python fast-con_gb300/build.py")
        L = ctypes.CDLL(LIB_PATH)
        sig = {
            "fc_opts_init": (None, [_VP]),
            "fc_graph_load_edgelist": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, _VP]),
            "fc_graph_from_csr": (ctypes.c_int, [_VP, _I32, _VP, _I64, ctypes.c_int, _VP]),
            "fc_graph_from_edges": (ctypes.c_int, [_VP, _VP, _I64, _I32, ctypes.c_int, _VP]),
            "fc_graph_from_device_edges": (ctypes.c_int, [_VP, _VP, _I64, _I32, ctypes.c_int, _VP]),
            "fc_graph_generate_rmat": (ctypes.c_int, [_I32, _I64, ctypes.c_double, ctypes.c_double,
                                                      ctypes.c_double, ctypes.c_uint64, _I64, _VP]),
            "fc_graph_generate_grid": (ctypes.c_int, [_I32, _I32, ctypes.c_double, ctypes.c_uint64,
                                                      _I64, ctypes.c_uint64, _VP]),
            "fc_graph_generate_graph500": (ctypes.c_int, [_I32, _I64, ctypes.c_uint64,
                                                          ctypes.c_uint64, _VP, _VP]),
            "fc_graph_generate_graph500_edges": (ctypes.c_int, [_I32, _I64, ctypes.c_uint64,
                                                                ctypes.c_uint64, _VP, _VP, _VP]),
            "fc_bfs_trace": (ctypes.c_int, [_VP, _VP, _VP, _VP, _I32]),
            "fc_selftest_primitives": (ctypes.c_int, [_I32, _VP, _I32, _VP, _VP]),
            "fc_graph_info": (ctypes.c_int, [_VP, _VP, _VP, _VP]),
            "fc_graph_get_csr": (ctypes.c_int, [_VP, _VP, _VP]),
            "fc_graph_free": (None, [_VP]),
            "fc_bfs_levels": (ctypes.c_int, [_VP, _I32, _VP]),
            "fc_bfs_levels_ex": (ctypes.c_int, [_VP, _I32, _VP, _VP, _VP]),
            "fc_stcon": (ctypes.c_int, [_VP, _I32, _I32, _VP, _VP]),
            "fc_stcon_ex": (ctypes.c_int, [_VP, _I32, _I32, _VP, _VP, _VP, _VP]),
            "fc_stcon_depth": (ctypes.c_int, [_VP, _I32, _I32, _VP]),
            "fc_stcon_batch": (ctypes.c_int, [_VP, _I32, _VP, _VP, _VP, _I32, _VP, _VP, _VP, _VP]),
            "fc_stcon_batch_device": (ctypes.c_int, [_VP, _I32, _VP, _VP, _VP, _I32, _VP, _VP, _VP, _VP]),
            "fc_stcon_batch_noalloc": (ctypes.c_int, [_VP, _VP, _I32, _I64, _VP, _VP, _VP, _VP,
                                                      _I32, _VP, _VP, _I32, _VP]),
            "fc_sched_set_weights": (ctypes.c_int, [_VP, _I32]),
            "fc_sched_get_weights": (ctypes.c_int, [_VP, _I32]),
            "fc_mlp_loss_grad": (ctypes.c_int, [_VP, _VP, _VP, _I32, _VP, _VP, _VP]),
            "fc_mlp_train": (ctypes.c_int, [_VP, _VP, _VP, _I32, _I32, _I32, ctypes.c_float, _VP,
                                            _VP]),
            "fc_stcon_batch_scripted": (ctypes.c_int, [_VP, _VP, _VP, _I32, _VP, _I32, _VP, _VP,
                                                       _VP, _VP, _I32, _VP]),
            "fc_selftest_wait": (ctypes.c_int, [_I32, _VP]),
            "fc_bfs_parents": (ctypes.c_int, [_VP, _I32, _VP, _VP]),
            "fc_stcon_multiseed": (ctypes.c_int, [_VP, _I32, _I32, _I32, ctypes.c_uint64, _VP, _VP]),
            "fc_autotune_batch": (ctypes.c_int, [_VP, _I32, _VP, _VP, _VP, _I32, _I32, _VP, _VP]),
            "fc_parse_edgelist": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, _VP, _VP,
                                                 _I64, _VP, _VP, _VP]),
            "fc_stcon_path": (ctypes.c_int, [_VP, _I32, _I32, _VP, _I32, _VP]),
            "fc_validate_bfs": (ctypes.c_int, [_VP, _I32, _VP, _VP]),
            "fc_strerror": (ctypes.c_char_p, [ctypes.c_int]),
            "fc_last_error_message": (ctypes.c_char_p, []),
            "fc_device_info": (ctypes.c_int, [_VP, _VP, _VP, _VP]),
            "fc_version": (ctypes.c_int, []),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc: int, what: str):
    if rc != OK:
        L = lib()
        detail = L.fc_last_error_message().decode(errors="replace")
        raise FastconError(rc, f"{what}: {L.fc_strerror(rc).decode()}: {detail}")


def _P(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def make_opts(sched=SCHED_HEURISTIC, engine=ENGINE_AUTO, block=0, ctas_per_sm=0, use_graph=0,
              max_slots=0, stream=None, cta_work_k=0, variant=0, tile_entries=0,
              job_entries=0, private_variant=0, vertex_order=0, slot_log_cap=0) -> Opts:
    """variant: 0 = chosen by the schedule, 1 hybrid, 2 warp-centric, 3 lane per row;
    tile_entries / job_entries: work-sharing tile and row-job sizes (0 = defaults);
    vertex_order: numbering the search runs on (ORDER_AUTO / ORDER_GIVEN /
    ORDER_DEGREE): the plain BFS engine and s-t batches of undirected graphs
    (single queries only with ORDER_DEGREE); ids in and levels out are always
    the caller's; slot_log_cap: at most this many entries in each batch query
    slot's visit log (0 = as large as fits; at least 1,024)."""
    o = Opts()
    lib().fc_opts_init(ctypes.byref(o))
    o.sched, o.engine, o.block, o.ctas_per_sm = sched, engine, block, ctas_per_sm
    o.use_graph, o.max_slots = use_graph, max_slots
    o.stream = stream
    o.cta_work_k = cta_work_k
    o.variant = variant
    o.tile_entries, o.job_entries = tile_entries, job_entries
    o.private_variant = private_variant
    o.vertex_order = vertex_order
    o.slot_log_cap = slot_log_cap
    return o


class Graph:
    """Owner of one device CSR (fc_graph*)."""

    def __init__(self, handle: int):
        self._h = ctypes.c_void_p(handle)
        nv = np.zeros(1, np.int32)
        ne = np.zeros(1, np.int64)
        d = np.zeros(1, np.int32)
        _check(lib().fc_graph_info(self._h, _P(nv), _P(ne), _P(d)), "fc_graph_info")
        self.nv, self.ne, self.directed = int(nv[0]), int(ne[0]), bool(d[0])

    # -- construction -------------------------------------------------------
    @classmethod
    def _make(cls, fn, *args, what=""):
        h = ctypes.c_void_p()
        _check(fn(*args, ctypes.byref(h)), what)
        return cls(h.value)

    @classmethod
    def load_edgelist(cls, path: str, force_dir: int = -1, relabel: bool = False) -> "Graph":
        return cls._make(lib().fc_graph_load_edgelist, path.encode(), int(force_dir), int(relabel),
                         what="fc_graph_load_edgelist")

    @classmethod
    def from_csr(cls, row_ptr, col, directed: bool = False) -> "Graph":
        rp, c = _i32(row_ptr), _i32(col)
        return cls._make(lib().fc_graph_from_csr, _P(rp), len(rp) - 1, _P(c) if len(c) else None,
                         len(c), int(directed), what="fc_graph_from_csr")

    @classmethod
    def from_edges(cls, src, dst, nv: int, flags: int = 0) -> "Graph":
        s, d = _i32(src), _i32(dst)
        return cls._make(lib().fc_graph_from_edges, _P(s) if len(s) else None,
                         _P(d) if len(d) else None, len(s), int(nv), int(flags),
                         what="fc_graph_from_edges")

    @classmethod
    def from_device_edges(cls, src_ptr: int, dst_ptr: int, n: int, nv: int, flags: int = 0):
        return cls._make(lib().fc_graph_from_device_edges, ctypes.c_void_p(src_ptr),
                         ctypes.c_void_p(dst_ptr), int(n), int(nv), int(flags),
                         what="fc_graph_from_device_edges")

    @classmethod
    def rmat(cls, scale: int, nedges: int, a=0.57, b=0.19, c=0.19, seed: int = 3,
             perm_seed: int = -1) -> "Graph":
        return cls._make(lib().fc_graph_generate_rmat, int(scale), int(nedges), float(a), float(b),
                         float(c), int(seed), int(perm_seed), what="fc_graph_generate_rmat")

    @classmethod
    def graph500(cls, scale: int, nedges: int, seed1: int, seed2: int,
                 initiator=(0.57, 0.19, 0.19, 0.05)) -> "Graph":
        """The reference driver's Graph500 graph (make_graph), made on the device."""
        ini = np.ascontiguousarray(initiator, dtype=np.float64)
        return cls._make(lib().fc_graph_generate_graph500, int(scale), int(nedges), int(seed1),
                         int(seed2), _P(ini), what="fc_graph_generate_graph500")

    @classmethod
    def grid(cls, w: int, h: int, p_del=0.05, del_seed: int = 5, shortcuts: int = 0,
             sc_seed: int = 6) -> "Graph":
        return cls._make(lib().fc_graph_generate_grid, int(w), int(h), float(p_del), int(del_seed),
                         int(shortcuts), int(sc_seed), what="fc_graph_generate_grid")

    def free(self):
        if self._h:
            lib().fc_graph_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- data ---------------------------------------------------------------
    def csr(self):
        rp = np.zeros(self.nv + 1, np.int32)
        col = np.zeros(max(1, self.ne), np.int32)
        _check(lib().fc_graph_get_csr(self._h, _P(rp), _P(col)), "fc_graph_get_csr")
        return rp, col[: self.ne]

    def degrees(self):
        rp, _ = self.csr_row_ptr()
        return np.diff(rp)

    def csr_row_ptr(self):
        rp = np.zeros(self.nv + 1, np.int32)
        _check(lib().fc_graph_get_csr(self._h, _P(rp), None), "fc_graph_get_csr")
        return rp, None

    # -- queries ------------------------------------------------------------
    def bfs_levels(self, s: int, opts: Opts | None = None, stats: bool = False):
        lev = np.empty(self.nv, np.int32)
        st = Stats()
        _check(lib().fc_bfs_levels_ex(self._h, int(s), _P(lev),
                                      ctypes.byref(opts) if opts else None, ctypes.byref(st)),
               "fc_bfs_levels")
        return (lev, st.as_dict()) if stats else lev

    def stcon_multiseed(self, s: int, t: int, nseeds: int = 320, seed: int = 1,
                        stats: bool = False):
        """Connectivity only, by multi-seed region growth (undirected)."""
        c = np.zeros(1, np.int32)
        st = Stats()
        _check(lib().fc_stcon_multiseed(self._h, int(s), int(t), int(nseeds), int(seed), _P(c),
                                        ctypes.byref(st)), "fc_stcon_multiseed")
        return (bool(c[0]), st.as_dict()) if stats else bool(c[0])

    def bfs_parents(self, s: int, with_levels: bool = False):
        """Deterministic BFS tree (smallest-id parent one level closer)."""
        par = np.empty(self.nv, np.int32)
        lev = np.empty(self.nv, np.int32) if with_levels else None
        _check(lib().fc_bfs_parents(self._h, int(s), _P(par), _P(lev)), "fc_bfs_parents")
        return (par, lev) if with_levels else par

    def stcon_path(self, s: int, t: int):
        """A shortest s -> t path as a vertex array (empty if unreachable)."""
        n = np.zeros(1, np.int32)
        cap = 1 << 16
        while True:
            path = np.empty(cap, np.int32)
            rc = lib().fc_stcon_path(self._h, int(s), int(t), _P(path), cap, _P(n))
            if rc == ERR_OVERFLOW and n[0] > cap:
                cap = int(n[0])
                continue
            _check(rc, "fc_stcon_path")
            return path[:n[0]].copy()

    def validate_bfs(self, root: int, parents):
        """Graph500 validation counters of a predecessor map (see the header)."""
        par = np.ascontiguousarray(parents, dtype=np.int32)
        err = np.zeros(8, np.int64)
        _check(lib().fc_validate_bfs(self._h, int(root), _P(par), _P(err)), "fc_validate_bfs")
        return err

    def stcon(self, s: int, t: int, opts: Opts | None = None, stats: bool = False):
        c = np.zeros(1, np.int32)
        h = np.zeros(1, np.int32)
        st = Stats()
        _check(lib().fc_stcon_ex(self._h, int(s), int(t), _P(c), _P(h),
                                 ctypes.byref(opts) if opts else None, ctypes.byref(st)),
               "fc_stcon")
        r = (bool(c[0]), int(h[0]))
        return (r, st.as_dict()) if stats else r

    def stcon_depth(self, s: int, t: int) -> int:
        d = np.zeros(1, np.int32)
        _check(lib().fc_stcon_depth(self._h, int(s), int(t), _P(d)), "fc_stcon_depth")
        return int(d[0])


def stcon_batch(graphs, s, t, graph_idx=None, opts: Opts | None = None, stats: bool = False,
                out=None):
    """Many (s, t) queries over one or several graphs; host arrays in/out.
    out: optional (connected, hops) int32 arrays of at least len(s) entries to
    fill (page-locked ones keep the result copies asynchronous).  Statistics
    are gathered only when stats is true (they add a copy of per-query
    counters to the call)."""
    if isinstance(graphs, Graph):
        graphs = [graphs]
    arr = (ctypes.c_void_p * len(graphs))(*[g.handle.value for g in graphs])
    s, t = _i32(s), _i32(t)
    gi = _i32(graph_idx) if graph_idx is not None else None
    nq = len(s)
    if out is not None:
        conn, hops = out
        for a in (conn, hops):
            if a.dtype != np.int32 or not a.flags["C_CONTIGUOUS"] or len(a) < nq:
                raise ValueError("out arrays must be contiguous int32 of at least len(s) entries")
    else:
        conn = np.zeros(nq, np.int32)
        hops = np.zeros(nq, np.int32)
    st = Stats() if stats else None
    _check(lib().fc_stcon_batch(arr, len(graphs), _P(gi), _P(s), _P(t), nq, _P(conn), _P(hops),
                                ctypes.byref(opts) if opts else None,
                                ctypes.byref(st) if st is not None else None),
           "fc_stcon_batch")
    return (conn, hops, st.as_dict()) if stats else (conn, hops)


def stcon_batch_device(graphs, s_ptr, t_ptr, nq, conn_ptr, hops_ptr, graph_idx_ptr=None,
                       opts: Opts | None = None, stats: bool = False):
    """Device-pointer variant (inputs resident in HBM; pointers as ints)."""
    if isinstance(graphs, Graph):
        graphs = [graphs]
    arr = (ctypes.c_void_p * len(graphs))(*[g.handle.value for g in graphs])
    st = Stats()
    _check(lib().fc_stcon_batch_device(arr, len(graphs),
                                       ctypes.c_void_p(graph_idx_ptr) if graph_idx_ptr else None,
                                       ctypes.c_void_p(s_ptr), ctypes.c_void_p(t_ptr), int(nq),
                                       ctypes.c_void_p(conn_ptr), ctypes.c_void_p(hops_ptr),
                                       ctypes.byref(opts) if opts else None,
                                       ctypes.byref(st) if stats else None),
           "fc_stcon_batch_device")
    return st.as_dict() if stats else None


def autotune_batch(graphs, s_ptr, t_ptr, nq, graph_idx_ptr=None, opts: Opts | None = None,
                   reps: int = 3):
    """Pick the fastest batched-engine settings on a sample batch (device
    pointers).  Returns (opts, best_ms)."""
    if isinstance(graphs, Graph):
        graphs = [graphs]
    arr = (ctypes.c_void_p * len(graphs))(*[g.handle.value for g in graphs])
    o = Opts()
    if opts is not None:
        ctypes.memmove(ctypes.byref(o), ctypes.byref(opts), ctypes.sizeof(Opts))
    else:
        lib().fc_opts_init(ctypes.byref(o))
    ms = np.zeros(1, np.float64)
    _check(lib().fc_autotune_batch(arr, len(graphs),
                                   ctypes.c_void_p(graph_idx_ptr) if graph_idx_ptr else None,
                                   ctypes.c_void_p(s_ptr), ctypes.c_void_p(t_ptr), int(nq), int(reps),
                                   ctypes.byref(o), _P(ms)), "fc_autotune_batch")
    return o, float(ms[0])


def parse_edgelist(path: str, relabel: bool = False, nthreads: int = 0):
    """Host-side parse of an edge-list file: (nv, src, dst, file_directed)."""
    n = np.zeros(1, np.int64)
    nv = np.zeros(1, np.int32)
    fd = np.zeros(1, np.int32)
    cap = 0
    src = dst = None
    while True:
        rc = lib().fc_parse_edgelist(path.encode(), int(bool(relabel)), int(nthreads), _P(src),
                                     _P(dst), cap, _P(n), _P(nv), _P(fd))
        if rc == ERR_OVERFLOW and n[0] > cap:
            cap = int(n[0])
            src = np.empty(cap, np.int32)
            dst = np.empty(cap, np.int32)
            continue
        _check(rc, "fc_parse_edgelist")
        k = int(n[0])
        if src is None:
            src = dst = np.empty(0, np.int32)
        return int(nv[0]), src[:k].copy(), dst[:k].copy(), int(fd[0])


def selftest_wait(timeout_ms: int = 200):
    """Run the bounded-wait self-test; returns (status code, kernel ms)."""
    ms = np.zeros(1, np.float64)
    rc = lib().fc_selftest_wait(int(timeout_ms), _P(ms))
    return rc, float(ms[0])


def bfs_trace(cap: int = 256):
    """Per-level trace of the last plain-BFS-engine search on this device:
    dict of level_ns, frontier, entries (numpy int64 arrays)."""
    n = ctypes.c_int32()
    ns = np.zeros(cap, np.int64)
    fr = np.zeros(cap, np.int64)
    en = np.zeros(cap, np.int64)
    _check(lib().fc_bfs_trace(ctypes.byref(n), _P(ns), _P(fr), _P(en), int(cap)), "fc_bfs_trace")
    k = min(n.value, cap)
    return {"levels": n.value, "level_ns": ns[:k], "frontier": fr[:k], "entries": en[:k]}


def graph500_edges(scale: int, nedges: int, seed1: int, seed2: int,
                   initiator=(0.57, 0.19, 0.19, 0.05)):
    """Raw edge list of the Graph500 generator (device), int32 (src, dst)."""
    ini = np.ascontiguousarray(initiator, dtype=np.float64)
    src = np.zeros(nedges, np.int32)
    dst = np.zeros(nedges, np.int32)
    _check(lib().fc_graph_generate_graph500_edges(int(scale), int(nedges), int(seed1), int(seed2),
                                                  _P(ini), _P(src), _P(dst)),
           "fc_graph_generate_graph500_edges")
    return src, dst


def selftest_primitives(which: int, data):
    """Run one of the library's primitives on `data` (see fc_selftest_primitives):
    returns (out, aux)."""
    a = _i32(data)
    n = len(a)
    if which == 2:
        out = np.zeros(max(1, int(a.sum())), np.int32)
    else:
        out = np.zeros(max(1, n), np.int32)
    aux = np.zeros(max(1, (n + 255) // 256), np.int32)
    _check(lib().fc_selftest_primitives(int(which), _P(a) if n else None, n, _P(out), _P(aux)),
           "fc_selftest_primitives")
    if which == 2:
        return out[: int(a.sum())], aux
    return out[:n], aux


def device_info():
    sm = np.zeros(1, np.int32)
    mem = np.zeros(1, np.int64)
    ma = np.zeros(1, np.int32)
    mi = np.zeros(1, np.int32)
    _check(lib().fc_device_info(_P(sm), _P(mem), _P(ma), _P(mi)), "fc_device_info")
    return {"sm_count": int(sm[0]), "total_mem": int(mem[0]), "cc": (int(ma[0]), int(mi[0]))}
