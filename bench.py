"""Benchmark: batched s-t connectivity on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl fastcon|reference]
                    [--config rmat24|rmat22|er65536|grid4096|batched512] [--sched heuristic|plain|learned]
    python bench.py --bfs plain|heuristic [--engine hostloop|persistent] [--config ...]

Default workload (rmat24): R-MAT scale 24 (16,777,216 vertices; 8 * 2^24 edge
samples with a/b/c/d = .57/.19/.19/.05 -> average degree ~16 after
symmetrisation and deduplication; ids permuted, seed 3), 1,024 (s, t) pairs
among vertices of degree >= 1 (seed 4).  One step = all queries of the
workload through the library's batched engine.  The rmat24, grid4096 and
batched512 graphs are larger than L2, so no L2 flush is added between steps.

The headline schedule is the learned one (the metric's "learned+batched");
`schedules` in the printed line gives plain, heuristic and learned on the same
workload.

Printed line (rank 0): value = queries/s with inputs resident in HBM (CUDA
events on the launching stream); e2e = the same through fc_stcon_batch with
pinned host arrays (copies inside the timed region); roofline of the
dominant kernel (algorithmic bytes per launch / its CUDA-event time); cpu_baseline =
the reference's CPU path (one full BFS per query, Graph::bfs semantics) on the
host cores; plain = the plain level-synchronous GPU form (host-driven,
alternating sides, top-down) on a sample; one_launch_per_query = the library's
single-query call in a loop on a sample.

--impl reference times the reference's CPU path alone (rank 0) on bounded
samples of the same workload and prints the same metric with impl=reference.
Multi-GPU: queries do not exchange data, so N ranks run N independent
replicas (one per GPU) and value sums them (scaling = weak).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "fast-con_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "ST-CON queries/s & GTEPS: learned+batched vs plain on 1 GB300, exact answers"
UNIT = "queries/s"

CONFIGS = {
    "rmat24": dict(kind="rmat", scale=24, edge_samples=8 << 24, seed=3, perm_seed=3, nq=1024,
                   qseed=4),
    "er65536": dict(kind="er", n=65536, m=524288, seed=1, nq=64, qseed=2),
    "grid4096": dict(kind="grid", w=4096, h=4096, p_del=0.05, del_seed=5, sc_seed=6, nq=256,
                     qseed=7, min_manhattan=2000),
    "batched512": dict(kind="multi", ngraphs=512, first_seed=100, per_graph=8),
    # smaller R-MATs (same parameters) used for profiler captures
    "rmat22": dict(kind="rmat", scale=22, edge_samples=8 << 22, seed=3, perm_seed=3, nq=1024,
                   qseed=4),
    "rmat21": dict(kind="rmat", scale=21, edge_samples=8 << 21, seed=3, perm_seed=3, nq=1024,
                   qseed=4),
}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region (read only)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            time.sleep(0.3)  # let the sampler start before the timed region
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.15)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def reduce_over_ranks(ws, x: float, op: str) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------------------
# workloads: (graphs, graph index per query or None, s, t)
# ---------------------------------------------------------------------------
def multi_specs(cfg):
    from fastcon import graphs
    scales = graphs.batched_scales(cfg["ngraphs"], cfg["first_seed"])
    return [(cfg["first_seed"] + i, sc) for i, sc in enumerate(scales)]


def make_workload_gpu(fc, cfg):
    from fastcon import graphs
    if cfg["kind"] == "rmat":
        G = fc.Graph.rmat(cfg["scale"], cfg["edge_samples"], seed=cfg["seed"],
                          perm_seed=cfg["perm_seed"])
        rp, _ = G.csr_row_ptr()
        s, t = graphs.pairs_with_degree(np.diff(rp), cfg["nq"], seed=cfg["qseed"])
        return [G], None, s, t
    if cfg["kind"] == "er":
        u, v = graphs.er_edges(cfg["n"], cfg["m"], seed=cfg["seed"])
        G = fc.Graph.from_edges(u, v, cfg["n"])
        s, t = graphs.uniform_pairs(cfg["n"], cfg["nq"], seed=cfg["qseed"])
        return [G], None, s, t
    if cfg["kind"] == "grid":
        n = cfg["w"] * cfg["h"]
        G = fc.Graph.grid(cfg["w"], cfg["h"], p_del=cfg["p_del"], del_seed=cfg["del_seed"],
                          shortcuts=graphs.grid_shortcut_count(n), sc_seed=cfg["sc_seed"])
        s, t = graphs.grid_pairs(cfg["w"], cfg["h"], cfg["nq"], cfg["qseed"], cfg["min_manhattan"])
        return [G], None, s, t
    Gs, ss, ts, gi = [], [], [], []
    for k, (seed, scale) in enumerate(multi_specs(cfg)):
        G = fc.Graph.rmat(scale, 8 << scale, seed=seed, perm_seed=seed)
        rp, _ = G.csr_row_ptr()
        s, t = graphs.pairs_with_degree(np.diff(rp), cfg["per_graph"], seed=seed)
        Gs.append(G)
        ss.append(s)
        ts.append(t)
        gi.append(np.full(len(s), k, np.int32))
    return Gs, np.concatenate(gi), np.concatenate(ss), np.concatenate(ts)


def make_workload_cpu(cfg, nthreads, only_graphs=None):
    """Host CSRs for the CPU arm, built without any GPU code (oracle C)."""
    import oracle
    from fastcon import graphs
    if cfg["kind"] == "rmat":
        n = 1 << cfg["scale"]
        u, v = oracle.gen_rmat(cfg["scale"], cfg["edge_samples"], seed=cfg["seed"],
                               perm_seed=cfg["perm_seed"], nthreads=nthreads)
        rp, col = oracle.build_csr(n, u, v, nthreads=nthreads)
        del u, v
        s, t = graphs.pairs_with_degree(np.diff(rp), cfg["nq"], seed=cfg["qseed"])
        return [(rp, col)], None, s, t
    if cfg["kind"] == "er":
        u, v = graphs.er_edges(cfg["n"], cfg["m"], seed=cfg["seed"])
        rp, col = oracle.build_csr(cfg["n"], u, v, nthreads=nthreads)
        s, t = graphs.uniform_pairs(cfg["n"], cfg["nq"], seed=cfg["qseed"])
        return [(rp, col)], None, s, t
    if cfg["kind"] == "grid":
        n = cfg["w"] * cfg["h"]
        u, v = graphs.grid_edges(cfg["w"], cfg["h"], cfg["p_del"], cfg["del_seed"],
                                 graphs.grid_shortcut_count(n), cfg["sc_seed"])
        rp, col = oracle.build_csr(n, u, v, nthreads=nthreads)
        s, t = graphs.grid_pairs(cfg["w"], cfg["h"], cfg["nq"], cfg["qseed"], cfg["min_manhattan"])
        return [(rp, col)], None, s, t
    csrs, ss, ts, gi = [], [], [], []
    for k, (seed, scale) in enumerate(multi_specs(cfg)):
        if only_graphs is not None and k not in only_graphs:
            csrs.append(None)
            continue
        u, v = oracle.gen_rmat(scale, 8 << scale, seed=seed, perm_seed=seed, nthreads=nthreads)
        rp, col = oracle.build_csr(1 << scale, u, v, nthreads=nthreads)
        s, t = graphs.pairs_with_degree(np.diff(rp), cfg["per_graph"], seed=seed)
        csrs.append((rp, col))
        ss.append(s)
        ts.append(t)
        gi.append(np.full(len(s), k, np.int32))
    return csrs, np.concatenate(gi), np.concatenate(ss), np.concatenate(ts)


def cpu_queries(csrs, gi, s, t, idx, nthreads, with_conn=False):
    """Run queries idx with the reference's CPU path (full BFS per query):
    hops, or (connected, hops) with with_conn."""
    import oracle
    conn = np.zeros(len(idx), np.int32)
    hops = np.zeros(len(idx), np.int32)
    if gi is None:
        rp, col = csrs[0]
        c, h, _ = oracle.stcon_batch(rp, col, s[idx], t[idx], nthreads=nthreads)
        return (c, h) if with_conn else h
    for g in np.unique(gi[idx]):
        m = gi[idx] == g
        rp, col = csrs[g]
        c, h, _ = oracle.stcon_batch(rp, col, s[idx][m], t[idx][m], nthreads=nthreads)
        conn[m] = c
        hops[m] = h
    return (conn, hops) if with_conn else hops


def cpu_single_thread(csrs, gi, s, t, min_seconds=6.0, max_queries=8):
    """The same CPU path on one thread, a few queries of the workload."""
    done, t0 = 0, time.perf_counter()
    while True:
        cpu_queries(csrs, gi, s, t, np.array([done % len(s)]), 1)
        done += 1
        el = time.perf_counter() - t0
        if el >= min_seconds or done >= max_queries:
            break
    return {"value": done / el, "unit": UNIT, "cores": 1, "sample": f"{done} queries ({el:.1f} s)"}


def cpu_model():
    """CPU model name of the host (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


def same_csr(G, csr):
    """Device CSR of G equal to the oracle's CSR of the same graph."""
    if csr is None:
        return True
    rp, col = G.csr()
    return bool(len(rp) == len(csr[0]) and (rp == csr[0]).all() and len(col) == len(csr[1])
                and (col == csr[1]).all())


def plain_bfs_block(fc, G, peak, nsrc=4, reps=5):
    """Plain expansion: full level-synchronous top-down BFS of G (the plain
    schedule, the library's default BFS engine) from nsrc sources next to
    the three-quarter point of the degree order; device time per call from
    the library's CUDA events.  Algorithmic bytes = 8 per adjacency entry
    read + 20 per reached vertex (the library's statistics), so frac is the
    effective-byte fraction of the HBM peak."""
    rp, _ = G.csr_row_ptr()
    deg = np.diff(rp)
    order = np.argsort(deg, kind="stable")
    srcs = [int(order[len(deg) // 2 + len(deg) // 4 + k]) for k in range(nsrc)]
    o = fc.make_opts(sched=fc.SCHED_PLAIN)
    for _ in range(2):
        G.bfs_levels(srcs[0], o)
    per = []
    tot_ms, tot_bytes, tot_entries = 0.0, 0, 0
    lev0 = None
    for src in srcs:
        ms = []
        for _ in range(reps):
            lev, st = G.bfs_levels(src, o, stats=True)
            ms.append(st["gpu_ms"])
        if lev0 is None:
            lev0 = lev
        m = statistics.median(ms)
        tot_ms += m
        tot_bytes += st["alg_bytes"]
        tot_entries += st["edges_inspected"]
        per.append({"source": src, "ms": m, "levels": int(lev.max()) + 1,
                    "entries": int(st["edges_inspected"]), "reached": int((lev >= 0).sum())})
    achieved = tot_bytes / 1e9 / (tot_ms / 1e3)
    # DRAM bytes of the search: a small-case ncu capture of the same kernel,
    # scaled by the algorithmic bytes (both grow per entry and per vertex)
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic_per_unit.json")
    if os.path.exists(tp):
        ratio = json.load(open(tp)).get("k_bfs_plain", {}).get("dram_bytes_per_alg_byte")
        if ratio:
            traffic = float(ratio) * tot_bytes / len(srcs)
    return {"form": "full BFS, plain schedule (level-synchronous, top-down), library default engine",
            "kernel": "k_bfs_plain",
            "ms": tot_ms / len(srcs), "alg_bytes": tot_bytes / len(srcs),
            "achieved_gbs": achieved, "peak": peak, "frac": achieved / peak,
            "traffic": traffic,
            "traffic_source": "profiles/traffic_per_unit.json (scaled small-case capture)",
            "gteps_entries": tot_entries / (tot_ms * 1e6), "sources": per,
            "bytes_rule": "8 per adjacency entry read + 20 per reached vertex",
            "_source": srcs[0], "_levels": lev0}


def ka16_block(fc):
    """The reference's only published ST-CON run, replayed: Graph500 R-MAT
    scale 16 (seeds 670021781 / 1422323141) and its 100 (RED-V, BLUE-V)
    pairs, as the reference ran them (one query per call, DEPTH =
    ceil(hops / 2), make_stcon's answer) and batched."""
    gdir = os.path.join(ROOT, "tests", "golden")
    z = np.load(os.path.join(gdir, "rmat16_graph500_edges.npz"))
    u = np.cumsum(z["du"].astype(np.int64)).astype(np.int32)
    v = z["v"].astype(np.int32)
    ka = json.load(open(os.path.join(gdir, "stcon_known_answer.json")))
    rows = ka["rows"]
    red = np.array([r["red"] for r in rows], np.int32)
    blue = np.array([r["blue"] for r in rows], np.int32)
    depth_ref = np.array([r["depth"] for r in rows], np.int32)
    G = fc.Graph.from_edges(u, v, 1 << 16)
    for k in range(10):
        G.stcon_depth(int(red[k]), int(blue[k]))
    t0 = time.perf_counter()
    depth = np.array([G.stcon_depth(int(a), int(b)) for a, b in zip(red, blue)], np.int32)
    single_s = time.perf_counter() - t0
    fc.stcon_batch(G, red, blue)
    t0 = time.perf_counter()
    reps = 20
    for _ in range(reps):
        conn, hops = fc.stcon_batch(G, red, blue)
    batch_s = (time.perf_counter() - t0) / reps
    bdepth = np.where(conn != 0, (hops + 1) // 2, -1)
    G.free()
    return {"workload": "Graph500 R-MAT scale 16, edgefactor 16, 100 (RED-V, BLUE-V) pairs of "
                        "the reference's logged run",
            "single_query": {"ms_per_query": 1000 * single_s / len(red),
                             "conps": len(red) / single_s,
                             "form": "fc_stcon_depth per query from Python, host to host"},
            "batched": {"queries_per_s": len(red) / batch_s,
                        "form": "fc_stcon_batch of the 100 pairs, host arrays"},
            "depth_match": f"{int((depth == depth_ref).sum())}/{len(red)}",
            "batched_depth_match": f"{int((bdepth == depth_ref).sum())}/{len(red)}",
            "published": {"ms_per_query": 0.57856, "conps": 1756.99, "hardware": "RTX 2070",
                          "source": "bernaschi/ST_CONN_ONE_ATOMIC/current-st/st-conn/data/"
                                    "st_stats_20200418_140644:112-116"}}


def cpu_rate(csrs, gi, s, t, nthreads, min_seconds=10.0, max_queries=None, order=None):
    nq = len(s)
    order = np.arange(nq) if order is None else order
    done = 0
    t0 = time.perf_counter()
    while True:
        idx = order[np.arange(done, done + nthreads) % len(order)]
        cpu_queries(csrs, gi, s, t, idx, nthreads)
        done += len(idx)
        el = time.perf_counter() - t0
        if el >= min_seconds or (max_queries and done >= max_queries):
            break
    return done / el, done, el


def config_desc(name, cfg, nq):
    d = {"workload": name, "queries": nq}
    if cfg["kind"] == "rmat":
        d.update({"graph": f"R-MAT scale {cfg['scale']}, {cfg['edge_samples']} edge samples "
                           "(edge factor 16 counted as average degree), a/b/c/d=.57/.19/.19/.05, "
                           f"ids permuted (seed {cfg['perm_seed']})",
                  "query_seed": cfg["qseed"], "l2": "inputs larger than L2 (CSR > 126 MB)"})
    elif cfg["kind"] == "er":
        d.update({"graph": f"G(n,m) n={cfg['n']} m={cfg['m']} seed {cfg['seed']}",
                  "l2": "graph fits in L2 (small config)"})
    elif cfg["kind"] == "grid":
        d.update({"graph": f"{cfg['w']}x{cfg['h']} grid, {cfg['p_del']:.0%} edges deleted "
                           "(seed 5), 0.01% n shortcuts (seed 6)",
                  "min_manhattan": cfg["min_manhattan"], "l2": "inputs larger than L2"})
    else:
        d.update({"graph": f"{cfg['ngraphs']} R-MAT graphs, scale uniform in [12,20], 8*2^scale "
                           f"samples each, seeds {cfg['first_seed']}..{cfg['first_seed'] + cfg['ngraphs'] - 1}",
                  "l2": "inputs larger than L2"})
    return d


# ---------------------------------------------------------------------------
# reference arm (CPU only)
# ---------------------------------------------------------------------------
def run_reference(args, cfg):
    ws, rank, _ = dist_env()
    if ws > 1 and rank != 0:
        return
    nthreads = os.cpu_count() or 1
    only = None
    if cfg["kind"] == "multi":
        only = set(range(0, cfg["ngraphs"], 16))  # bounded sample of graphs
    csrs, gi, s, t = make_workload_cpu(cfg, nthreads, only)
    per_step = max(nthreads, 32)
    order = np.arange(len(s)) if gi is None else np.flatnonzero(np.isin(gi, list(only)))
    el_total, q_total, k = 0.0, 0, 0
    for i in range(args.warmup + args.steps):
        idx = order[np.arange(i * per_step, (i + 1) * per_step) % len(order)]
        t0 = time.perf_counter()
        cpu_queries(csrs, gi, s, t, idx, nthreads)
        el = time.perf_counter() - t0
        if i >= args.warmup:
            el_total += el
            q_total += len(idx)
            k += 1
    value = q_total / el_total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * el_total / k,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic", "config": config_desc(args.config, cfg, len(s)),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": f"{per_step} queries of the workload per step, one full BFS "
                                   f"from s per query (Graph::bfs restated in oracle/fc_oracle.c), "
                                   f"{nthreads} threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_fastcon(args, cfg):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import fastcon as fc

    sched = {"heuristic": fc.SCHED_HEURISTIC, "plain": fc.SCHED_PLAIN,
             "learned": fc.SCHED_LEARNED}[args.sched]
    from fastcon import learn
    learned_ready = os.path.exists(learn.WEIGHTS_PATH)
    if learned_ready:
        learn.load_default_weights()
    elif args.sched == "learned":
        raise SystemExit("learned schedule asked for but no weights at " + learn.WEIGHTS_PATH)
    Gs, gi, s, t = make_workload_gpu(fc, cfg)
    nq = len(s)
    # a dedicated stream: the library launches on it and the events record on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    # repeated batches of one shape: the library replays one captured CUDA
    # graph per batch (use_graph), as a serving loop would
    opt = fc.make_opts(sched=sched, engine=fc.ENGINE_BATCHED, stream=stream.cuda_stream,
                       use_graph=1, max_slots=args.max_slots)
    d_s = torch.from_numpy(s).cuda()
    d_t = torch.from_numpy(t).cuda()
    d_g = torch.from_numpy(gi).cuda() if gi is not None else None
    d_c = torch.empty(nq, dtype=torch.int32, device="cuda")
    d_h = torch.empty(nq, dtype=torch.int32, device="cuda")
    gptr = d_g.data_ptr() if d_g is not None else None

    def step(stats=False):
        return fc.stcon_batch_device(Gs, d_s.data_ptr(), d_t.data_ptr(), nq, d_c.data_ptr(),
                                     d_h.data_ptr(), graph_idx_ptr=gptr, opts=opt, stats=stats)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    hops_gpu = d_h.cpu().numpy()

    clocks = ClockSampler(local)
    barrier(ws)
    torch.cuda.synchronize()
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(ws)
    ms = reduce_over_ranks(ws, e0.elapsed_time(e1), "max")
    total_q = reduce_over_ranks(ws, float(nq * args.steps), "sum")
    value = total_q / (ms / 1000.0)

    # per-kernel split and algorithmic bytes (same workload, statistics on)
    kms, kbytes, ins, esc, launches, vadj = np.zeros(2), np.zeros(2), 0, 0, 0, 0
    for _ in range(args.steps):
        st = step(stats=True)
        kms += np.array(st["kernel_ms"])
        kbytes += np.array(st["kernel_alg_bytes"])
        ins += st["edges_inspected"]
        vadj += st["visited_adjacency"]
        esc = st["escalated"]
        launches = st["launches"]
    kms /= args.steps
    kbytes /= args.steps
    dom = int(np.argmax(kms))
    peak, peak_src = peaks()
    achieved = (kbytes[dom] / 1e9) / (kms[dom] / 1e3) if kms[dom] > 0 else 0.0
    # DRAM traffic per launch: an ncu capture of a smaller case of the same
    # kernel, scaled by the algorithmic bytes this launch processes
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic_per_unit.json")
    if os.path.exists(tp):
        ratio = json.load(open(tp)).get("k_pool", {}).get("dram_bytes_per_alg_byte")
        if ratio:
            traffic = float(ratio) * float(kbytes[dom])
    # the same launch in DRAM bytes: scaled traffic over the kernel's time
    achieved_dram = (traffic / 1e9) / (kms[dom] / 1e3) if traffic and kms[dom] > 0 else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "achieved_dram": achieved_dram,
                "dram_frac": achieved_dram / peak if achieved_dram else None,
                "traffic_source": "profiles/traffic_per_unit.json (scaled small-case capture)",
                "kernel": "k_pool" + (" (shared-work pass)" if dom == 0 else " (exclusive pass)"),
                "peak_source": f"{peak_src} hbm_gbs (MEASURED_PEAKS.json)",
                "kernel_ms": kms.tolist(), "kernel_alg_bytes": kbytes.tolist(),
                "escalated_queries": esc}

    # every schedule on the same device-resident workload (CUDA events)
    schedules = {}
    for name, sc in (("plain", fc.SCHED_PLAIN), ("heuristic", fc.SCHED_HEURISTIC),
                     ("learned", fc.SCHED_LEARNED)):
        if sc == fc.SCHED_LEARNED and not learned_ready:
            continue
        so = fc.make_opts(sched=sc, engine=fc.ENGINE_BATCHED, stream=stream.cuda_stream)
        for _ in range(max(3, args.warmup)):
            fc.stcon_batch_device(Gs, d_s.data_ptr(), d_t.data_ptr(), nq, d_c.data_ptr(),
                                  d_h.data_ptr(), graph_idx_ptr=gptr, opts=so)
        k = max(3, min(args.steps, 10))
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a0.record(stream)
        for _ in range(k):
            fc.stcon_batch_device(Gs, d_s.data_ptr(), d_t.data_ptr(), nq, d_c.data_ptr(),
                                  d_h.data_ptr(), graph_idx_ptr=gptr, opts=so)
        a1.record(stream)
        torch.cuda.synchronize()
        sms = a0.elapsed_time(a1) / k
        schedules[name] = {"value": nq / (sms / 1000.0), "unit": UNIT, "ms_per_step": sms,
                           "exact": bool((d_h.cpu().numpy() == hops_gpu).all())}

    # e2e: host arrays (pinned), copies inside the timed region
    hs = torch.from_numpy(s).pin_memory().numpy()
    ht = torch.from_numpy(t).pin_memory().numpy()
    hg = torch.from_numpy(gi).pin_memory().numpy() if gi is not None else None
    # results land in page-locked host arrays allocated once, like the inputs
    hc = torch.empty(nq, dtype=torch.int32).pin_memory().numpy()
    hh = torch.empty(nq, dtype=torch.int32).pin_memory().numpy()
    e2e_opt = fc.make_opts(sched=sched, engine=fc.ENGINE_BATCHED, use_graph=1)
    fc.stcon_batch(Gs, hs, ht, graph_idx=hg, opts=e2e_opt, out=(hc, hh))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        conn, hops = fc.stcon_batch(Gs, hs, ht, graph_idx=hg, opts=e2e_opt, out=(hc, hh))
    e2e_s = reduce_over_ranks(ws, time.perf_counter() - t0, "max")
    e2e = {"value": total_q / e2e_s, "unit": UNIT, "h2d_bytes_per_step": (8 if gi is None else 12) * nq,
           "d2h_bytes_per_step": 8 * nq}
    exact = bool((hops == hops_gpu).all()) and all(v["exact"] for v in schedules.values())

    # plain level-synchronous form and one-launch-per-query form, on samples
    plain_n = min(nq, 128 if cfg["kind"] != "grid" else 16)
    samp = np.arange(plain_n) * max(1, nq // plain_n)
    popt = fc.make_opts(sched=fc.SCHED_PLAIN, engine=fc.ENGINE_HOSTLOOP)
    t0 = time.perf_counter()
    pc, ph = fc.stcon_batch(Gs, s[samp], t[samp], graph_idx=None if gi is None else gi[samp],
                            opts=popt)
    plain_s = time.perf_counter() - t0
    exact = exact and bool((ph == hops_gpu[samp]).all())
    plain = {"value": plain_n / plain_s, "unit": UNIT, "sample": plain_n,
             "form": "host loop, one launch per level, alternating sides, top-down"}
    sopt = fc.make_opts(sched=sched)
    t0 = time.perf_counter()
    for k in samp:
        c1, h1 = Gs[0 if gi is None else gi[k]].stcon(int(s[k]), int(t[k]), sopt)
        exact = exact and h1 == hops_gpu[k]
    single_s = time.perf_counter() - t0
    single = {"value": plain_n / single_s, "unit": UNIT, "sample": plain_n,
              "form": "fc_stcon per query (one persistent launch each)"}

    # plain expansion: one full top-down BFS of the workload's graph
    plain_bfs = plain_bfs_block(fc, Gs[0], peak) if gi is None else None
    # the reference's only published run, replayed (Graph500 R-MAT 16)
    ka16 = ka16_block(fc)

    if rank == 0:
        cpu = None
        oracle_check = None
        if ws == 1:
            nthreads = os.cpu_count() or 1
            # every answer of this very workload against the oracle (outside
            # the timed region), on a CSR the oracle builds itself from the
            # same generator -- so the device ingest is checked too
            t0 = time.perf_counter()
            csrs, gi_c, s_c, t_c = make_workload_cpu(cfg, nthreads)
            build_s = time.perf_counter() - t0
            csr_match = all(same_csr(G, c) for G, c in zip(Gs, csrs))
            csr_match = csr_match and bool((s_c == s).all() and (t_c == t).all())
            conn_gpu = d_c.cpu().numpy()
            t0 = time.perf_counter()
            want_c, want_h = cpu_queries(csrs, gi, s, t, np.arange(nq), nthreads, with_conn=True)
            el = time.perf_counter() - t0
            mism = int(((hops_gpu != want_h) | (conn_gpu != want_c)).sum())
            exact = exact and mism == 0
            oracle_check = {"checked": f"{nq}/{nq}", "mismatches": mism, "csr_match": csr_match,
                            "oracle": "Graph::bfs restated in oracle/fc_oracle.c, one full BFS "
                                      "from s per query, on the oracle's own CSR",
                            "oracle_csr_build_s": round(build_s, 1)}
            if plain_bfs is not None:
                src = plain_bfs.pop("_source")
                lev_gpu = plain_bfs.pop("_levels")
                import oracle
                lev_cpu, _ = oracle.bfs_levels(csrs[0][0], csrs[0][1], src)
                plain_bfs["levels_exact"] = bool((lev_gpu == lev_cpu).all())
                exact = exact and plain_bfs["levels_exact"]
            one = cpu_single_thread(csrs, gi, s, t)
            cpu = {"value": nq / el, "unit": UNIT, "cores": nthreads, "kind": "port",
                   "sample": f"all {nq} queries of the workload ({el:.1f} s), one full BFS from s "
                             "per query (Graph::bfs restated in oracle/fc_oracle.c)",
                   "cpu_model": cpu_model(), "single_thread": one}
        elif plain_bfs is not None:
            plain_bfs.pop("_source")
            plain_bfs.pop("_levels")
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": dict(config_desc(args.config, cfg, nq), engine="batched",
                           sched=args.sched, parallelism=f"replicas{ws}"),
            "exact": exact, "oracle_check": oracle_check,
            "gteps_inspected": ins / args.steps / (ms / args.steps / 1000.0) / 1e9,
            "edges_inspected_per_step": ins / args.steps,
            # the reference's TEPS numerator (count_visited_edges, S/adj_func.c:334-357)
            # counts every edge of every visited vertex, almost none of which an
            # early-exit search reads: context only, not a speed
            "visited_edges_convention": {
                "gteps": vadj / 2 / args.steps / (ms / args.steps / 1000.0) / 1e9,
                "note": "edges of the visited vertices per second (Graph500 count_visited_edges); "
                        "most were never read"},
            "plain_bfs": plain_bfs, "ka16": ka16,
            "plain": plain, "one_launch_per_query": single, "schedules": schedules,
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
            "gpu_launches": launches * args.steps,
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_bfs(args, cfg):
    """One full BFS of the workload's (first) graph from the vertex at three
    quarters of the degree order (a hub-connected source), --warmup untimed and
    --steps timed calls; prints level sizes and the fastest call's device time.
    The small case that the per-level ncu summaries profile."""
    import torch
    torch.cuda.set_device(0)
    import fastcon as fc
    Gs, _, _, _ = make_workload_gpu(fc, cfg)
    G = Gs[0]
    rp, _ = G.csr_row_ptr()
    deg = np.diff(rp)
    src = int(np.argsort(deg)[len(deg) // 2 + len(deg) // 4])
    o = fc.make_opts(sched=fc.SCHED_PLAIN if args.bfs == "plain" else fc.SCHED_HEURISTIC,
                     engine={"hostloop": fc.ENGINE_HOSTLOOP, "persistent": fc.ENGINE_PERSISTENT,
                             "auto": fc.ENGINE_AUTO}[args.engine],
                     vertex_order={"auto": fc.ORDER_AUTO, "given": fc.ORDER_GIVEN,
                                   "degree": fc.ORDER_DEGREE}[args.order],
                     ctas_per_sm=args.ctas)
    ms = []
    for k in range(args.warmup + args.steps):
        lev, st = G.bfs_levels(src, o, stats=True)
        if k >= args.warmup:
            ms.append(st["gpu_ms"])
    reached = lev >= 0
    entries = int(deg[reached].sum())
    trace = None
    if args.bfs == "plain" and args.engine == "auto":
        tr = fc.bfs_trace()
        trace = {"level_us": (tr["level_ns"] / 1e3).round(1).tolist(),
                 "frontier": tr["frontier"].tolist(), "entries": tr["entries"].tolist()}
    print(json.dumps({"bfs": args.bfs, "engine": args.engine, "order": args.order,
                      "ctas": args.ctas, "trace": trace,
                      "workload": args.config,
                      "source": src, "levels": np.bincount(lev[reached]).tolist(),
                      "ms": min(ms), "entries_inspected": int(st["edges_inspected"]),
                      "gteps_entries": entries / (min(ms) * 1e6)}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="fastcon", choices=["fastcon", "reference"])
    ap.add_argument("--config", default="rmat24", choices=sorted(CONFIGS))
    ap.add_argument("--sched", default="learned", choices=["heuristic", "plain", "learned"])
    ap.add_argument("--max-slots", type=int, default=0,
                    help="cap on the batch's concurrent query slots (0 = all resident CTAs); "
                         "small profiler captures only")
    ap.add_argument("--bfs", default=None, choices=["plain", "heuristic"],
                    help="time one full BFS of the workload's graph instead of the batch")
    ap.add_argument("--engine", default="auto", choices=["auto", "hostloop", "persistent"],
                    help="engine of --bfs (auto: the plain BFS engine for --bfs plain)")
    ap.add_argument("--order", default="auto", choices=["auto", "given", "degree"],
                    help="vertex numbering of the plain BFS engine (--bfs plain --engine auto)")
    ap.add_argument("--ctas", type=int, default=0,
                    help="resident CTAs per SM of the plain BFS engine (2, 3 or 4; 0 = default)")
    args = ap.parse_args()
    cfg = CONFIGS[args.config]
    import oracle
    oracle.build()
    if args.impl == "reference":
        run_reference(args, cfg)
    else:
        import importlib.util
        spec = importlib.util.spec_from_file_location(
            "fastcon_build", os.path.join(ROOT, "fast-con_gb300", "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
        if args.bfs:
            run_bfs(args, cfg)
        else:
            run_fastcon(args, cfg)


if __name__ == "__main__":
    main()
