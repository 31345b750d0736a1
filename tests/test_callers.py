"""Compiled callers of the C ABI, written as the reference's drivers would
call the library after the swap (tests/callers/):

* stcon_driver.c -- the bernaschi ST-CON driver's calls (S/main.c:378,438,
  S/make_stcon.c:446): built with gcc against include/fastcon.h and
  libfastcon.so; on a GPU it runs the reference's logged known-answer run
  (Graph500 R-MAT scale 16, 100 pairs, S/data/st_stats_20200418_140644) and
  its depths, distances and batch answers are checked;
* bfs4k_wrapper.cpp -- the BFS-4K cudaGraph drop-in (K/include/device/
  cudaGraph.cuh:14-35) built with g++ against the reference's own host
  header K/include/host/graph.h and its readers; compiled and linked where
  the reference tree is present (it cannot be carried to a GPU machine).
"""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT, known_answer_graph, load_json

CALLERS = os.path.join(ROOT, "tests", "callers")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "fast-con_gb300", "fastcon")
REF = os.environ.get("FASTCON_REFERENCE", "/root/reference")


def _build_driver(out_dir):
    exe = os.path.join(out_dir, "stcon_driver")
    cmd = ["gcc", "-O2", "-std=c11", "-Wall", "-Werror", "-I" + INCLUDE,
           os.path.join(CALLERS, "stcon_driver.c"), "-o", exe, "-L" + LIBDIR, "-lfastcon",
           "-Wl,-rpath," + LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_driver_builds_against_the_header(fastcon_lib):
    with tempfile.TemporaryDirectory() as td:
        exe = _build_driver(td)
        assert os.path.exists(exe)
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 2  # usage: nothing touched the device


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "BFS-4K")),
                    reason="reference tree not present")
def test_bfs4k_wrapper_builds_against_reference_header(fastcon_lib):
    K = os.path.join(REF, "BFS-4K")
    srcs = [os.path.join(K, "src", "host", "graph.cpp")] + [
        os.path.join(K, "Util", f) for f in ("readGraphHeader.cpp", "readGraphSTD.cpp",
                                              "readUtil.cpp", "fUtil.cpp")]
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "bfs4k_wrapper")
        cmd = ["g++", "-O2", "-std=c++11", "-w", "-I" + INCLUDE,
               "-I" + os.path.join(K, "include", "host"), "-I" + os.path.join(K, "Util"),
               "-I/usr/local/cuda/include", os.path.join(CALLERS, "bfs4k_wrapper.cpp")] + srcs + \
              ["-o", exe, "-L" + LIBDIR, "-lfastcon", "-Wl,-rpath," + LIBDIR]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        assert os.path.exists(exe)


@pytest.mark.gpu
@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_c_driver_runs_the_known_answer_run(fastcon_lib, oracle_mod):
    ka = load_json("stcon_known_answer.json")
    nv, u, v = known_answer_graph()
    red = [r["red"] for r in ka["rows"]]
    blue = [r["blue"] for r in ka["rows"]]
    with tempfile.TemporaryDirectory() as td:
        exe = _build_driver(td)
        gpath = os.path.join(td, "rmat16.txt")
        with open(gpath, "w") as f:
            f.write(f"# Undirected graph: Graph500 R-MAT scale 16\n# Nodes: {nv} Edges: {len(u)}\n"
                    "# FromNodeId\tToNodeId\n")
            f.write("".join(f"{a}\t{b}\n" for a, b in zip(u.tolist(), v.tolist())))
        ppath = os.path.join(td, "pairs.txt")
        with open(ppath, "w") as f:
            f.write("".join(f"{a} {b}\n" for a, b in zip(red, blue)))
        r = subprocess.run([exe, gpath, ppath], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
    q, b, lev = {}, {}, None
    for ln in r.stdout.splitlines():
        p = ln.split()
        if p[0] == "q":
            q[int(p[1])] = tuple(int(x) for x in p[2:])
        elif p[0] == "b":
            b[int(p[1])] = tuple(int(x) for x in p[2:])
        elif p[0] == "levels":
            lev = tuple(int(x) for x in p[1:])
    assert len(q) == len(b) == 100
    for i, row in enumerate(ka["rows"]):
        depth, conn, hops = q[i]
        assert depth == row["depth"], (i, depth, row["depth"])  # make_stcon's DEPTH
        assert conn == 1 and hops == ka["ref_bfs_hops"][i]       # Graph::bfs distance
        assert b[i] == (1, hops)
    rp, col = oracle_mod.build_csr(nv, u, v)
    want, _ = oracle_mod.bfs_levels(rp, col, red[0])
    assert lev == (red[0], int((want >= 0).sum()), int(want[want >= 0].sum()))
