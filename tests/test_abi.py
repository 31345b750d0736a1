"""The C-ABI library loads and exports every entry point include/fastcon.h
declares; argument errors come back as status codes (no GPU needed: none of
these calls reaches a kernel)."""
import ctypes
import os
import re

import numpy as np
from conftest import ROOT


def declared_functions():
    text = open(os.path.join(ROOT, "include", "fastcon.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fc_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(fastcon_lib):
    names = declared_functions()
    assert len(names) >= 20
    L = fastcon_lib.lib()
    for n in names:
        assert hasattr(L, n), n
    assert sorted(fastcon_lib.EXPORTS) == names


def test_status_codes_without_device(fastcon_lib):
    L = fastcon_lib.lib()
    assert L.fc_strerror(0) == b"ok"
    assert L.fc_strerror(6) == b"device-side wait timed out"
    assert L.fc_strerror(99) == b"unknown error"
    h = ctypes.c_void_p()
    # NULL arrays / bad sizes are rejected before any device work
    assert L.fc_graph_from_csr(None, 4, None, 0, 0, ctypes.byref(h)) == fastcon_lib.ERR_INVALID
    rp = np.array([0, 2, 1], np.int32)  # decreasing
    col = np.array([1], np.int32)
    assert L.fc_graph_from_csr(rp.ctypes.data, 2, col.ctypes.data, 1, 0,
                               ctypes.byref(h)) == fastcon_lib.ERR_INVALID
    assert b"decreases" in L.fc_last_error_message()
    rp = np.array([0, 1, 1], np.int32)
    bad = np.array([7], np.int32)
    assert L.fc_graph_from_csr(rp.ctypes.data, 2, bad.ctypes.data, 1, 0,
                               ctypes.byref(h)) == fastcon_lib.ERR_INVALID
    assert L.fc_graph_from_edges(None, None, 0, 0, 0, ctypes.byref(h)) == fastcon_lib.ERR_INVALID
    c = ctypes.c_int32()
    assert L.fc_stcon(None, 0, 1, ctypes.byref(c), ctypes.byref(c)) == fastcon_lib.ERR_INVALID
    assert L.fc_bfs_levels(None, 0, None) == fastcon_lib.ERR_INVALID
    assert L.fc_graph_load_edgelist(b"/nonexistent/file.txt", -1, 0,
                                    ctypes.byref(h)) == fastcon_lib.ERR_IO
    assert L.fc_selftest_wait(0, None) == fastcon_lib.ERR_INVALID
    assert L.fc_selftest_wait(5000, None) == fastcon_lib.ERR_INVALID
    assert L.fc_version() == 100


def test_opts_layout(fastcon_lib):
    o = fastcon_lib.make_opts(sched=2, engine=3, block=256)
    assert (o.sched, o.engine, o.block) == (2, 3, 256)
    assert ctypes.sizeof(fastcon_lib.Opts) == 4 * 6 + 8 + 4 * 8
    # fc_stats: 2 x int64, 2 x int32, double, int64, 2 x int32, 2 x double,
    # 2 x int64, 2 x int32, int64
    assert ctypes.sizeof(fastcon_lib.Stats) == 16 + 8 + 8 + 8 + 8 + 16 + 16 + 8 + 8


def test_struct_offsets_match_the_header(fastcon_lib, tmp_path):
    """Every field of fc_opts and fc_stats sits where include/fastcon.h puts
    it: a C program built against the header prints offsetof and sizeof, and
    the ctypes mirror must agree field by field."""
    import shutil
    import subprocess

    import pytest
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    structs = {"fc_opts": fastcon_lib.Opts, "fc_stats": fastcon_lib.Stats}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "fastcon.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "offsets.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "offsets"
    r = subprocess.run(["gcc", "-std=c11", "-I" + os.path.join(ROOT, "include"), str(src), "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for ln in out:
        if ln:
            c, f, v = ln.split()
            got[(c, f)] = int(v)
    for cname, py in structs.items():
        assert got[(cname, "sizeof")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
