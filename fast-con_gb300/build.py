"""Build recipe for libfastcon.so (sm_103a only).

Compiles every csrc/*.cu translation unit in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo`` and links the
shared library in-tree at fastcon/libfastcon.so.  Objects go to _build/
(git-ignored).  A unit is rebuilt when it or any header is newer than its
object.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "fastcon", "libfastcon.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
         "-I" + INCLUDE, "-I" + CSRC]
# per-unit flags: the Graph500 generator rounds its doubles as the reference
# generator does, so its multiply-adds must not be fused
UNIT_FLAGS = {"fc_g500.cu": ["-fmad=false"]}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _headers_mtime() -> float:
    hs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def _compile(src: str, obj: str, extra: list[str]) -> None:
    cmd = [nvcc()] + ARCH + FLAGS + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stderr}")


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    extra = list(extra or [])
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdr_t = _headers_mtime()
    jobs = []
    objs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_t):
            jobs.append((s, o))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            futs = [ex.submit(_compile, s, o, extra + UNIT_FLAGS.get(os.path.basename(s), []))
                    for s, o in jobs]
            for f in futs:
                f.result()
    newest = max(os.path.getmtime(o) for o in objs)
    if force or jobs or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        # shared CUDA runtime: one runtime state (current device, streams) with
        # the host process's other CUDA users
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr)
        if verbose:
            print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
