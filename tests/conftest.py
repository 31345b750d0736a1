"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on a
CPU-only machine.  The oracle (oracle/) is used here only as the checker."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (os.path.join(ROOT, "fast-con_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def fastcon_lib():
    """Builds (if needed) and loads libfastcon.so."""
    sys.path.insert(0, os.path.join(ROOT, "fast-con_gb300"))
    import build as fcbuild
    fcbuild.build()
    import fastcon
    fastcon.lib()
    return fastcon


def load_json(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def known_answer_graph():
    """(nv, upper-triangle u, v) of the Graph500 R-MAT scale-16 fixture."""
    z = np.load(os.path.join(GOLDEN, "rmat16_graph500_edges.npz"))
    u = np.cumsum(z["du"].astype(np.int64)).astype(np.int32)
    v = z["v"].astype(np.int32)
    return 1 << 16, u, v


@pytest.fixture(scope="session")
def ka():
    return load_json("stcon_known_answer.json")


@pytest.fixture(scope="session")
def er_golden():
    return load_json("ref_bfs_er65536.json")


@pytest.fixture(scope="session")
def tiny_golden():
    return load_json("ref_bfs_tiny.json")
