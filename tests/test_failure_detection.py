"""Failure detection on the GPU without a fault: a device-side wait that can
only expire must end at its time limit with FC_ERR_TIMEOUT, and the device
must stay usable afterwards."""
import numpy as np
import pytest

from fastcon import graphs

pytestmark = pytest.mark.gpu


def test_bounded_wait_expires_and_device_stays_usable(fastcon_lib, oracle_mod):
    fc = fastcon_lib
    for limit in (50, 200):
        rc, ms = fc.selftest_wait(limit)
        assert rc == fc.ERR_TIMEOUT
        assert 0.8 * limit <= ms <= limit + 2000, ms
        assert "expired" in fc.lib().fc_last_error_message().decode()
    # the context is intact: a batch on every engine still gives exact answers
    u, v = graphs.rmat_edges(12, 8 << 12, seed=31, perm_seed=32)
    G = fc.Graph.from_edges(u, v, 1 << 12)
    rp, col = oracle_mod.build_csr(1 << 12, u, v)
    s, t = graphs.uniform_pairs(1 << 12, 200, seed=33)
    _, want, _ = oracle_mod.stcon_batch(rp, col, s, t, nthreads=4)
    for eng in (fc.ENGINE_BATCHED, fc.ENGINE_PERSISTENT, fc.ENGINE_HOSTLOOP):
        conn, hops = fc.stcon_batch(G, s, t, opts=fc.make_opts(engine=eng))
        assert (hops == want).all(), eng
