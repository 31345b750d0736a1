"""The Graph500 generator on the device against the reference's own
generator (make_graph, bernaschi/ST_CONN_ONE_ATOMIC/current-st/generator/
make_graph.c:35-104, compiled into oracle/_ref/graph500_gen): the raw edge
list (sorted, self-loops and repeats included) and the CSR built from it must
be identical, at every size and seed of tests/golden/ref_graph500.json --
among them the scale-16 graph of the reference's logged ST-CON run."""
import hashlib

import numpy as np
import pytest

from conftest import load_json

pytestmark = pytest.mark.gpu


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()


def _sha_csr(rp, col):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(rp, dtype="<i4").tobytes())
    h.update(np.ascontiguousarray(col, dtype="<i4").tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("case", load_json("ref_graph500.json"),
                         ids=lambda c: f"scale{c['scale']}-ef{c['edgefactor']}-s{c['seed1']}")
def test_generator_matches_reference(fastcon_lib, case):
    fc = fastcon_lib
    scale, m = case["scale"], case["nedges"]
    src, dst = fc.graph500_edges(scale, m, case["seed1"], case["seed2"])
    assert int((src == dst).sum()) == case["self_loops"]
    o = np.lexsort((dst, src))
    assert _sha(np.stack([src[o], dst[o]], 1).reshape(-1)) == case["sorted_edges_sha256"]
    G = fc.Graph.graph500(scale, m, case["seed1"], case["seed2"])
    rp, col = G.csr()
    assert G.ne == case["directed_entries"] and _sha_csr(rp, col) == case["csr_sha256"]
    G.free()


def test_known_answer_graph_and_depths(fastcon_lib):
    """The graph of the reference's logged run, generated on the device, gives
    its 100 logged depths."""
    fc = fastcon_lib
    ka = load_json("stcon_known_answer.json")
    gi = ka["graph"]
    G = fc.Graph.graph500(gi["scale"], gi["generated_edges"], gi["seed1"], gi["seed2"])
    rp, col = G.csr()
    assert _sha_csr(rp, col) == gi["csr_sha256"]
    red = np.array([r["red"] for r in ka["rows"]], np.int32)
    blue = np.array([r["blue"] for r in ka["rows"]], np.int32)
    conn, hops = fc.stcon_batch(G, red, blue)
    assert ((hops + 1) // 2 == np.array([r["depth"] for r in ka["rows"]])).all()


def test_generator_rejects_bad_arguments(fastcon_lib):
    fc = fastcon_lib
    with pytest.raises(fc.FastconError):
        fc.Graph.graph500(0, 10, 1, 2)
    with pytest.raises(fc.FastconError):
        fc.Graph.graph500(10, 100, 1, 2, initiator=(0.5, 0.5, 0.5, 0.5))
    G = fc.Graph.graph500(6, 1, 3, 4)  # one edge: walks down from the root
    assert G.ne in (0, 2)
