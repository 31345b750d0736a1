"""The scan, compaction and search primitives of the expansion steps
(fc_step.cuh, fc_internal.cuh), run on the GPU through fc_selftest_primitives
and compared element by element with plain restatements: inclusive scans
(std::inclusive_scan per warp / per block), the load-balanced search's row of
every entry (each row's entries in order, np.repeat), and the claim
compaction (every offered value exactly once).  The reference takes these
from Thrust and CUB (S/mythrustlib.cu:25-34,175-185) and checks its scan
with check_queue_off (S/test/gputestfunc.cu:225-258)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _group_cumsum(a, g):
    out = np.empty_like(a)
    tot = []
    for b in range(0, len(a), g):
        out[b:b + g] = np.cumsum(a[b:b + g])
        tot.append(int(a[b:b + g].sum()))
    return out, np.array(tot)


@pytest.mark.parametrize("n", [1, 31, 32, 1000, 65537])
def test_warp_and_block_scans(fastcon_lib, n):
    fc = fastcon_lib
    rng = np.random.default_rng(n)
    a = rng.integers(-1000, 1000, n).astype(np.int32)
    out, _ = fc.selftest_primitives(0, a)
    assert (out == _group_cumsum(a, 32)[0]).all()
    out, aux = fc.selftest_primitives(1, a)
    want, tot = _group_cumsum(a, 256)
    assert (out == want).all() and (aux[:len(tot)] == tot).all()


def test_load_balanced_search(fastcon_lib):
    fc = fastcon_lib
    rng = np.random.default_rng(7)
    lens = rng.integers(0, 40, 256 * 9 + 77).astype(np.int32)
    lens[100:180] = 0              # runs of empty rows
    lens[300] = 5000               # a row longer than a tile's round
    lens[256 * 3:256 * 4] = 0      # an empty tile
    lens[-1] = 0
    out, _ = fc.selftest_primitives(2, lens)
    want = np.concatenate([np.repeat(np.arange(len(lens[b:b + 256])), lens[b:b + 256])
                           for b in range(0, len(lens), 256)])
    assert len(out) == len(want) and (out == want).all()


@pytest.mark.parametrize("density", [0.0, 0.02, 0.3, 1.0])
def test_claim_compaction(fastcon_lib, density):
    fc = fastcon_lib
    rng = np.random.default_rng(int(density * 100) + 3)
    n = 50000
    vals = rng.permutation(n).astype(np.int32)
    keep = rng.random(n) < density
    a = np.where(keep, vals, -1).astype(np.int32)
    out, aux = fc.selftest_primitives(3, a)
    cnt = int(aux[0])
    assert cnt == int(keep.sum())
    assert (np.sort(out[:cnt]) == np.sort(vals[keep])).all()
