"""Seeded synthetic graphs and query sets (host-side restatement).

The generators use one counter-based hash, so every edge and every query is
a pure function of (seed, stream, index).  The same hash is implemented in
CUDA (``csrc/fc_gen.cu``); the GPU generators must reproduce these arrays
bit for bit, which the tests check at small sizes.  Large graphs (R-MAT
scale 24, the 4096x4096 grid) are generated on the GPU; the numpy versions
here are for small graphs and for the parity tests.

Workloads (they stand in for the reference's SNAP/DIMACS files, which are not
available; shapes and seeds follow the benchmark configurations):

* ``er_edges``    -- G(n, m): undirected pairs drawn uniformly until m unique
  non-loop edges exist (first-drawn order wins).
* ``rmat_edges``  -- R-MAT with initiator (a, b, c, d); one 32-bit draw per
  level picks the quadrant with integer thresholds; vertex ids permuted by a
  seeded bijection of [0, 2^scale).
* ``grid_edges``  -- W x H 4-neighbour grid, each edge deleted with
  probability p_del (Bernoulli per edge), plus k random shortcuts.
"""
from __future__ import annotations

import numpy as np

M64 = (1 << 64) - 1
GOLDEN = 0x9E3779B97F4A7C15


def _mix64(z):
    """splitmix64 finaliser on uint64 numpy arrays (wrapping arithmetic)."""
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def hash64(seed: int, stream: int, idx) -> np.ndarray:
    """h(seed, stream, i) = mix64(mix64(seed*G + stream) + (i+1)*G) mod 2^64."""
    base = _mix64(np.uint64((seed * GOLDEN + stream) & M64))
    i = np.asarray(idx, dtype=np.uint64)
    with np.errstate(over="ignore"):
        return _mix64(base + (i + np.uint64(1)) * np.uint64(GOLDEN))


def _scale_to(x32, n: int) -> np.ndarray:
    """Map 32-bit draws to [0, n) by multiply-shift."""
    return ((x32.astype(np.uint64) * np.uint64(n)) >> np.uint64(32)).astype(np.int64)


def er_edges(n: int, m: int, seed: int = 1):
    """Undirected G(n, m) edge list (u < v), in draw order."""
    keys_all = []
    have = 0
    start = 0
    seen = np.empty(0, dtype=np.int64)
    out_u = []
    out_v = []
    while have < m:
        cnt = max(1024, int((m - have) * 1.3))
        r = hash64(seed, 0, np.arange(start, start + cnt, dtype=np.uint64))
        start += cnt
        u = _scale_to(r & np.uint64(0xFFFFFFFF), n)
        v = _scale_to(r >> np.uint64(32), n)
        a = np.minimum(u, v)
        b = np.maximum(u, v)
        ok = a != b
        a, b = a[ok], b[ok]
        key = a * n + b
        # first occurrence within this batch, then drop keys seen before
        _, first = np.unique(key, return_index=True)
        first.sort()
        key, a, b = key[first], a[first], b[first]
        new = ~np.isin(key, seen)
        key, a, b = key[new], a[new], b[new]
        take = min(len(key), m - have)
        out_u.append(a[:take])
        out_v.append(b[:take])
        seen = np.concatenate([seen, key[:take]])
        have += take
        keys_all.append(take)
    return np.concatenate(out_u).astype(np.int32), np.concatenate(out_v).astype(np.int32)


def _perm_params(scale: int, perm_seed: int):
    mask = (1 << scale) - 1
    mults, adds = [], []
    for r in range(3):
        h = int(hash64(perm_seed, 0x5EED0 + r, np.array([0], dtype=np.uint64))[0])
        mults.append((h | 1) & mask if scale > 0 else 0)
        adds.append((h >> 32) & mask)
    shift = scale // 2 + 1
    return mask, mults, adds, shift


def permute_ids(x, scale: int, perm_seed: int) -> np.ndarray:
    """Seeded bijection of [0, 2^scale): three rounds of odd-multiply-add and
    xor-shift, each a bijection on scale-bit integers."""
    mask, mults, adds, shift = _perm_params(scale, perm_seed)
    x = np.asarray(x, dtype=np.uint64)
    mk = np.uint64(mask)
    with np.errstate(over="ignore"):
        for r in range(3):
            x = (x * np.uint64(mults[r]) + np.uint64(adds[r])) & mk
            x = x ^ (x >> np.uint64(shift))
    return x.astype(np.int64)


def rmat_thresholds(a: float, b: float, c: float):
    t1 = int(a * 4294967296.0)
    t2 = int((a + b) * 4294967296.0)
    t3 = int((a + b + c) * 4294967296.0)
    return t1, t2, t3


def rmat_edges(scale: int, nedges: int, a=0.57, b=0.19, c=0.19, seed: int = 3,
               perm_seed: int | None = None, chunk: int = 1 << 22):
    """R-MAT edge list (raw samples: loops and duplicates included)."""
    t1, t2, t3 = rmat_thresholds(a, b, c)
    us, vs = [], []
    for lo in range(0, nedges, chunk):
        idx = np.arange(lo, min(nedges, lo + chunk), dtype=np.uint64)
        u = np.zeros(len(idx), dtype=np.uint64)
        v = np.zeros(len(idx), dtype=np.uint64)
        for k in range(scale):
            x = hash64(seed, k + 1, idx) >> np.uint64(32)
            ub = (x >= np.uint64(t2)).astype(np.uint64)
            vb = (((x >= np.uint64(t1)) & (x < np.uint64(t2))) | (x >= np.uint64(t3))).astype(np.uint64)
            u |= ub << np.uint64(k)
            v |= vb << np.uint64(k)
        us.append(u)
        vs.append(v)
    u = np.concatenate(us) if us else np.zeros(0, np.uint64)
    v = np.concatenate(vs) if vs else np.zeros(0, np.uint64)
    if perm_seed is not None:
        u = permute_ids(u, scale, perm_seed)
        v = permute_ids(v, scale, perm_seed)
    return u.astype(np.int32), v.astype(np.int32)


def grid_edges(w: int, h: int, p_del: float = 0.05, del_seed: int = 5,
               shortcuts: int = 0, sc_seed: int = 6):
    """W x H 4-neighbour grid (vertex r*w + c); each edge j survives unless
    hash(del_seed, 0, j) >> 32 < p_del * 2^32.  Edge j enumerates horizontal
    edges first (j = r*(w-1) + c), then vertical (j = H + r*w + c)."""
    n = w * h
    r, cc = np.divmod(np.arange(h * (w - 1), dtype=np.int64), w - 1)
    hu = r * w + cc
    hv = hu + 1
    r2, c2 = np.divmod(np.arange((h - 1) * w, dtype=np.int64), w)
    vu = r2 * w + c2
    vv = vu + w
    u = np.concatenate([hu, vu])
    v = np.concatenate([hv, vv])
    thr = np.uint64(int(p_del * 4294967296.0))
    keep = (hash64(del_seed, 0, np.arange(len(u), dtype=np.uint64)) >> np.uint64(32)) >= thr
    u, v = u[keep], v[keep]
    if shortcuts:
        rs = hash64(sc_seed, 0, np.arange(shortcuts, dtype=np.uint64))
        su = _scale_to(rs & np.uint64(0xFFFFFFFF), n)
        sv = _scale_to(rs >> np.uint64(32), n)
        u = np.concatenate([u, su])
        v = np.concatenate([v, sv])
    return u.astype(np.int32), v.astype(np.int32)


def grid_shortcut_count(n: int, frac: float = 0.0001) -> int:
    """0.01% of the vertex count, rounded to nearest."""
    return int(round(n * frac))


def uniform_pairs(n: int, count: int, seed: int):
    r = hash64(seed, 0, np.arange(count, dtype=np.uint64))
    s = _scale_to(r & np.uint64(0xFFFFFFFF), n)
    t = _scale_to(r >> np.uint64(32), n)
    return s.astype(np.int32), t.astype(np.int32)


def pairs_with_degree(deg: np.ndarray, count: int, seed: int, min_deg: int = 1):
    """(s, t) with deg >= min_deg at both ends, drawn in order from the hash
    stream (rejection sampling)."""
    n = len(deg)
    out_s, out_t = [], []
    start = 0
    have = 0
    while have < count:
        cnt = max(1024, 4 * (count - have))
        s, t = uniform_pairs_range(n, start, cnt, seed)
        start += cnt
        ok = (deg[s] >= min_deg) & (deg[t] >= min_deg)
        s, t = s[ok], t[ok]
        take = min(len(s), count - have)
        out_s.append(s[:take])
        out_t.append(t[:take])
        have += take
    return np.concatenate(out_s).astype(np.int32), np.concatenate(out_t).astype(np.int32)


def uniform_pairs_range(n: int, start: int, count: int, seed: int):
    r = hash64(seed, 0, np.arange(start, start + count, dtype=np.uint64))
    s = _scale_to(r & np.uint64(0xFFFFFFFF), n)
    t = _scale_to(r >> np.uint64(32), n)
    return s, t


def grid_pairs(w: int, h: int, count: int, seed: int, min_manhattan: int):
    out_s, out_t = [], []
    start = 0
    have = 0
    n = w * h
    while have < count:
        cnt = 4096
        s, t = uniform_pairs_range(n, start, cnt, seed)
        start += cnt
        md = np.abs(s // w - t // w) + np.abs(s % w - t % w)
        ok = md >= min_manhattan
        s, t = s[ok], t[ok]
        take = min(len(s), count - have)
        out_s.append(s[:take])
        out_t.append(t[:take])
        have += take
    return np.concatenate(out_s).astype(np.int32), np.concatenate(out_t).astype(np.int32)


def batched_scales(count: int = 512, first_seed: int = 100, lo: int = 12, hi: int = 20):
    """Scales of the many-graph workload: graph i (seed first_seed + i) has
    scale lo + (hash(seed, 0x5CA1E, 0) mod (hi - lo + 1)), i.e. uniform in
    [lo, hi]."""
    out = []
    for i in range(count):
        h = int(hash64(first_seed + i, 0x5CA1E, np.array([0], dtype=np.uint64))[0])
        out.append(lo + h % (hi - lo + 1))
    return out


def csr_from_edges(nv: int, u: np.ndarray, v: np.ndarray):
    """Canonical CSR in numpy (symmetrised, loops dropped, deduped, rows
    sorted) for small graphs in tests."""
    u = np.asarray(u, np.int64)
    v = np.asarray(v, np.int64)
    ok = u != v
    u, v = u[ok], v[ok]
    a = np.concatenate([u, v])
    b = np.concatenate([v, u])
    key = np.unique(a * nv + b)
    src = key // nv
    dst = (key % nv).astype(np.int32)
    rp = np.zeros(nv + 1, np.int64)
    np.add.at(rp, src + 1, 1)
    rp = np.cumsum(rp).astype(np.int32)
    return rp, dst
