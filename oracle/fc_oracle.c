/*
 * fc_oracle.c -- CPU oracle for the ST-CON / BFS hot path (test
 * infrastructure only; see fc_oracle.h for the rules and the parity pins).
 *
 * Reference paths are relative to the reference project root:
 *   K/ = BFS-4K/,  S/ = bernaschi/ST_CONN_ONE_ATOMIC/current-st/st-conn/
 */
#define _GNU_SOURCE
#include "fc_oracle.h"

#include <ctype.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* BFS: restates Graph::BfsInit (K/src/host/graph.cpp:70-81) and Graph::bfs  */
/* (K/src/host/graph.cpp:83-97).  The reference keeps a separate Visited     */
/* bit vector and an int Distance array initialised to INF; here the level   */
/* array doubles as the visited mark (-1 == INF), which is the same state.   */
/* ------------------------------------------------------------------------ */
int32_t oracle_bfs_levels(int32_t nv, const int32_t *row_ptr, const int32_t *col,
                          int32_t src, int32_t *levels, int32_t *queue,
                          int64_t *edges_inspected)
{
    int32_t left = 0, right = 1;
    int64_t inspected = 0;
    for (int32_t i = 0; i < nv; ++i) levels[i] = -1;
    levels[src] = 0;
    queue[0] = src;
    while (left < right) {
        int32_t q = queue[left++];
        int32_t lq = levels[q];
        int32_t b = row_ptr[q], e = row_ptr[q + 1];
        inspected += e - b;
        for (int32_t i = b; i < e; ++i) {
            int32_t d = col[i];
            if (levels[d] < 0) {
                levels[d] = lq + 1;
                queue[right++] = d;
            }
        }
    }
    if (edges_inspected) *edges_inspected = inspected;
    return right;
}

/* ------------------------------------------------------------------------ */
/* Multi-threaded query pools.                                               */
/* ------------------------------------------------------------------------ */
typedef struct {
    int32_t nv;
    const int32_t *row_ptr, *col;
    int32_t nq;
    const int32_t *s, *t;
    int32_t *connected, *hops;
    int64_t *edges;
    int bidir;
    int nthreads, tid;
} pool_arg;

static int64_t bidir_one(int32_t nv, const int32_t *row_ptr, const int32_t *col,
                         int32_t s, int32_t t, int8_t *side, int32_t *lev,
                         int32_t *qs, int32_t *qt, int32_t *hops_out);

static void *pool_worker(void *p)
{
    pool_arg *a = (pool_arg *)p;
    int32_t *levels = (int32_t *)malloc(sizeof(int32_t) * (size_t)a->nv);
    int32_t *queue = (int32_t *)malloc(sizeof(int32_t) * (size_t)a->nv);
    int32_t *queue2 = a->bidir ? (int32_t *)malloc(sizeof(int32_t) * (size_t)a->nv) : NULL;
    int8_t *side = a->bidir ? (int8_t *)malloc((size_t)a->nv) : NULL;
    if (a->bidir && side) memset(side, 0, (size_t)a->nv);
    for (int32_t q = a->tid; q < a->nq; q += a->nthreads) {
        int64_t ins = 0;
        int32_t h;
        if (a->bidir) {
            ins = bidir_one(a->nv, a->row_ptr, a->col, a->s[q], a->t[q], side, levels,
                            queue, queue2, &h);
        } else {
            oracle_bfs_levels(a->nv, a->row_ptr, a->col, a->s[q], levels, queue, &ins);
            h = levels[a->t[q]];
        }
        a->connected[q] = h >= 0;
        a->hops[q] = h;
        if (a->edges) a->edges[q] = ins;
    }
    free(levels);
    free(queue);
    free(queue2);
    free(side);
    return NULL;
}

static int run_pool(pool_arg proto, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 1024) nthreads = 1024;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    pool_arg *args = (pool_arg *)malloc(sizeof(pool_arg) * (size_t)nthreads);
    for (int i = 0; i < nthreads; ++i) {
        args[i] = proto;
        args[i].nthreads = nthreads;
        args[i].tid = i;
        if (nthreads == 1)
            pool_worker(&args[i]);
        else
            pthread_create(&th[i], NULL, pool_worker, &args[i]);
    }
    if (nthreads > 1)
        for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
    free(th);
    free(args);
    return 0;
}

int oracle_stcon_batch(int32_t nv, const int32_t *row_ptr, const int32_t *col,
                       int32_t nq, const int32_t *s, const int32_t *t,
                       int32_t *connected, int32_t *hops,
                       int64_t *edges_inspected, int nthreads)
{
    for (int32_t q = 0; q < nq; ++q)
        if (s[q] < 0 || s[q] >= nv || t[q] < 0 || t[q] >= nv) return -1;
    pool_arg a;
    memset(&a, 0, sizeof(a));
    a.nv = nv; a.row_ptr = row_ptr; a.col = col; a.nq = nq; a.s = s; a.t = t;
    a.connected = connected; a.hops = hops; a.edges = edges_inspected; a.bidir = 0;
    return run_pool(a, nthreads);
}

/* Bidirectional BFS (stronger CPU baseline, not a reference routine).  Each
 * step expands every vertex of the side whose frontier has the smaller
 * degree sum; the first edge into the other side's ball gives
 * d = level_x + 1 + radius_y (complete, disjoint balls).  side[] is cleared
 * again from the two queues before returning, so it can be reused. */
static int64_t bidir_one(int32_t nv, const int32_t *row_ptr, const int32_t *col,
                         int32_t s, int32_t t, int8_t *side, int32_t *lev,
                         int32_t *qs, int32_t *qt, int32_t *hops_out)
{
    (void)nv;
    (void)lev;
    int64_t ins = 0;
    if (s == t) { *hops_out = 0; return 0; }
    int32_t *q[2] = {qs, qt};
    int32_t head[2] = {0, 0}, tail[2] = {1, 1}, radius[2] = {0, 0};
    int64_t fdeg[2];
    qs[0] = s; qt[0] = t;
    side[s] = 1; side[t] = 2;
    fdeg[0] = row_ptr[s + 1] - row_ptr[s];
    fdeg[1] = row_ptr[t + 1] - row_ptr[t];
    int32_t hops = -1;
    while (head[0] < tail[0] && head[1] < tail[1] && hops < 0) {
        int x = fdeg[0] <= fdeg[1] ? 0 : 1;
        int8_t mine = (int8_t)(x + 1), other = (int8_t)(2 - x);
        int32_t b = head[x], e = tail[x];
        int64_t nd = 0;
        for (int32_t i = b; i < e && hops < 0; ++i) {
            int32_t u = q[x][i];
            int32_t rb = row_ptr[u], re = row_ptr[u + 1];
            ins += re - rb;
            for (int32_t j = rb; j < re; ++j) {
                int32_t v = col[j];
                if (side[v] == 0) {
                    side[v] = mine;
                    q[x][tail[x]++] = v;
                    nd += row_ptr[v + 1] - row_ptr[v];
                } else if (side[v] == other) {
                    hops = radius[x] + 1 + radius[1 - x];
                    break;
                }
            }
        }
        head[x] = e;
        radius[x] += 1;
        fdeg[x] = nd;
    }
    for (int x = 0; x < 2; ++x)
        for (int32_t i = 0; i < tail[x]; ++i) side[q[x][i]] = 0;
    *hops_out = hops;
    return ins;
}

int oracle_stcon_bidir_batch(int32_t nv, const int32_t *row_ptr, const int32_t *col,
                             int32_t nq, const int32_t *s, const int32_t *t,
                             int32_t *connected, int32_t *hops,
                             int64_t *edges_inspected, int nthreads)
{
    for (int32_t q = 0; q < nq; ++q)
        if (s[q] < 0 || s[q] >= nv || t[q] < 0 || t[q] >= nv) return -1;
    pool_arg a;
    memset(&a, 0, sizeof(a));
    a.nv = nv; a.row_ptr = row_ptr; a.col = col; a.nq = nq; a.s = s; a.t = t;
    a.connected = connected; a.hops = hops; a.edges = edges_inspected; a.bidir = 1;
    return run_pool(a, nthreads);
}

/* ------------------------------------------------------------------------ */
/* Canonical CSR (make_g_undirect + make_own_csr_nomulti semantics).         */
/* ------------------------------------------------------------------------ */
static int cmp_i32(const void *a, const void *b)
{
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

typedef struct {
    int32_t *col;
    const int64_t *cnt;
    int32_t lo, hi;
} sort_arg;

static void *sort_rows(void *p)
{
    sort_arg *a = (sort_arg *)p;
    for (int32_t u = a->lo; u < a->hi; ++u)
        qsort(a->col + a->cnt[u], (size_t)(a->cnt[u + 1] - a->cnt[u]), sizeof(int32_t), cmp_i32);
    return NULL;
}

int64_t oracle_build_csr(int32_t nv, int64_t n, const int32_t *src, const int32_t *dst,
                         int flags, int32_t *row_ptr, int32_t *col)
{
    return oracle_build_csr_mt(nv, n, src, dst, flags, row_ptr, col, 1);
}

int64_t oracle_build_csr_mt(int32_t nv, int64_t n, const int32_t *src, const int32_t *dst,
                            int flags, int32_t *row_ptr, int32_t *col, int nthreads)
{
    int sym = flags & ORACLE_SYMMETRIZE, loops = flags & ORACLE_DROP_LOOPS,
        dedupe = flags & ORACLE_DEDUPE;
    int64_t *cnt = (int64_t *)calloc((size_t)nv + 1, sizeof(int64_t));
    for (int64_t i = 0; i < n; ++i) {
        int32_t u = src[i], v = dst[i];
        if (u < 0 || u >= nv || v < 0 || v >= nv) { free(cnt); return -1; }
        if (loops && u == v) continue;
        cnt[u + 1]++;
        if (sym) cnt[v + 1]++;
    }
    for (int32_t i = 0; i < nv; ++i) cnt[i + 1] += cnt[i];
    int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * ((size_t)nv + 1));
    memcpy(fill, cnt, sizeof(int64_t) * ((size_t)nv + 1));
    for (int64_t i = 0; i < n; ++i) {
        int32_t u = src[i], v = dst[i];
        if (loops && u == v) continue;
        col[fill[u]++] = v;
        if (sym) col[fill[v]++] = u;
    }
    /* Sort each row (the reference sorts all (u,v) pairs; per-row sorting
     * after the counting pass yields the same order), then drop repeats. */
    if (dedupe) {
        if (nthreads < 1) nthreads = 1;
        if (nthreads > 256) nthreads = 256;
        pthread_t th[256];
        sort_arg sa[256];
        for (int i = 0; i < nthreads; ++i) {
            sa[i].col = col;
            sa[i].cnt = cnt;
            sa[i].lo = (int32_t)((int64_t)nv * i / nthreads);
            sa[i].hi = (int32_t)((int64_t)nv * (i + 1) / nthreads);
            if (nthreads == 1)
                sort_rows(&sa[i]);
            else
                pthread_create(&th[i], NULL, sort_rows, &sa[i]);
        }
        if (nthreads > 1)
            for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
    }
    int64_t out = 0;
    row_ptr[0] = 0;
    for (int32_t u = 0; u < nv; ++u) {
        int64_t b = cnt[u], e = cnt[u + 1];
        for (int64_t j = b; j < e; ++j) {
            if (dedupe && j > b && col[j] == col[j - 1]) continue;
            col[out++] = col[j];
        }
        if (out > INT32_MAX) { free(cnt); free(fill); return -1; }
        row_ptr[u + 1] = (int32_t)out;
    }
    free(cnt);
    free(fill);
    return out;
}

/* ------------------------------------------------------------------------ */
/* R-MAT samples (input generation; same hash as fastcon/graphs.py).         */
/* ------------------------------------------------------------------------ */
#define GOLDEN64 0x9E3779B97F4A7C15ULL
static uint64_t mix64(uint64_t z);

static uint64_t hash_base(uint64_t seed, uint64_t stream) { return mix64(seed * GOLDEN64 + stream); }
static uint64_t hash_at(uint64_t base, uint64_t i) { return mix64(base + (i + 1) * GOLDEN64); }

typedef struct {
    int scale;
    int64_t lo, hi;
    uint32_t t1, t2, t3;
    uint64_t seed;
    int perm;
    uint64_t mask, mult[3], add[3];
    int shift;
    int32_t *src, *dst;
} rmat_arg;

static void *rmat_worker(void *p)
{
    rmat_arg *a = (rmat_arg *)p;
    uint64_t bases[64];
    for (int k = 0; k < a->scale; ++k) bases[k] = hash_base(a->seed, (uint64_t)(k + 1));
    for (int64_t i = a->lo; i < a->hi; ++i) {
        uint64_t u = 0, v = 0;
        for (int k = 0; k < a->scale; ++k) {
            uint32_t x = (uint32_t)(hash_at(bases[k], (uint64_t)i) >> 32);
            uint64_t ub = x >= a->t2;
            uint64_t vb = (x >= a->t1 && x < a->t2) || x >= a->t3;
            u |= ub << k;
            v |= vb << k;
        }
        if (a->perm) {
            for (int r = 0; r < 3; ++r) {
                u = (u * a->mult[r] + a->add[r]) & a->mask;
                u ^= u >> a->shift;
                v = (v * a->mult[r] + a->add[r]) & a->mask;
                v ^= v >> a->shift;
            }
        }
        a->src[i] = (int32_t)u;
        a->dst[i] = (int32_t)v;
    }
    return NULL;
}

void oracle_gen_rmat(int scale, int64_t nedges, double a, double b, double c, uint64_t seed,
                     int64_t perm_seed, int32_t *src, int32_t *dst, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    rmat_arg proto;
    memset(&proto, 0, sizeof(proto));
    proto.scale = scale;
    proto.t1 = (uint32_t)(a * 4294967296.0);
    proto.t2 = (uint32_t)((a + b) * 4294967296.0);
    proto.t3 = (uint32_t)((a + b + c) * 4294967296.0);
    proto.seed = seed;
    proto.perm = perm_seed >= 0;
    proto.mask = (1ULL << scale) - 1;
    for (int r = 0; r < 3; ++r) {
        uint64_t h = hash_at(hash_base((uint64_t)perm_seed, 0x5EED0ULL + (uint64_t)r), 0);
        proto.mult[r] = (h | 1ULL) & proto.mask;
        proto.add[r] = (h >> 32) & proto.mask;
    }
    proto.shift = scale / 2 + 1;
    proto.src = src;
    proto.dst = dst;
    pthread_t th[256];
    rmat_arg args[256];
    for (int i = 0; i < nthreads; ++i) {
        args[i] = proto;
        args[i].lo = nedges * i / nthreads;
        args[i].hi = nedges * (i + 1) / nthreads;
        if (nthreads == 1)
            rmat_worker(&args[i]);
        else
            pthread_create(&th[i], NULL, rmat_worker, &args[i]);
    }
    if (nthreads > 1)
        for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
}

int64_t oracle_count_visited_edges(int32_t nv, const int32_t *row_ptr, const int32_t *col,
                                   const int32_t *levels)
{
    int64_t c = 0;
    for (int32_t v = 0; v < nv; ++v) {
        if (levels[v] < 0) continue;
        for (int32_t j = row_ptr[v]; j < row_ptr[v + 1]; ++j)
            if (col[j] <= v) ++c;
    }
    return c;
}

/* ------------------------------------------------------------------------ */
/* Edge-list reader.                                                          */
/* ------------------------------------------------------------------------ */
typedef struct { int64_t *keys; int32_t *vals; int64_t cap, size; } idmap;

static uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

static int32_t idmap_insert(idmap *m, int64_t key)
{
    if ((m->size + 1) * 2 > m->cap) {
        int64_t nc = m->cap ? m->cap * 2 : 1024;
        int64_t *nk = (int64_t *)malloc(sizeof(int64_t) * (size_t)nc);
        int32_t *nvl = (int32_t *)malloc(sizeof(int32_t) * (size_t)nc);
        for (int64_t i = 0; i < nc; ++i) nk[i] = -1;
        for (int64_t i = 0; i < m->cap; ++i) {
            if (m->keys[i] < 0) continue;
            uint64_t h = mix64((uint64_t)m->keys[i]) & (uint64_t)(nc - 1);
            while (nk[h] >= 0) h = (h + 1) & (uint64_t)(nc - 1);
            nk[h] = m->keys[i];
            nvl[h] = m->vals[i];
        }
        free(m->keys);
        free(m->vals);
        m->keys = nk; m->vals = nvl; m->cap = nc;
    }
    uint64_t h = mix64((uint64_t)key) & (uint64_t)(m->cap - 1);
    while (m->keys[h] >= 0) {
        if (m->keys[h] == key) return m->vals[h];
        h = (h + 1) & (uint64_t)(m->cap - 1);
    }
    m->keys[h] = key;
    m->vals[h] = (int32_t)m->size;
    return (int32_t)m->size++;
}

/* Reads the next unsigned/signed decimal integer on the current line.
 * Returns 1 and advances *pp on success, 0 at end of line. */
static int next_int(const char **pp, int64_t *out)
{
    const char *p = *pp;
    while (*p == ' ' || *p == '\t' || *p == '\r') ++p;
    if (!(*p == '-' || isdigit((unsigned char)*p))) { *pp = p; return 0; }
    char *end;
    long long v = strtoll(p, &end, 10);
    if (end == p) return 0;
    *out = v;
    *pp = end;
    return 1;
}

int oracle_read_edgelist(const char *path, int relabel, int32_t *nv_out, int64_t *n_out,
                         int *file_directed, int32_t *src, int32_t *dst)
{
    FILE *f = fopen(path, "r");
    if (!f) return -1;
    char *line = NULL;
    size_t cap = 0;
    ssize_t len;
    int fmt = 0; /* 1 snap, 2 mm, 3 dimacs9, 4 dimacs10 */
    int64_t nodes = -1, declared = -1, n = 0;
    int dir = -1;
    int header_done = 0;
    int64_t d10_line = 0;
    int mm_sizes_read = 0;
    idmap map = {0, 0, 0, 0};
    int64_t maxid = -1;
    int bad = 0;
    while ((len = getline(&line, &cap, f)) > 0) {
        const char *p = line;
        while (*p == ' ' || *p == '\t') ++p;
        if (fmt == 0) {
            if (*p == '\n' || *p == 0) continue;
            if (p[0] == '#') fmt = 1;
            else if (strncmp(p, "%%MatrixMarket", 14) == 0) fmt = 2;
            else if (p[0] == 'c' || p[0] == 'p') fmt = 3;
            else if (p[0] == '%' || isdigit((unsigned char)p[0])) fmt = 4;
            else { bad = 1; break; }
        }
        if (fmt == 1) {
            if (p[0] == '#') {
                if (strstr(p, "Undirected")) dir = 0;
                else if (strstr(p, "Directed") && dir < 0) dir = 1;
                const char *q = strstr(p, "Nodes:");
                if (q) {
                    long long a = -1, b = -1;
                    if (sscanf(q, "Nodes: %lld Edges: %lld", &a, &b) >= 1) { nodes = a; declared = b; }
                }
                continue;
            }
            int64_t a, b;
            if (!next_int(&p, &a)) continue;
            if (!next_int(&p, &b) || a < 0 || b < 0) { bad = 1; break; }
            if (relabel) { a = idmap_insert(&map, a); b = idmap_insert(&map, b); }
            if (a > maxid) maxid = a;
            if (b > maxid) maxid = b;
            if (src) { src[n] = (int32_t)a; dst[n] = (int32_t)b; }
            ++n;
        } else if (fmt == 2) {
            if (p[0] == '%') {
                if (strncmp(p, "%%MatrixMarket", 14) == 0)
                    dir = strstr(p, "symmetric") ? 0 : 1;
                continue;
            }
            int64_t a, b, c;
            if (!mm_sizes_read) {
                if (!next_int(&p, &a)) continue;
                if (!next_int(&p, &b) || !next_int(&p, &c)) { bad = 1; break; }
                nodes = a; declared = c; mm_sizes_read = 1;
                continue;
            }
            if (!next_int(&p, &a)) continue;
            if (!next_int(&p, &b) || a < 1 || b < 1) { bad = 1; break; }
            if (src) { src[n] = (int32_t)(a - 1); dst[n] = (int32_t)(b - 1); }
            if (a - 1 > maxid) maxid = a - 1;
            if (b - 1 > maxid) maxid = b - 1;
            ++n;
        } else if (fmt == 3) {
            if (p[0] == 'p') {
                char w1[64], w2[64];
                long long a = -1, b = -1;
                if (sscanf(p, "%63s %63s %lld %lld", w1, w2, &a, &b) == 4) { nodes = a; declared = b; }
                continue;
            }
            if (p[0] != 'a') continue;
            ++p;
            int64_t a, b;
            if (!next_int(&p, &a) || !next_int(&p, &b) || a < 1 || b < 1) { bad = 1; break; }
            if (src) { src[n] = (int32_t)(a - 1); dst[n] = (int32_t)(b - 1); }
            if (a - 1 > maxid) maxid = a - 1;
            if (b - 1 > maxid) maxid = b - 1;
            ++n;
        } else {
            if (p[0] == '%') continue;
            if (!header_done) {
                int64_t a, b, c;
                if (!next_int(&p, &a)) continue;
                if (!next_int(&p, &b)) { bad = 1; break; }
                nodes = a; declared = b;
                dir = (next_int(&p, &c) && c == 100) ? 1 : 0;
                header_done = 1;
                continue;
            }
            if (d10_line >= nodes) continue;
            int64_t a;
            while (next_int(&p, &a)) {
                if (a < 1) { bad = 1; break; }
                if (src) { src[n] = (int32_t)d10_line; dst[n] = (int32_t)(a - 1); }
                if (a - 1 > maxid) maxid = a - 1;
                ++n;
            }
            if (bad) break;
            ++d10_line;
        }
    }
    free(line);
    fclose(f);
    free(map.keys);
    free(map.vals);
    (void)declared;
    if (bad || fmt == 0) return -1;
    /* renumbered SNAP ids: the header's node count when larger, as
     * readGraphHeader sizes the graph from it (K/Util/readGraphHeader.cpp:101-114) */
    int64_t nvv = relabel && fmt == 1 ? (map.size > nodes ? map.size : nodes) : nodes;
    if (nvv < maxid + 1) nvv = maxid + 1;
    if (nvv > INT32_MAX) return -1;
    *nv_out = (int32_t)nvv;
    *n_out = n;
    if (file_directed) *file_directed = dir;
    return 0;
}
