// fc_step.cuh -- one expansion step of one side, for any team of CTAs.
//
// A "team" is the set of CTAs that cooperates on one query: the whole
// cooperative grid (persistent engine), every CTA of an ordinary launch
// (host-loop engine), or a single CTA (batched engine).  The step functions
// take the team rank/size and never synchronise across CTAs themselves; the
// engine puts a team barrier between steps.
//
// Top-down expansion (the hybrid variant) reads a tile's rows by load-balanced
// search: a CTA prefix scan lays the rows end to end and every thread reads
// GATHER_PER_THREAD entries per round, finding each entry's row by binary
// search in shared memory, whatever the mix of row lengths (after Merrill,
// Garland & Grimshaw, "Scalable GPU Graph Traversal", PPoPP 2012, and the
// load-balanced strategy of Gunrock).  Rows longer than the engine's job
// length become row jobs that the whole team shares.  Long rows in the other
// variants are walked with 16-byte int4 loads of the column array.  Newly
// claimed vertices are appended to the log with a warp ballot/shuffle scan
// and one atomicAdd per warp; the load-balanced search first gathers them in
// a per-warp buffer in shared memory and reserves log space once per
// WARP_LOG claims (or at the end of the tile), so that a level whose
// neighbours are mostly visited already does not send one returning atomic
// per warp and round to the same counter.
#pragma once

#include <climits>

#include "fc_internal.cuh"

namespace fc {

constexpr int GATHER_PER_THREAD = 8;  // load-balanced search: entries per thread per round
constexpr int GATHER_TEAM = 16;       // the same in team steps (whole-grid levels), where more
                                      // loads in flight pay: plain BFS on R-MAT 24 5.1 -> 4.0 ms
constexpr long long TEAM_TILE_E = 16384;  // team steps: adjacency entries a tile aims at

// Frontier vertices per top-down tile of a team step: T, or fewer (a power
// of two, at least 1) when the frontier's m entries over F vertices would
// give tiles of more than TEAM_TILE_E entries.
template <int T>
__host__ __device__ inline int team_tile_v(long long F, long long m)
{
    if (F <= 0 || m <= (long long)F * (TEAM_TILE_E / T)) return T;
    const long long want = TEAM_TILE_E * F / m;
    int tv = 1;
    while (tv * 2 <= want && tv * 2 <= T) tv *= 2;
    return tv;
}
constexpr int BU_GROUP = 4;  // bottom-up: neighbours loaded together
constexpr int TINY_STEP_E = 1024;  // a one-warp frontier reading at most this many entries
                                   // is expanded by one warp without CTA barriers

struct AppendTarget {
    int32_t *log;       // log base of the slot
    int32_t nv;         // graph size: side 1 writes log[nv - 1 - pos]
    int32_t side;
    int *tail;          // cumulative append counter of this side
    unsigned long long *deg;  // cumulative degree sum of appended vertices
    const int32_t *row_ptr;   // CSR used to expand this side next time
    unsigned long long *hist; // nullable: packed counts of claimed vertices of degree < 8
                              // (low 32 bits) and >= 128 (high 32 bits)
    unsigned long long *reads; // nullable: adjacency entries actually read (a step
                               // that stops early reads fewer than its frontier holds)
    int *wlog = nullptr;  // nullable (shared memory): per-warp claim buffers of
                          // WARP_LOG entries, warp w's at wlog + w * WARP_LOG
    int *wcnt = nullptr;  // their fill counts, one per warp
};
constexpr int WARP_LOG = 128;

__device__ __forceinline__ void log_write(const AppendTarget &a, int pos, int v)
{
    if (a.side == 0)
        a.log[pos] = v;
    else
        a.log[a.nv - 1 - pos] = v;
}

// Degree-sum and histogram counters of claims whose degrees d[k] are known:
// one warp reduction, then one (non-returning) add by lane 0.  All 32 lanes
// call it.
template <int K>
__device__ __forceinline__ void warp_count_degrees(const int (&c)[K], const int (&d)[K],
                                                   const AppendTarget &a)
{
    long long dsum = 0;
    int h0 = 0, h2 = 0;
#pragma unroll
    for (int k = 0; k < K; ++k)
        if (c[k] >= 0) {
            dsum += d[k];
            h0 += d[k] < 8;
            h2 += d[k] >= 128;
        }
    dsum = warp_sum_ll(dsum);
    if (lane_id() == 0 && dsum) atomicAdd(a.deg, (unsigned long long)dsum);
    if (a.hist) {  // uniform: same pointer in every lane
        const unsigned long long w =
            (unsigned long long)warp_sum_i(h0) | ((unsigned long long)warp_sum_i(h2) << 32);
        if (lane_id() == 0 && w) atomicAdd(a.hist, w);
    }
}

// Move the warp's buffered claims to the log: one reservation on the tail
// counter (their degrees were counted when they were buffered).  All 32
// lanes call it; the buffer is empty afterwards.
__device__ __forceinline__ void warp_flush(const AppendTarget &a)
{
    const int w = (int)(threadIdx.x >> 5), lane = (int)lane_id();
    const int n = a.wcnt[w];
    if (n == 0) return;
    const int *buf = a.wlog + w * WARP_LOG;
    int base = 0;
    if (lane == 0) base = atomicAdd(a.tail, n);
    base = __shfl_sync(0xffffffffu, base, 0);
#pragma unroll
    for (int j = 0; j < WARP_LOG / 32; ++j) {
        const int i = j * 32 + lane;
        if (i < n) log_write(a, base + i, buf[i]);
    }
    __syncwarp();
    if (lane == 0) a.wcnt[w] = 0;
    __syncwarp();
}

// Append the claimed vertices c[k] >= 0, whose degrees in the CSR the side
// expands next are d[k].  All 32 lanes of the warp must call this with the
// same K.
template <int K>
__device__ __forceinline__ void warp_append_deg(const int (&c)[K], const int (&d)[K],
                                                const AppendTarget &a)
{
    int cnt = 0;
#pragma unroll
    for (int k = 0; k < K; ++k) cnt += c[k] >= 0;
    unsigned any = __ballot_sync(0xffffffffu, cnt > 0);
    if (!any) return;
    warp_count_degrees<K>(c, d, a);
    int incl = warp_inclusive_scan(cnt);
    int total = __shfl_sync(0xffffffffu, incl, 31);
    if (a.wlog && total <= WARP_LOG) {
        const int w = (int)(threadIdx.x >> 5);
        int n0 = a.wcnt[w];
        if (n0 + total > WARP_LOG) {
            warp_flush(a);
            n0 = 0;
        }
        int *buf = a.wlog + w * WARP_LOG;
        int pos = n0 + incl - cnt;
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (c[k] >= 0) buf[pos++] = c[k];
        __syncwarp();
        if (lane_id() == 0) a.wcnt[w] = n0 + total;
        __syncwarp();
        return;
    }
    int base = 0;
    if (lane_id() == 0) base = atomicAdd(a.tail, total);
    base = __shfl_sync(0xffffffffu, base, 0);
    int pos = base + incl - cnt;
#pragma unroll
    for (int k = 0; k < K; ++k)
        if (c[k] >= 0) log_write(a, pos++, c[k]);
}

// The same for claims whose degrees are not known yet: they are read here.
template <int K>
__device__ __forceinline__ void warp_append(const int (&c)[K], const AppendTarget &a)
{
    int d[K];
#pragma unroll
    for (int k = 0; k < K; ++k)
        d[k] = c[k] >= 0 ? __ldg(a.row_ptr + c[k] + 1) - __ldg(a.row_ptr + c[k]) : 0;
    warp_append_deg<K>(c, d, a);
}

// ---------------------------------------------------------------------------
// Visitors: what happens at one neighbour v of a frontier vertex, in three
// phases so that a thread has several neighbours' loads AND claims in flight:
// probe(v) reads v's state; attempt(v, p) issues the claim when v looked free
// and returns the state the claim found (or p); resolve(v, r) returns v when
// this thread claimed it, else -1.  Only r is kept between attempt and
// resolve.  visit() = all three.
//
// The s-t claim needs no compare: one side expands per step and every claim
// of a step writes the same code, so an atomicAnd that clears the bits that
// are 0 in the code turns an unvisited byte (0xFF) into the code and leaves a
// byte claimed earlier in the step as it was; the byte it returns says which
// happened.  (A byte of the other side or of an earlier step is never free
// when probed, so it is never the target of a claim.)  The neighbouring bytes
// of the word are ANDed with ones and do not change.
// ---------------------------------------------------------------------------
struct VisitSTCON {
    uint8_t *status;
    uint8_t next_code;  // st_code(side, level + 1)
    int side;
    int *found;
    __device__ __forceinline__ unsigned *word(int v) const
    {
        return reinterpret_cast<unsigned *>(status + (v & ~3));
    }
    __device__ __forceinline__ static uint8_t byte_of(unsigned w, int v)
    {
        return (uint8_t)(w >> ((unsigned)(v & 3) * 8u));
    }
    __device__ __forceinline__ int probe(int v) const { return (int)__ldcg(word(v)); }
    __device__ __forceinline__ bool looks_free(int v, int p) const
    {
        return byte_of((unsigned)p, v) == ST_UNVISITED;
    }
    __device__ __forceinline__ int attempt(int v, int p) const
    {
        if (byte_of((unsigned)p, v) != ST_UNVISITED) return p;
        const unsigned sh = (unsigned)(v & 3) * 8u;
        return (int)atomicAnd(word(v), ~((0xFFu ^ (unsigned)next_code) << sh));
    }
    __device__ __forceinline__ int resolve(int v, int r) const
    {
        const uint8_t s = byte_of((unsigned)r, v);
        if (s == ST_UNVISITED) return v;
        if ((int)(s >> 7) != side) *(volatile int *)found = 1;
        return -1;
    }
    __device__ __forceinline__ int visit(int v) const { return resolve(v, attempt(v, probe(v))); }
};

struct VisitBFS {
    int32_t *levels;
    int32_t next_level;
    __device__ __forceinline__ int probe(int v) const { return ld_cg(levels + v); }
    __device__ __forceinline__ bool looks_free(int, int p) const { return p < 0; }
    __device__ __forceinline__ int attempt(int v, int p) const
    {
        return p >= 0 ? p : atomicCAS(levels + v, -1, next_level);
    }
    __device__ __forceinline__ int resolve(int v, int r) const { return r == -1 ? v : -1; }
    __device__ __forceinline__ int visit(int v) const { return resolve(v, attempt(v, probe(v))); }
};

// K neighbours at once: all K probes are issued before the first claim, and
// all K claims before the first claim's result is examined.
// v[k] < 0 marks an empty entry (c[k] = -1).
template <int K, class Vis>
__device__ __forceinline__ void visit_k(const Vis &vis, const int (&v)[K], int (&c)[K])
{
    int r[K];
#pragma unroll
    for (int k = 0; k < K; ++k) r[k] = v[k] >= 0 ? vis.probe(v[k]) : 0;
#pragma unroll
    for (int k = 0; k < K; ++k) r[k] = v[k] >= 0 ? vis.attempt(v[k], r[k]) : 0;
#pragma unroll
    for (int k = 0; k < K; ++k) c[k] = v[k] >= 0 ? vis.resolve(v[k], r[k]) : -1;
}

// The same, and the degrees d[k] (in the CSR `rp` the side expands next) of
// the claimed vertices: the row range of every neighbour whose probe found it
// free is read together with its claim, so the degree costs no round trip
// of its own after the claim returns.  A neighbour that another thread
// claims first costs two loads for nothing; the probe keeps those rare.
template <int K, class Vis>
__device__ __forceinline__ void visit_k_deg(const Vis &vis, const int32_t *__restrict__ rp,
                                            const int (&v)[K], int (&c)[K], int (&d)[K])
{
    int r[K];
#pragma unroll
    for (int k = 0; k < K; ++k) r[k] = v[k] >= 0 ? vis.probe(v[k]) : 0;
    int rb[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const bool f = v[k] >= 0 && vis.looks_free(v[k], r[k]);
        rb[k] = f ? __ldg(rp + v[k]) : 0;
        d[k] = f ? __ldg(rp + v[k] + 1) : 0;
    }
#pragma unroll
    for (int k = 0; k < K; ++k) r[k] = v[k] >= 0 ? vis.attempt(v[k], r[k]) : 0;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        c[k] = v[k] >= 0 ? vis.resolve(v[k], r[k]) : -1;
        d[k] -= rb[k];
    }
}

// ---------------------------------------------------------------------------
// Walk col[b, e) with `nlanes` threads (lane_idx in [0, nlanes)); every warp
// of the group must call it (loop trip counts are uniform per warp).  The
// aligned middle is read with two 16-byte loads per lane and round; the at
// most 6 unaligned entries at the ends are scalar loads of the group's first
// lanes that join the first round, so a row costs one dependent chain of
// loads, probes and claims per round and no extra one for its ends.
// ---------------------------------------------------------------------------
template <class Vis>
__device__ __forceinline__ void walk_range(const int32_t *__restrict__ col, int b, int e,
                                           int lane_idx, int nlanes, const Vis &vis,
                                           const AppendTarget &app)
{
    if (app.reads && lane_idx == 0 && e > b) atomicAdd(app.reads, (unsigned long long)(e - b));
    const int a = min((b + 3) & ~3, e);
    const int z = max(e & ~3, a);
    const int nhead = a - b, ntail = e - z;
    int hv = -1;
    if (lane_idx < nhead)
        hv = __ldg(col + b + lane_idx);
    else if (lane_idx < nhead + ntail)
        hv = __ldg(col + z + lane_idx - nhead);
    const int4 *col4 = reinterpret_cast<const int4 *>(col);
    const int k_end = z >> 2;
    int k0 = a >> 2;
    do {  // at least one round: it carries the scalar ends
        int v[9], c[9];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int k = k0 + h * nlanes + lane_idx;
            int4 x = make_int4(-1, -1, -1, -1);
            if (k < k_end) x = __ldg(col4 + k);
            v[4 * h + 0] = x.x;
            v[4 * h + 1] = x.y;
            v[4 * h + 2] = x.z;
            v[4 * h + 3] = x.w;
        }
        v[8] = hv;
        hv = -1;
        visit_k<9>(vis, v, c);
        warp_append<9>(c, app);
        k0 += 2 * nlanes;
    } while (k0 < k_end);
}

template <int T>
struct SmemTopDown {
    int stop;
    int warp_tot[T / 32];
    int total;
    int off[T];  // load-balanced search: exclusive prefix of the tile's row lengths
    int rbs[T];  // and the rows' first entries
    int wcnt[T / 32];           // per-warp claim buffers (AppendTarget::wlog)
    int wlog[T / 32][WARP_LOG];
};

// Block-wide inclusive scan of x; *total receives the sum.  All threads call.
template <int T>
__device__ __forceinline__ int block_inclusive_scan(int x, int *warp_tot, int *total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = warp_inclusive_scan(x);
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int w = lane < T / 32 ? warp_tot[lane] : 0;
        int wi = warp_inclusive_scan(w);
        if (lane < T / 32) warp_tot[lane] = wi - w;  // exclusive prefix of warps
        if (lane == 31) *total = wi;
    }
    __syncthreads();
    int r = incl + warp_tot[wid];
    return r;
}

// Hook for rows too long for one CTA: a published (shared) step hands them
// out as row jobs; everywhere else rows are walked in place.
struct NoSink {
    __device__ __forceinline__ bool push_row(int, int) const { return false; }
};

// Row jobs of a team step (grid or host-loop engines): rows longer than
// TEAM_SPLIT_E entries are cut into TEAM_SPLIT_E-entry pieces that the whole
// team walks after the step's tiles (cap == 0: no jobs, rows walked in place).
// Slots are taken with one atomicAdd on *njobs; a push that would pass cap
// writes nothing and its row is walked in place, so the pushes that succeed
// fill exactly the slots below the first failing one; *nok counts them and
// is what the team reads.
constexpr int TEAM_SPLIT_E = 4096;
struct TeamSink {
    int2 *jobs;
    int cap;
    int *njobs;
    int *nok;
    __device__ __forceinline__ bool push_row(int b, int e) const
    {
        if (cap == 0 || e - b <= TEAM_SPLIT_E) return false;
        const int n = (e - b + TEAM_SPLIT_E - 1) / TEAM_SPLIT_E;
        const int k = atomicAdd(njobs, n);
        if (k + n > cap) return false;  // job space exhausted: walk in place
        for (int i = 0; i < n; ++i)
            jobs[k + i] = make_int2(b + i * TEAM_SPLIT_E, min(e, b + (i + 1) * TEAM_SPLIT_E));
        atomicAdd(nok, n);
        return true;
    }
};

// ---------------------------------------------------------------------------
// Expand one tile by load-balanced search (after Merrill, Garland & Grimshaw's
// scan-based gather and Gunrock's LB strategy): the tile's rows are laid end
// to end by a CTA prefix scan, and entry e of that concatenation is read by
// thread e mod T, which finds its row by binary search over the prefix in
// shared memory.  Every thread reads GATHER_PER_THREAD entries per round
// whatever the mix of row lengths, so a tile costs ceil(total / (T * K))
// dependent rounds and three barriers; no row is walked by one warp or one
// CTA alone.  Rows longer than the sink's job length go to the sink first.
// ---------------------------------------------------------------------------
template <int T>
__device__ __forceinline__ int lb_row(const int *off, int e)
{
    int lo = 0, hi = T;  // off[0] = 0 <= e: the last row starting at or before e
#pragma unroll
    for (int s = T / 2; s > 0; s >>= 1) {
        const int mid = lo + s;
        if (mid < hi && off[mid] <= e) lo = mid;
    }
    return lo;
}

template <int T, class Vis, class Sink, int K = GATHER_PER_THREAD>
__device__ __forceinline__ void expand_lb(const int32_t *__restrict__ col, int rb, int re,
                                          const Vis &vis, const AppendTarget &app,
                                          SmemTopDown<T> &sm, const Sink &sink,
                                          const int *stop = nullptr)
{
    const int tid = threadIdx.x;
    if (re - rb > 0 && sink.push_row(rb, re)) rb = re;
    const int d = re - rb;
    const int incl = block_inclusive_scan<T>(d, sm.warp_tot, &sm.total);
    sm.off[tid] = incl - d;
    sm.rbs[tid] = rb;
    __syncthreads();
    const int total = sm.total;
    int nread = 0;
    AppendTarget bapp = app;  // claims gathered per warp, flushed below
    bapp.wlog = &sm.wlog[0][0];
    bapp.wcnt = sm.wcnt;
    if (lane_id() == 0) sm.wcnt[tid >> 5] = 0;
    __syncwarp();
    for (int base = 0; base < total; base += T * K) {
        // a set stop flag (the sides met) ends the tile within one round;
        // the test is warp-uniform, the rounds hold no CTA barrier
        if (stop && base > 0 && __any_sync(0xffffffffu, *(volatile const int *)stop != 0)) break;
        int v[K], c[K];
#pragma unroll
        for (int j = 0; j < K; ++j) {
            const int e = base + j * T + tid;
            v[j] = -1;
            if (e < total) {
                ++nread;
                const int r = lb_row<T>(sm.off, e);
                v[j] = __ldg(col + sm.rbs[r] + (e - sm.off[r]));
            }
        }
        visit_k<K>(vis, v, c);
        warp_append<K>(c, bapp);
    }
    warp_flush(bapp);
    if (app.reads) {
        nread = warp_sum_i(nread);
        if (lane_id() == 0 && nread) atomicAdd(app.reads, (unsigned long long)nread);
    }
    __syncthreads();  // the next tile rewrites off / rbs
}

// ---------------------------------------------------------------------------
// Variant 1, warp-centric: the warp expands the rows of its 32 lanes without
// any CTA barrier.  Rows longer than `big` go to the sink (row jobs) when it
// takes them.  The remaining rows are laid end to end by a warp prefix scan
// and read GATHER_PER_THREAD entries per lane and round (256 per round, the
// lanes of a row on consecutive entries); each lane finds the row of an
// entry by a 5-step shuffle search over the scan.  A frontier of a few long
// rows and many short ones thus costs ceil(entries / 256) dependent rounds,
// not one round per long row plus one per 32 short-row entries.
// ---------------------------------------------------------------------------
template <class Vis, class Sink, bool SPEC_DEG = false>
__device__ __forceinline__ void expand_warp(const int32_t *__restrict__ col, int rb, int re,
                                            const Vis &vis, const AppendTarget &app,
                                            const Sink &sink, int big)
{
    constexpr int K = GATHER_PER_THREAD;
    const int lane = (int)lane_id();
    if (re - rb > big && sink.push_row(rb, re)) rb = re;
    const int d = re - rb;
    const int incl = warp_inclusive_scan(d);
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int excl = incl - d;
    if (app.reads && lane == 0 && total > 0) atomicAdd(app.reads, (unsigned long long)total);
    for (int base = 0; base < total; base += 32 * K) {
        int v[K], c[K];
#pragma unroll
        for (int j = 0; j < K; ++j) {
            const int e = base + j * 32 + lane;
            int pos = 0;  // number of lanes whose rows end at or before entry e
#pragma unroll
            for (int s = 16; s > 0; s >>= 1) {
                const int w = __shfl_sync(0xffffffffu, incl, pos + s - 1);
                if (w <= e) pos += s;
            }
            const int owner = pos < 32 ? pos : 31;
            const int ob = __shfl_sync(0xffffffffu, rb, owner);
            const int oe = __shfl_sync(0xffffffffu, excl, owner);
            v[j] = e < total ? __ldg(col + ob + (e - oe)) : -1;
        }
        if constexpr (SPEC_DEG) {
            int dg[K];
            visit_k_deg<K>(vis, app.row_ptr, v, c, dg);
            warp_append_deg<K>(c, dg, app);
        } else {
            visit_k<K>(vis, v, c);
            warp_append<K>(c, app);
        }
    }
}

// Variant 2, thread per vertex: every lane walks its own row; the warp loop
// runs to the longest row of the 32 (best for uniform low degrees).  Rows of
// 64 or more entries are walked by the whole warp first, so no lane walks a
// long row alone.
template <class Vis, class Sink>
__device__ __forceinline__ void expand_thread(const int32_t *__restrict__ col, int rb, int re,
                                              const Vis &vis, const AppendTarget &app,
                                              const Sink &sink, int big)
{
    const int lane = (int)lane_id();
    if (re - rb > big && sink.push_row(rb, re)) rb = re;
    while (true) {
        unsigned m = __ballot_sync(0xffffffffu, re - rb >= 64);
        if (!m) break;
        int leader = __ffs(m) - 1;
        int b = __shfl_sync(0xffffffffu, rb, leader);
        int e = __shfl_sync(0xffffffffu, re, leader);
        if (lane == leader) rb = re;
        walk_range(col, b, e, lane, 32, vis, app);
    }
    const int len = re - rb;
    int mx = len;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (app.reads) {
        const int sum = warp_sum_i(len);
        if (lane == 0 && sum > 0) atomicAdd(app.reads, (unsigned long long)sum);
    }
    for (int k = 0; k < mx; ++k) {
        int c[1] = {-1};
        if (k < len) c[0] = vis.visit(__ldg(col + rb + k));
        warp_append<1>(c, app);
    }
}

// Top-down step for variants 1 and 2: 32-vertex chunks dealt to the team's
// warps; `stop_flag` is polled by each warp once per chunk.
template <int T, int VARIANT, class Vis, class Sink>
__device__ void topdown_warps(const int32_t *__restrict__ row_ptr, const int32_t *__restrict__ col,
                              const int32_t *frontier, int F, int team_rank, int team_size,
                              const Vis &vis, const AppendTarget &app, const int *stop_flag,
                              const Sink &sink)
{
    const int lane = (int)lane_id(), wid = threadIdx.x >> 5;
    constexpr int W = T / 32;
    const long long step = (long long)team_size * W;
    for (long long chunk = (long long)team_rank * W + wid; chunk * 32 < F; chunk += step) {
        if (stop_flag) {
            int st = lane == 0 ? *(volatile const int *)stop_flag : 0;
            if (__shfl_sync(0xffffffffu, st, 0)) break;
        }
        const long long i = chunk * 32 + lane;
        int rb = 0, re = 0;
        if (i < F) {
            int u = ld_cg(frontier + i);
            rb = __ldg(row_ptr + u);
            re = __ldg(row_ptr + u + 1);
        }
        if (VARIANT == 1)
            expand_warp(col, rb, re, vis, app, sink, TEAM_SPLIT_E);
        else
            expand_thread(col, rb, re, vis, app, sink, TEAM_SPLIT_E);
    }
}

// ---------------------------------------------------------------------------
// Top-down step over frontier[0, F).  Tiles of T frontier vertices are dealt
// round-robin to the team's CTAs.  `stop_flag` (nullable) is polled once per
// tile; a set flag ends the step early (used when the two sides have met).
// ---------------------------------------------------------------------------
template <int T, class Vis, class Sink>
__device__ void topdown_step(const int32_t *__restrict__ row_ptr, const int32_t *__restrict__ col,
                             const int32_t *frontier, int F, int team_rank, int team_size,
                             const Vis &vis, const AppendTarget &app, SmemTopDown<T> &sm,
                             const int *stop_flag, const Sink &sink, int tile_v = T)
{
    const int tid = threadIdx.x;
    if (F <= 32 && team_size == 1) {
        // a frontier of one warp's worth of short rows: that warp alone, no
        // CTA barrier (the caller synchronises after the step); every warp
        // reads the same rows and takes the same branch
        const int lane = (int)lane_id();
        int rb = 0, re = 0;
        if (lane < F) {
            const int u = ld_cg(frontier + lane);
            rb = __ldg(row_ptr + u);
            re = __ldg(row_ptr + u + 1);
        }
        if (warp_sum_i(re - rb) <= TINY_STEP_E) {
            if (tid < 32) expand_warp<Vis, NoSink, true>(col, rb, re, vis, app, NoSink{}, INT_MAX);
            return;
        }
    }
    // tiles of tile_v (<= T) frontier vertices, one per thread, dealt
    // round-robin: frontiers of high degree get tiles of fewer vertices
    const long long step = (long long)team_size * tile_v;
    for (long long base = (long long)team_rank * tile_v; base < F; base += step) {
        const long long i = base + tid;
        int rb = 0, re = 0;
        if (tid < tile_v && i < F) {
            int u = ld_cg(frontier + i);
            rb = __ldg(row_ptr + u);
            re = __ldg(row_ptr + u + 1);
        }
        if (team_size > 1)
            expand_lb<T, Vis, Sink, GATHER_TEAM>(col, rb, re, vis, app, sm, sink, stop_flag);
        else
            expand_lb<T>(col, rb, re, vis, app, sm, sink, stop_flag);
        // the stop flag matters only when another tile of this CTA follows
        if (stop_flag && base + step < F) {
            if (tid == 0) sm.stop = *(volatile const int *)stop_flag;
            __syncthreads();
            if (sm.stop) break;
        }
    }
}

// The team walks the row jobs [0, njobs) of a step, job j on team member
// j mod team_size; `stop_flag` (nullable) ends it early.  All threads call.
template <int T, class Vis>
__device__ void team_jobs(const int32_t *__restrict__ col, const int2 *jobs, int njobs,
                          int team_rank, int team_size, const Vis &vis, const AppendTarget &app,
                          SmemTopDown<T> &sm, const int *stop_flag)
{
    for (int j = team_rank; j < njobs; j += team_size) {
        if (stop_flag) {
            if (threadIdx.x == 0) sm.stop = *(volatile const int *)stop_flag;
            __syncthreads();
            if (sm.stop) break;
        }
        const int2 J = jobs[j];
        walk_range(col, J.x, J.y, threadIdx.x, T, vis, app);
    }
}

// Clear the status bytes of the claimed vertices in log entries [lo, hi)
// (entries below n0 are side 0's, read from the front; the rest side 1's,
// read from the back of the log), thread `first` of `stride`.  Eight log
// reads are in flight per thread before its stores: a byte store may alias
// the log as far as the compiler knows, so a plain loop waits for every
// read in turn.
__device__ __forceinline__ void clear_claimed(uint8_t *status, const int32_t *log, int cap,
                                              long long n0, long long lo, long long hi,
                                              long long first, long long stride)
{
    for (long long base = lo + first; base < hi; base += 8 * stride) {
        int v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const long long i = base + k * stride;
            v[k] = i < hi ? __ldcg(i < n0 ? log + i : log + (cap - 1 - (i - n0))) : -1;
        }
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (v[k] >= 0) status[v[k]] = ST_UNVISITED;
    }
}

// ---------------------------------------------------------------------------
// Bottom-up step.  Every vertex v of [0, nv) not yet owned by the expanding
// side scans its (reverse-graph) neighbours for one in the expanding side's
// frontier and stops at the first hit:
//   v unvisited                 -> v joins the side at level + 1
//   v owned by the other side,
//   at that side's frontier     -> meeting
// Only the thread that owns v writes v's status, so no CAS is needed, and the
// new code (level + 1) never equals the frontier code (level): no chaining.
// ---------------------------------------------------------------------------
struct BottomUpSTCON {
    uint8_t *status;
    uint8_t front_code;   // st_code(side, level)
    uint8_t next_code;    // st_code(side, level + 1)
    uint8_t other_front;  // st_code(other side, its radius)
    int *found;
    __device__ __forceinline__ int check(int v, const int32_t *__restrict__ row_ptr,
                                         const int32_t *__restrict__ col, int &inspected) const
    {
        uint8_t s = ld_cg_u8(status + v);
        bool unvisited = s == ST_UNVISITED;
        if (!unvisited && s != other_front) return -1;
        int b = __ldg(row_ptr + v), e = __ldg(row_ptr + v + 1);
        // neighbours in groups of BU_GROUP: the group's column and status
        // loads are independent and overlap; the first hit in row order
        // decides, and only the neighbours up to it count as inspected
        for (int j = b; j < e; j += BU_GROUP) {
            int u[BU_GROUP];
            uint8_t su[BU_GROUP];
#pragma unroll
            for (int k = 0; k < BU_GROUP; ++k) u[k] = j + k < e ? __ldg(col + j + k) : -1;
#pragma unroll
            for (int k = 0; k < BU_GROUP; ++k) su[k] = u[k] >= 0 ? ld_cg_u8(status + u[k]) : 0;
#pragma unroll
            for (int k = 0; k < BU_GROUP; ++k) {
                if (u[k] < 0) break;
                ++inspected;
                if (su[k] == front_code) {
                    if (unvisited) {
                        status[v] = next_code;
                        return v;
                    }
                    *(volatile int *)found = 1;
                    return -1;
                }
            }
        }
        return -1;
    }
};

struct BottomUpBFS {
    int32_t *levels;
    int32_t level;  // frontier level
    __device__ __forceinline__ int check(int v, const int32_t *__restrict__ row_ptr,
                                         const int32_t *__restrict__ col, int &inspected) const
    {
        if (ld_cg(levels + v) >= 0) return -1;
        int b = __ldg(row_ptr + v), e = __ldg(row_ptr + v + 1);
        for (int j = b; j < e; j += BU_GROUP) {
            int u[BU_GROUP], lu[BU_GROUP];
#pragma unroll
            for (int k = 0; k < BU_GROUP; ++k) u[k] = j + k < e ? __ldg(col + j + k) : -1;
#pragma unroll
            for (int k = 0; k < BU_GROUP; ++k) lu[k] = u[k] >= 0 ? ld_cg(levels + u[k]) : -1;
#pragma unroll
            for (int k = 0; k < BU_GROUP; ++k) {
                if (u[k] < 0) break;
                ++inspected;
                if (lu[k] == level) {
                    levels[v] = level + 1;
                    return v;
                }
            }
        }
        return -1;
    }
};

template <int T, class BU>
__device__ void bottomup_step(const int32_t *__restrict__ row_ptr, const int32_t *__restrict__ col,
                              int nv, int team_rank, int team_size, const BU &bu,
                              const AppendTarget &app, unsigned long long *inspected_total)
{
    int inspected = 0;
    for (long long v0 = (long long)team_rank * T; v0 < nv; v0 += (long long)team_size * T) {
        int v = (int)v0 + threadIdx.x;
        int c[1] = {-1};
        if (v < nv) c[0] = bu.check(v, row_ptr, col, inspected);
        warp_append<1>(c, app);
    }
    int w = warp_sum_i(inspected);
    if (lane_id() == 0 && w) atomicAdd(inspected_total, (unsigned long long)w);
}

}  // namespace fc
