// fc_sched.cuh -- per-query control state shared by every engine: the
// counters a step updates, the scheduling decision, root set-up, results.
#pragma once

#include "fc_engine.h"
#include "fc_step.cuh"

namespace fc {

// The counters a team reads after a step, as they stood when the step's last
// CTA reached the grid barrier (grid_barrier_snap): faster CTAs may already be
// adding the next step's claims to the live counters.
struct TeamSnap {
    int tail[2];
    int found;
    int nok[2];
    int pad;
    unsigned long long deg[2];
    unsigned long long inspected;
    unsigned long long hist[2];
};

struct TeamCounters {
    int tail[2];
    int found;
    int err;
    unsigned long long deg[2];
    unsigned long long inspected;  // bottom-up adjacency reads
    int invalid;
    int pad;
    unsigned long long hist[2];     // claimed vertices per side of degree < 8 (low 32 bits)
                                    // and >= 128 (high 32 bits), learned schedule
    int njobs[2];                   // row-job slots taken, by step parity
    int nok[2];                     // row jobs written (a prefix of the slots)
    TeamSnap snap[2];               // by barrier generation parity
    // grid barrier words in a line of their own: waiting CTAs poll them
    // while the working ones update the counters above
    alignas(128) int bar[2];
};

struct SnapTeam {
    TeamCounters *tc;
    __device__ __forceinline__ void operator()(int p) const
    {
        TeamSnap &s = tc->snap[p];
        for (int x = 0; x < 2; ++x) {
            s.tail[x] = ld_cg(&tc->tail[x]);
            s.nok[x] = ld_cg(&tc->nok[x]);
            s.deg[x] = ld_cg_u64(&tc->deg[x]);
            s.hist[x] = ld_cg_u64(&tc->hist[x]);
        }
        s.found = ld_cg(&tc->found);
        s.inspected = ld_cg_u64(&tc->inspected);
    }
};

// degree bins of the frontier histogram: < 8, < 128, >= 128; the counters
// keep the outer two packed in one word (the middle one is the remainder)
__host__ __device__ inline int deg_bin(long long d) { return d < 8 ? 0 : (d < 128 ? 1 : 2); }
__host__ __device__ inline unsigned long long hist_word(long long d)
{
    return d < 8 ? 1ull : (d >= 128 ? (1ull << 32) : 0ull);
}

struct GraphPair {
    DGraph fwd, rev;
};
static_assert(sizeof(GraphPair) == sizeof(GraphPairH), "graph table layout");

enum { MODE_BFS = 0, MODE_STCON = 1 };
enum { DIR_TD = 0, DIR_BU = 1 };

// ---------------------------------------------------------------------------
// Per-query control state.  Every CTA of a team holds an identical copy; it
// is advanced from the team's counters after each barrier, so all copies take
// the same decisions without another barrier.
// ---------------------------------------------------------------------------
struct QLocal {
    int head[2], tail[2];
    unsigned long long dh[2], dt[2];
    int radius[2];
    int steps, bu_steps;
    unsigned long long inspected, bu_seen, alg_bytes;
    int done, connected, hops, escalate;
    int side, dir, variant;
    int two;
    int nv;
    long long ne;
    unsigned long long hh[2][2], ht[2][2];  // bins < 8 and >= 128 at head / tail
    int last_side;
    float feat[12];                          // features of the last decision
};

__host__ __device__ inline void ql_start(QLocal &q, int two, int nv, long long ne, int s, int t,
                                         unsigned long long deg_s, unsigned long long deg_t)
{
    for (int x = 0; x < 2; ++x)
        for (int b = 0; b < 2; ++b) q.hh[x][b] = q.ht[x][b] = 0;
    q.ht[0][0] = deg_s < 8;
    q.ht[0][1] = deg_s >= 128;
    if (two && s != t) {
        q.ht[1][0] = deg_t < 8;
        q.ht[1][1] = deg_t >= 128;
    }
    q.last_side = -1;
    q.head[0] = q.head[1] = 0;
    q.tail[0] = 1;
    q.tail[1] = (two && s != t) ? 1 : 0;
    q.dh[0] = q.dh[1] = 0;
    q.dt[0] = deg_s;
    q.dt[1] = (two && s != t) ? deg_t : 0;
    q.radius[0] = q.radius[1] = 0;
    q.steps = q.bu_steps = 0;
    q.inspected = q.bu_seen = q.alg_bytes = 0;
    q.done = 0;
    q.connected = 0;
    q.hops = -1;
    q.escalate = 0;
    q.side = 0;
    q.dir = DIR_TD;
    q.variant = 0;
    q.two = two;
    q.nv = nv;
    q.ne = ne;
    if (two && s == t) {
        q.done = 1;
        q.connected = 1;
        q.hops = 0;
    }
}

// Expansion variants of a top-down step (answers never depend on them):
enum {
    VAR_HYBRID = 0,  // CTA / warp / scan classes per row length (CTA barriers)
    VAR_WARP = 1,    // warp-centric, no CTA barriers
    VAR_THREAD = 2,  // one lane per row
};

// Choose the next step.  allow_bu = 0 where a bottom-up step would be run by
// one CTA (it scans every vertex).  bu_level_cap limits bottom-up to levels
// whose status code is exact (s-t status bytes hold min(level, 126)).
// long_rows_split: the engine hands very long rows to many CTAs, so the
// warp-centric variant is safe for frontiers with hubs.
__host__ __device__ inline void ql_decide(QLocal &q, int sched, int allow_bu, int bu_level_cap,
                                          int long_rows_split = 0, int force_variant = -1)
{
    int side;
    if (!q.two)
        side = 0;
    else if (sched == FC_SCHED_PLAIN)
        side = q.steps & 1;
    else {
        unsigned long long m0 = q.dt[0] - q.dh[0], m1 = q.dt[1] - q.dh[1];
        side = m0 <= m1 ? 0 : 1;
    }
    q.side = side;
    q.dir = DIR_TD;
    q.variant = VAR_HYBRID;
    if (sched != FC_SCHED_PLAIN) {
        // low average degree: one lane per row; otherwise the CTA hybrid,
        // which measured fastest on R-MAT frontiers in every engine (the
        // warp-centric variant is left to the learned schedule)
        const long long nf = q.tail[side] - q.head[side];
        const long long mf = (long long)(q.dt[side] - q.dh[side]);
        if (mf < 8 * nf) q.variant = VAR_THREAD;
        (void)long_rows_split;
    }
    if (sched != FC_SCHED_PLAIN && allow_bu && q.radius[side] + 1 <= bu_level_cap) {
        long long mf = (long long)(q.dt[side] - q.dh[side]);
        long long unexplored = q.ne - (long long)(q.dt[0] + q.dt[1]);
        long long nf = q.tail[side] - q.head[side];
        // Beamer, Asanovic & Patterson (SC'12) thresholds: alpha = 14, beta = 24
        if (mf * 14 > unexplored && nf * 24 > q.nv) q.dir = DIR_BU;
    }
    if (force_variant >= 0) q.variant = force_variant;
}

// Advance after the step on q.side finished (counters final).
__host__ __device__ inline void ql_update(QLocal &q, int found, int tail_x,
                                          unsigned long long deg_x, unsigned long long bu_total)
{
    const int x = q.side;
    // algorithmic bytes of the step (4-byte status words, 8 bytes per row
    // range, 4 per column entry and per queue entry):
    //   top-down   4|F| + 8|F| + 4 E_F + 4 E_F + 4|N| + 4|N|
    //   bottom-up  sum over scanned v of (4 + 8 + 8 k_v), plus 8|N|
    const unsigned long long nnew = (unsigned long long)(tail_x - q.tail[x]);
    // entries actually read (the steps add them to one counter): a meeting
    // step that stops early reads fewer than its frontier's degree sum
    const unsigned long long k = bu_total - q.bu_seen;
    if (q.dir == DIR_TD) {
        const unsigned long long nf = (unsigned long long)(q.tail[x] - q.head[x]);
        q.inspected += k;
        q.alg_bytes += 12ull * nf + 8ull * k + 8ull * nnew;
    } else {
        q.inspected += k;
        q.alg_bytes += 12ull * (unsigned long long)q.nv + 8ull * k + 8ull * nnew;
        q.bu_steps++;
    }
    q.bu_seen = bu_total;
    q.steps++;
    q.last_side = x;
    if (found && q.two) {
        q.done = 1;
        q.connected = 1;
        q.hops = q.radius[x] + 1 + q.radius[1 - x];
    }
    q.head[x] = q.tail[x];
    q.tail[x] = tail_x;
    q.dh[x] = q.dt[x];
    q.dt[x] = deg_x;
    q.radius[x]++;
    if (!q.done && q.tail[x] == q.head[x]) {
        q.done = 1;
        q.connected = 0;
        q.hops = -1;
    }
}

// After ql_update for side x: move the side's histogram window forward
// (`word` = the side's packed counter).
__host__ __device__ inline void ql_update_hist(QLocal &q, int x, unsigned long long word)
{
    q.hh[x][0] = q.ht[x][0];
    q.hh[x][1] = q.ht[x][1];
    q.ht[x][0] = word & 0xFFFFFFFFull;
    q.ht[x][1] = word >> 32;
}

// ---------------------------------------------------------------------------
// Learned schedule.  Twelve features per decision (all from integer counters,
// scaled so that graphs of different sizes give comparable values):
//   0,1   log2(1 + frontier vertices) / log2(2 + nv), side 0 and side 1
//   2,3   log2(1 + frontier adjacency entries) / log2(2 + ne), sides 0 and 1
//   4     unexplored fraction: adjacency entries of unclaimed vertices / ne
//   5     side expanded last (0 or 1; 0.5 before the first step)
//   6,7   side 0 frontier: fraction of degree < 8, fraction of degree >= 128
//   8,9   side 1 frontier: the same
//   10,11 log2(1 + radius) / 8 of side 0, side 1 (levels expanded so far)
// MLP 12 -> 32 (ReLU) -> 32 (ReLU) -> 7 logits: side (2), direction (2),
// expansion variant (3).  1,703 float parameters in this order:
//   W1[32][12], b1[32], W2[32][32], b2[32], W3[7][32], b3[7];
// optionally followed by the feature box of the training data, lo[12] and
// hi[12]: outside the box the network is not consulted (the heuristic
// decides), so graphs unlike the training graphs fall back to the heuristic.
// ---------------------------------------------------------------------------
constexpr int MLP_IN = 12, MLP_H = 32, MLP_OUT = 7;
constexpr int MLP_W1 = 0, MLP_B1 = MLP_W1 + MLP_H * MLP_IN, MLP_W2 = MLP_B1 + MLP_H,
              MLP_B2 = MLP_W2 + MLP_H * MLP_H, MLP_W3 = MLP_B2 + MLP_H,
              MLP_B3 = MLP_W3 + MLP_OUT * MLP_H, MLP_PARAMS = MLP_B3 + MLP_OUT;
constexpr int MLP_BOX = MLP_PARAMS, MLP_STORE = MLP_PARAMS + 2 * MLP_IN;
// Slack of the trust region in ql_apply_logits (adjacency entries).
constexpr long long MLP_MIN_EDGES = 1024;
// The network is consulted only where its answer can change the step: the
// heuristic's step reads at least MLP_CONSULT_EDGES entries (smaller steps
// cost little whichever way they go) and the other side's step lies inside
// the trust region (otherwise the side stays, and the direction and variant
// heads are not applied against the heuristic's).  On R-MAT 24 batches this
// cut the learned schedule's time 0.288 -> 0.276 ms (threshold 1,024 and
// every step consulted before) for 1-2% more entries read.
constexpr long long MLP_CONSULT_EDGES = 4096;

__host__ __device__ inline bool mlp_worth(const QLocal &q)
{
    const int x = q.side;
    const unsigned long long mh = q.dt[x] - q.dh[x];
    if (!q.two || (long long)mh < MLP_CONSULT_EDGES) return false;
    const unsigned long long mw = q.dt[1 - x] - q.dh[1 - x];
    return mw <= 2 * mh + (unsigned long long)MLP_MIN_EDGES;
}
static_assert(MLP_PARAMS == 1703, "parameter count");

__host__ __device__ inline void ql_features(const QLocal &q, float *f)
{
    // single precision throughout: FP64 is slow on this part and the
    // features need no more than float resolution
    const float n0 = (float)(q.tail[0] - q.head[0]), n1 = (float)(q.tail[1] - q.head[1]);
    const float m0 = (float)(q.dt[0] - q.dh[0]), m1 = (float)(q.dt[1] - q.dh[1]);
    long long un = q.ne - (long long)(q.dt[0] + q.dt[1]);
    if (un < 0) un = 0;
    const float lv = 1.f / log2f(2.f + (float)q.nv), le = 1.f / log2f(2.f + (float)q.ne);
    f[0] = log2f(1.f + n0) * lv;
    f[1] = log2f(1.f + n1) * lv;
    f[2] = log2f(1.f + m0) * le;
    f[3] = log2f(1.f + m1) * le;
    f[4] = q.ne > 0 ? (float)un / (float)q.ne : 0.f;
    f[5] = q.last_side < 0 ? 0.5f : (float)q.last_side;
    for (int x = 0; x < 2; ++x) {
        // every claim is counted, so the bins of the frontier add up to its size
        const float tot = (float)(q.tail[x] - q.head[x]);
        f[6 + 2 * x] = tot > 0.f ? (float)(q.ht[x][0] - q.hh[x][0]) / tot : 0.f;
        f[7 + 2 * x] = tot > 0.f ? (float)(q.ht[x][1] - q.hh[x][1]) / tot : 0.f;
        f[10 + x] = log2f(1.f + (float)q.radius[x]) * 0.125f;
    }
}

// True when every feature lies inside the training box (W[MLP_BOX..]).
__host__ __device__ inline bool mlp_in_box(const float *W, const float *f)
{
    bool in = true;
    for (int i = 0; i < MLP_IN; ++i)
        in = in && f[i] >= W[MLP_BOX + i] && f[i] <= W[MLP_BOX + MLP_IN + i];
    return in;
}

// Forward pass by one thread (host-loop engine on the host, grid engine on
// the device).
__host__ __device__ inline void mlp_forward_scalar(const float *W, const float *f, float *out)
{
    float h1[MLP_H], h2[MLP_H];
    for (int j = 0; j < MLP_H; ++j) {
        float a = W[MLP_B1 + j];
        for (int i = 0; i < MLP_IN; ++i) a += W[MLP_W1 + j * MLP_IN + i] * f[i];
        h1[j] = a > 0.f ? a : 0.f;
    }
    for (int j = 0; j < MLP_H; ++j) {
        float a = W[MLP_B2 + j];
        for (int k = 0; k < MLP_H; ++k) a += W[MLP_W2 + j * MLP_H + k] * h1[k];
        h2[j] = a > 0.f ? a : 0.f;
    }
    for (int o = 0; o < MLP_OUT; ++o) {
        float a = W[MLP_B3 + o];
        for (int k = 0; k < MLP_H; ++k) a += W[MLP_W3 + o * MLP_H + k] * h2[k];
        out[o] = a;
    }
}

// Forward pass by one warp: lane j computes hidden unit j of both layers; the
// 7 outputs are warp reductions.  Every lane returns all 7 logits.  W is the
// CTA's shared-memory copy of the weights (the batched engine stages them
// once per launch), so no step waits on an L2 round trip for them.
__device__ __forceinline__ void mlp_forward_warp(const float *W, const float *f, float *out)
{
    const int j = (int)lane_id();
    float a = W[MLP_B1 + j];
#pragma unroll
    for (int i = 0; i < MLP_IN; ++i) a += W[MLP_W1 + j * MLP_IN + i] * f[i];
    const float h1 = a > 0.f ? a : 0.f;
    a = W[MLP_B2 + j];
#pragma unroll 8
    for (int k = 0; k < MLP_H; ++k) a += W[MLP_W2 + j * MLP_H + k] * __shfl_sync(0xffffffffu, h1, k);
    const float h2 = a > 0.f ? a : 0.f;
#pragma unroll
    for (int o = 0; o < MLP_OUT; ++o) {
        float v = W[MLP_W3 + o * MLP_H + j] * h2;
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
        out[o] = v + W[MLP_B3 + o];
    }
}

// Turn logits into the step, within the engine's constraints (one side only
// for BFS, bottom-up only where allowed).  Each head overrides the
// heuristic's choice (already in q) only when confident: a logit margin above
// MLP_MARGIN over every other class (softmax probability above 0.75 for two
// classes); otherwise the fixed-threshold heuristic stands.
constexpr float MLP_MARGIN = 1.0986f;  // ln 3

__host__ __device__ inline void ql_apply_logits(QLocal &q, const float *o, int allow_bu,
                                                int bu_level_cap)
{
    const int side0 = q.side;
    if (q.two) {
        const float d = o[1] - o[0];
        const int want = d > MLP_MARGIN ? 1 : (d < -MLP_MARGIN ? 0 : side0);
        // trust region: the other side only while its step is at most twice
        // the heuristic's (a wrong call then costs at most one such step)
        const unsigned long long mw = q.dt[want] - q.dh[want];
        const unsigned long long mh = q.dt[side0] - q.dh[side0];
        if (want != side0 && mw <= 2 * mh + (unsigned long long)MLP_MIN_EDGES) q.side = want;
    }
    // direction stays the heuristic's (top-down when the side changed): a
    // bottom-up step scans every vertex of the graph, and in batches the
    // network's bottom-up calls cost more than the entries they saved (three
    // of them took a 512-graph batch from 0.54 to 0.81 ms); the direction
    // head is trained and traced but not applied
    (void)allow_bu;
    (void)bu_level_cap;
    if (q.side != side0) q.dir = DIR_TD;
    int v = 0;
    if (o[5] > o[4 + v]) v = 1;
    if (o[6] > o[4 + v]) v = 2;
    float second = -3.0e38f;
    for (int k = 0; k < 3; ++k)
        if (k != v && o[4 + k] > second) second = o[4 + k];
    if (o[4 + v] - second > MLP_MARGIN) q.variant = v;
}

// Scripted action byte: bit 0 side, bit 1 bottom-up, bits 2-3 variant + 1
// (0 = the schedule's variant); 0xFF = no script for this step.
__host__ __device__ inline void ql_apply_script(QLocal &q, unsigned char a, int allow_bu,
                                                int bu_level_cap)
{
    q.side = q.two ? (a & 1) : 0;
    q.dir = ((a >> 1) & 1) && allow_bu && q.radius[q.side] + 1 <= bu_level_cap ? DIR_BU : DIR_TD;
    const int v = (a >> 2) & 3;
    if (v) q.variant = v - 1;
}

__device__ __forceinline__ const int32_t *ql_frontier(const QLocal &q, const int32_t *log, int cap,
                                                     int x, int *F)
{
    *F = q.tail[x] - q.head[x];
    return x == 0 ? log + q.head[0] : log + (cap - q.tail[1]);
}

// ---------------------------------------------------------------------------
// One step for a team of CTAs.
// ---------------------------------------------------------------------------
template <int T, class Vis>
__device__ __forceinline__ void topdown_variant(int variant, const DGraph &gx,
                                                const int32_t *frontier, int F, int team_rank,
                                                int team_size, const Vis &vis,
                                                const AppendTarget &app, SmemTopDown<T> &sm,
                                                const int *stop, const TeamSink &sink,
                                                int tile_v = T)
{
    if (variant == VAR_WARP)
        topdown_warps<T, VAR_WARP>(gx.row_ptr, gx.col, frontier, F, team_rank, team_size, vis,
                                   app, stop, sink);
    else if (variant == VAR_THREAD)
        topdown_warps<T, VAR_THREAD>(gx.row_ptr, gx.col, frontier, F, team_rank, team_size, vis,
                                     app, stop, sink);
    else
        topdown_step<T>(gx.row_ptr, gx.col, frontier, F, team_rank, team_size, vis, app, sm, stop,
                        sink, tile_v);
}

template <int T>
__device__ void run_step(int mode, const GraphPair &gp, int side, int dir, int level,
                         int other_radius, const int32_t *frontier, int F, int team_rank,
                         int team_size, uint8_t *status, int32_t *levels, int32_t *log, int cap,
                         int *tail_ctr, unsigned long long *deg_ctr, int *found,
                         unsigned long long *bu_ins, SmemTopDown<T> &sm, int variant = VAR_HYBRID,
                         unsigned long long *hist = nullptr,
                         TeamSink sink = TeamSink{nullptr, 0, nullptr, nullptr},
                         int tile_v = T)
{
    const DGraph &gx = side ? gp.rev : gp.fwd;
    // top-down reads and bottom-up checks add to the same counter
    AppendTarget app{log, cap, side, tail_ctr, deg_ctr, gx.row_ptr, hist, bu_ins};
    if (dir == DIR_TD) {
        if (mode == MODE_BFS) {
            VisitBFS vis{levels, level + 1};
            topdown_variant<T>(variant, gx, frontier, F, team_rank, team_size, vis, app, sm,
                               nullptr, sink, tile_v);
        } else {
            VisitSTCON vis{status, st_code(side, level + 1), side, found};
            topdown_variant<T>(variant, gx, frontier, F, team_rank, team_size, vis, app, sm, found,
                               sink, tile_v);
        }
    } else {
        const DGraph &gr = side ? gp.fwd : gp.rev;
        if (mode == MODE_BFS) {
            BottomUpBFS bu{levels, level};
            bottomup_step<T>(gr.row_ptr, gr.col, gr.nv, team_rank, team_size, bu, app, bu_ins);
        } else {
            BottomUpSTCON bu{status, st_code(side, level), st_code(side, level + 1),
                             st_code(1 - side, other_radius), found};
            bottomup_step<T>(gr.row_ptr, gr.col, gr.nv, team_rank, team_size, bu, app, bu_ins);
        }
    }
}

// The row jobs a top-down step left (team engines), with the step's visitor.
template <int T>
__device__ void run_team_jobs(int mode, const GraphPair &gp, int side, int level, const int2 *jobs,
                              int njobs, int team_rank, int team_size, uint8_t *status,
                              int32_t *levels, int32_t *log, int cap, int *tail_ctr,
                              unsigned long long *deg_ctr, int *found, SmemTopDown<T> &sm,
                              unsigned long long *hist, unsigned long long *reads)
{
    const DGraph &gx = side ? gp.rev : gp.fwd;
    AppendTarget app{log, cap, side, tail_ctr, deg_ctr, gx.row_ptr, hist, reads};
    if (mode == MODE_BFS) {
        VisitBFS vis{levels, level + 1};
        team_jobs<T>(gx.col, jobs, njobs, team_rank, team_size, vis, app, sm, nullptr);
    } else {
        VisitSTCON vis{status, st_code(side, level + 1), side, found};
        team_jobs<T>(gx.col, jobs, njobs, team_rank, team_size, vis, app, sm, found);
    }
}

// Root initialisation (one thread).  Writes the counters, the roots' status
// (or level) and their log entries.
__device__ inline void init_roots(int mode, const GraphPair &gp, int s, int t, uint8_t *status,
                           int32_t *levels, int32_t *log, int cap, TeamCounters *tc)
{
    tc->found = 0;
    tc->inspected = 0;
    tc->invalid = 0;
    tc->njobs[0] = tc->njobs[1] = 0;
    tc->nok[0] = tc->nok[1] = 0;
    for (int x = 0; x < 2; ++x)
        tc->hist[x] = 0;
    if (mode == MODE_BFS) {
        levels[s] = 0;
        log[0] = s;
        tc->tail[0] = 1;
        tc->tail[1] = 0;
        tc->deg[0] = (unsigned long long)(gp.fwd.row_ptr[s + 1] - gp.fwd.row_ptr[s]);
        tc->deg[1] = 0;
        tc->hist[0] = hist_word((long long)tc->deg[0]);
        return;
    }
    tc->hist[0] = hist_word((long long)(gp.fwd.row_ptr[s + 1] - gp.fwd.row_ptr[s]));
    if (s != t) tc->hist[1] = hist_word((long long)(gp.rev.row_ptr[t + 1] - gp.rev.row_ptr[t]));
    status[s] = st_code(0, 0);
    log[0] = s;
    tc->tail[0] = 1;
    tc->deg[0] = (unsigned long long)(gp.fwd.row_ptr[s + 1] - gp.fwd.row_ptr[s]);
    if (s != t) {
        status[t] = st_code(1, 0);
        log[cap - 1] = t;
        tc->tail[1] = 1;
        tc->deg[1] = (unsigned long long)(gp.rev.row_ptr[t + 1] - gp.rev.row_ptr[t]);
    } else {
        tc->tail[1] = 0;
        tc->deg[1] = 0;
        tc->found = 1;
    }
}

__device__ __forceinline__ void write_result(int q, const QLocal &ql, int32_t *out_conn,
                                             int32_t *out_hops, QueryStat *qs, int escalated)
{
    if (!escalated) {
        if (out_conn) out_conn[q] = ql.connected;
        if (out_hops) out_hops[q] = ql.hops;
    }
    if (qs) {
        QueryStat r;
        r.inspected = (long long)ql.inspected;
        r.alg_bytes = (long long)ql.alg_bytes;
        r.steps = ql.steps;
        r.bu_steps = ql.bu_steps;
        r.visited = ql.tail[0] + ql.tail[1];
        r.visited_deg = (long long)(ql.dt[0] + ql.dt[1]);
        r.escalated = escalated;
        if (escalated) {
            // the persistent engine rewrites the record; keep the CTA's part
            qs[q].escalated = 1;
        } else {
            r.escalated = qs[q].escalated;
            qs[q] = r;
        }
    }
}

}  // namespace fc
