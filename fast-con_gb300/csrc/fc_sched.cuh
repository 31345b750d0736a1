// fc_sched.cuh -- per-query control state shared by every engine: the
// counters a step updates, the scheduling decision, root set-up, results.
#pragma once

#include "fc_engine.h"
#include "fc_step.cuh"

namespace fc {

struct TeamCounters {
    int tail[2];
    int found;
    int err;
    unsigned long long deg[2];
    unsigned long long inspected;  // bottom-up adjacency reads
    int bar[2];
    int invalid;
    int pad;
};

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
};

__host__ __device__ inline void ql_start(QLocal &q, int two, int nv, long long ne, int s, int t,
                                         unsigned long long deg_s, unsigned long long deg_t)
{
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
        const long long nf = q.tail[side] - q.head[side];
        const long long mf = (long long)(q.dt[side] - q.dh[side]);
        if (mf < 8 * nf)
            q.variant = VAR_THREAD;  // low, even degrees: one lane per row
        else if (long_rows_split)
            q.variant = VAR_WARP;
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
    if (q.dir == DIR_TD) {
        const unsigned long long ef = q.dt[x] - q.dh[x];
        const unsigned long long nf = (unsigned long long)(q.tail[x] - q.head[x]);
        q.inspected += ef;
        q.alg_bytes += 12ull * nf + 8ull * ef + 8ull * nnew;
    } else {
        const unsigned long long k = bu_total - q.bu_seen;
        q.inspected += k;
        q.alg_bytes += 12ull * (unsigned long long)q.nv + 8ull * k + 8ull * nnew;
        q.bu_steps++;
    }
    q.bu_seen = bu_total;
    q.steps++;
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
                                                const int *stop)
{
    if (variant == VAR_WARP)
        topdown_warps<T, VAR_WARP>(gx.row_ptr, gx.col, frontier, F, team_rank, team_size, vis,
                                   app, stop);
    else if (variant == VAR_THREAD)
        topdown_warps<T, VAR_THREAD>(gx.row_ptr, gx.col, frontier, F, team_rank, team_size, vis,
                                     app, stop);
    else
        topdown_step<T>(gx.row_ptr, gx.col, frontier, F, team_rank, team_size, vis, app, sm, stop);
}

template <int T>
__device__ void run_step(int mode, const GraphPair &gp, int side, int dir, int level,
                         int other_radius, const int32_t *frontier, int F, int team_rank,
                         int team_size, uint8_t *status, int32_t *levels, int32_t *log, int cap,
                         int *tail_ctr, unsigned long long *deg_ctr, int *found,
                         unsigned long long *bu_ins, SmemTopDown<T> &sm, int variant = VAR_HYBRID)
{
    const DGraph &gx = side ? gp.rev : gp.fwd;
    AppendTarget app{log, cap, side, tail_ctr, deg_ctr, gx.row_ptr};
    if (dir == DIR_TD) {
        if (mode == MODE_BFS) {
            VisitBFS vis{levels, level + 1};
            topdown_variant<T>(variant, gx, frontier, F, team_rank, team_size, vis, app, sm,
                               nullptr);
        } else {
            VisitSTCON vis{status, st_code(side, level + 1), side, found};
            topdown_variant<T>(variant, gx, frontier, F, team_rank, team_size, vis, app, sm, found);
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

// Root initialisation (one thread).  Writes the counters, the roots' status
// (or level) and their log entries.
__device__ inline void init_roots(int mode, const GraphPair &gp, int s, int t, uint8_t *status,
                           int32_t *levels, int32_t *log, int cap, TeamCounters *tc)
{
    tc->found = 0;
    tc->inspected = 0;
    tc->invalid = 0;
    if (mode == MODE_BFS) {
        levels[s] = 0;
        log[0] = s;
        tc->tail[0] = 1;
        tc->tail[1] = 0;
        tc->deg[0] = (unsigned long long)(gp.fwd.row_ptr[s + 1] - gp.fwd.row_ptr[s]);
        tc->deg[1] = 0;
        return;
    }
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
