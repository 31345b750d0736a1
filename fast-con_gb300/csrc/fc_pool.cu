// fc_pool.cu -- the work-sharing ("pool") engine: many s-t queries (or one
// BFS) per cooperative launch, with no host round trip and no grid barrier.
//
// Every CTA owns a slot (status bytes, visit log) and pulls queries from a
// global counter; small steps run privately inside the CTA with __syncthreads
// between levels (the one-CTA-per-source shape of BFS_4K_BLOCK,
// BFS_4K_BLOCK/.../BFS_WE_Block.cu:33-147).  A step whose frontier reads more
// than `private_edges` adjacency entries, every bottom-up step, and every step
// of a query run in exclusive mode is *published*: its work is cut into tiles
// (256 frontier vertices, 8192 vertices for bottom-up, 8192 log entries for the
// final status reset) that any CTA may claim.  Rows longer than 8192 entries
// found inside a tile become extra "row jobs", so a hub vertex is spread over
// many CTAs.  The owner claims tiles of its own step first, then claims tiles
// of other slots while it waits for its step to complete; CTAs without queries
// left only claim tiles.
//
// Claiming: slot.next packs {seq:20, ntiles:22, next tile:22} in one 64-bit
// word.  The owner publishes a step by writing its description and then
// storing a new seq (release).  Every CTA, the owner included, claims tile i
// of step seq with a CAS on the whole word, so a claim can never land on a
// newer step and the tile counter never passes ntiles.  A row job adds one to
// ntiles with an atomic
// add on the same word after writing its descriptor; a helper that claims a
// job waits (bounded) for the descriptor's seq stamp.  The step is complete
// when `done` (read first) equals ntiles (read second).
//
// All CTAs of the launch are co-resident (cooperative launch), so waiting on
// another CTA's progress is safe; every wait is still bounded by %globaltimer
// and reports FC_ERR_TIMEOUT through ctr[3] instead of hanging.
#include <climits>
#include <cstring>

#include "fc_pool.h"
#include "fc_sched.cuh"

namespace fc {

constexpr int POOL_TILE_V = 8192;    // vertices per bottom-up tile
constexpr int POOL_TILE_R = 8192;    // log entries per reset tile
constexpr int POOL_JOBS = 16384;     // row jobs per slot and step
// An owner waiting for the helpers of its published step takes other slots'
// tiles meanwhile (throughput) or only waits (its own query's latency).
constexpr bool OWNER_HELPS = true;
constexpr unsigned long long PK_MASK = (1ull << 22) - 1;
constexpr unsigned long long POOL_IDLE_NS = 4000000000ull;  // 4 s without progress

enum { DIR_RESET = 2 };
enum { CTR_NEXT = 0, CTR_FINISHED = 1, CTR_SPILL = 2, CTR_ERR = 3, CTR_INVALID = 4 };

__host__ __device__ inline unsigned long long pk(unsigned seq, unsigned long long ntiles,
                                                 unsigned long long tile)
{
    return ((unsigned long long)(seq & 0xFFFFFu) << 44) | (ntiles << 22) | tile;
}
__device__ __forceinline__ unsigned pk_seq(unsigned long long v) { return (unsigned)(v >> 44); }
__device__ __forceinline__ int pk_ntiles(unsigned long long v) { return (int)((v >> 22) & PK_MASK); }
__device__ __forceinline__ int pk_tile(unsigned long long v) { return (int)(v & PK_MASK); }

struct RowJob {
    int b, e;
    unsigned seq;
    int pad;
};

// Step description: written by the owner before it publishes the step.
struct PoolDesc {
    int q, gidx, mode, side, dir, level, other_radius, F, front_off, nvt, cap, nreset, variant;
    int tile_v;     // top-down: frontier vertices per tile (< T, or a multiple of T)
    int split_e;    // row-job length
    int track_hist; // count claimed vertices per degree bin (learned schedule)
    uint8_t *status;
    int32_t *levels;
    int32_t *log;
};

struct alignas(256) PoolSlot {
    unsigned long long next;
    int done;
    int njobs;
    PoolDesc d;
    TeamCounters tc;
};

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Row jobs of one published step.
struct SlotSink {
    PoolSlot *slot;
    RowJob *jobs;
    unsigned seq;
    int split;  // job length
    __device__ bool push_row(int b, int e) const
    {
        if (e - b <= split) return false;
        int n = (e - b + split - 1) / split;
        int k = atomicAdd(&slot->njobs, n);
        if (k + n > POOL_JOBS) return false;  // job space exhausted: walk in place
        // every descriptor, one fence, then the seq stamps a claimer waits
        // for (a fence per job serialised hub rows of ~50 jobs)
        for (int i = 0; i < n; ++i) {
            RowJob &J = jobs[k + i];
            J.b = b + i * split;
            J.e = min(e, J.b + split);
        }
        __threadfence();
        for (int i = 0; i < n; ++i) *(volatile unsigned *)&jobs[k + i].seq = seq;
        __threadfence();
        atomicAdd(&slot->next, (unsigned long long)n << 22);
        return true;
    }
};

template <int T>
struct SmemPool {
    SmemTopDown<T> td;
    QLocal ql;
    PoolDesc d;    // description of the step whose tile this CTA is running
    PoolDesc own;  // the owner's description of its query's steps (thread 0 writes it)
    int q, li, publish, flag, cand, claimed, cursor;
    unsigned seq, my_seq;
    int err;
    int nq;            // queries of the launch
    int tail;          // every query has an owner: idle CTAs are about
    unsigned backoff;  // idle polling pause, ns
    unsigned long long t_idle, t_step;
    // the owner's query counters while it runs steps alone: shared-memory
    // atomics and reads instead of global ones on every step's critical
    // path; copied to the slot before a published step and back after it
    TeamCounters stc;
    float mlp[MLP_STORE];  // the learned schedule's weights and box, staged per launch
};

// counters the helpers of a published step add to
__device__ __forceinline__ void counters_to_slot(PoolSlot *my, const TeamCounters &c)
{
    for (int x = 0; x < 2; ++x) {
        my->tc.tail[x] = c.tail[x];
        my->tc.deg[x] = c.deg[x];
        my->tc.hist[x] = c.hist[x];
    }
    my->tc.found = c.found;
    my->tc.inspected = c.inspected;
}

__device__ __forceinline__ void counters_from_slot(TeamCounters &c, const PoolSlot *my)
{
    for (int x = 0; x < 2; ++x) {
        c.tail[x] = ld_cg(&my->tc.tail[x]);
        c.deg[x] = ld_cg_u64(&my->tc.deg[x]);
        c.hist[x] = ld_cg_u64(&my->tc.hist[x]);
    }
    c.found = ld_cg(&my->tc.found);
    c.inspected = ld_cg_u64(&my->tc.inspected);
}

// Expand the tile's rows (one per thread) with the step's variant; rows longer
// than a row job go to the sink in every variant.
template <int T, class Vis>
__device__ __forceinline__ void pool_expand(int variant, const int32_t *__restrict__ col, int rb,
                                            int re, const Vis &vis, const AppendTarget &app,
                                            SmemTopDown<T> &td, const SlotSink &sink,
                                            const int *stop)
{
    if (variant == VAR_WARP)
        expand_warp(col, rb, re, vis, app, sink, sink.split);
    else if (variant == VAR_THREAD)
        expand_thread(col, rb, re, vis, app, sink, sink.split);
    else
        expand_lb<T>(col, rb, re, vis, app, td, sink, stop);
}

// ---------------------------------------------------------------------------
// One tile of a published step (any CTA).  sm.d holds the step description.
// ---------------------------------------------------------------------------
template <int T>
__device__ void pool_tile(const PoolArgs &a, PoolSlot *slot, int tile, unsigned seq,
                          SmemPool<T> &sm)
{
    const PoolDesc &d = sm.d;
    const int tid = threadIdx.x;
    if (d.dir == DIR_RESET) {
        const int n0 = d.F;  // entries of side 0; the rest belong to side 1
        const int lo = tile * POOL_TILE_R, hi = min(d.nreset, lo + POOL_TILE_R);
        clear_claimed(d.status, d.log, d.cap, n0, lo, hi, tid, T);
        return;
    }
    // already met: skip the tile (one read, shared, so the whole CTA agrees)
    __shared__ int s_met;
    if (tid == 0) s_met = d.mode == MODE_STCON && ld_cg(&slot->tc.found);
    __syncthreads();
    if (s_met) return;
    const GraphPair &gp = a.graphs[d.gidx];
    const DGraph &gx = d.side ? gp.rev : gp.fwd;
    AppendTarget app{d.log, d.cap, d.side, &slot->tc.tail[d.side], &slot->tc.deg[d.side],
                     gx.row_ptr, d.track_hist ? &slot->tc.hist[d.side] : nullptr, &slot->tc.inspected};
    if (tile >= d.nvt) {
        // row job: wait (bounded) until its descriptor carries this step's seq
        RowJob *J = a.jobs + (size_t)(slot - a.slots) * POOL_JOBS + (tile - d.nvt);
        __shared__ int jb, je;
        if (tid == 0) {
            unsigned long long t0 = global_timer_ns();
            jb = je = 0;
            while (true) {
                if (*(volatile unsigned *)&J->seq == seq) {
                    jb = *(volatile int *)&J->b;
                    je = *(volatile int *)&J->e;
                    break;
                }
                if (global_timer_ns() - t0 > BARRIER_TIMEOUT_NS) {
                    atomicCAS(&a.ctr[CTR_ERR], 0, FC_ERR_TIMEOUT);
                    break;
                }
                __nanosleep(32);
            }
        }
        __syncthreads();
        const int b = jb, e = je;
        __syncthreads();
        if (d.mode == MODE_BFS) {
            VisitBFS vis{d.levels, d.level + 1};
            walk_range(gx.col, b, e, tid, T, vis, app);
        } else {
            VisitSTCON vis{d.status, st_code(d.side, d.level + 1), d.side, &slot->tc.found};
            walk_range(gx.col, b, e, tid, T, vis, app);
        }
        return;
    }
    if (d.dir == DIR_TD) {
        SlotSink sink{slot, a.jobs + (size_t)(slot - a.slots) * POOL_JOBS, seq, d.split_e};
        const long long t0 = (long long)tile * d.tile_v;
        const long long t1 = min((long long)d.F, t0 + d.tile_v);
        for (long long base = t0; base < t1; base += T) {  // uniform loop
            const long long i = base + tid;
            int rb = 0, re = 0;
            if (i < t1) {
                int u = ld_cg(d.log + d.front_off + i);
                rb = __ldg(gx.row_ptr + u);
                re = __ldg(gx.row_ptr + u + 1);
            }
            if (d.mode == MODE_BFS) {
                VisitBFS vis{d.levels, d.level + 1};
                pool_expand<T>(d.variant, gx.col, rb, re, vis, app, sm.td, sink, nullptr);
            } else {
                VisitSTCON vis{d.status, st_code(d.side, d.level + 1), d.side, &slot->tc.found};
                pool_expand<T>(d.variant, gx.col, rb, re, vis, app, sm.td, sink, &slot->tc.found);
            }
        }
        return;
    }
    // bottom-up over vertices [tile * TILE_V, ...) of the reverse graph
    const DGraph &gr = d.side ? gp.fwd : gp.rev;
    const int nv = gr.nv;
    const int v0 = tile * POOL_TILE_V, v1 = min(nv, v0 + POOL_TILE_V);
    int inspected = 0;
    for (int base = v0; base < v1; base += T) {
        int v = base + tid;
        int c[1] = {-1};
        if (v < v1) {
            if (d.mode == MODE_BFS) {
                BottomUpBFS bu{d.levels, d.level};
                c[0] = bu.check(v, gr.row_ptr, gr.col, inspected);
            } else {
                BottomUpSTCON bu{d.status, st_code(d.side, d.level), st_code(d.side, d.level + 1),
                                 st_code(1 - d.side, d.other_radius), &slot->tc.found};
                c[0] = bu.check(v, gr.row_ptr, gr.col, inspected);
            }
        }
        warp_append<1>(c, app);
    }
    int w = warp_sum_i(inspected);
    if (lane_id() == 0 && w) atomicAdd(&slot->tc.inspected, (unsigned long long)w);
}

__device__ __forceinline__ void copy_desc(PoolDesc &dst, const PoolDesc *src)
{
    const int *s = reinterpret_cast<const int *>(src);
    int *d = reinterpret_cast<int *>(&dst);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(PoolDesc) / sizeof(int)); ++i) d[i] = __ldcg(s + i);
}

// Claim and run one tile of some other open step.  Returns true only when a
// tile was run (callers treat that as progress).  All threads call.
template <int T>
__device__ bool pool_steal(const PoolArgs &a, SmemPool<T> &sm)
{
    const int P = gridDim.x, tid = threadIdx.x;
    if (tid == 0) sm.cand = INT_MAX;
    __syncthreads();
    const int cur = sm.cursor;
    // the open hints are one coalesced read; only open slots' tile words
    // (one 256-byte record each) are read
    for (int k = tid; k < P; k += T) {
        int j = (cur + k) % P;
        if (!ld_cg(a.open + j)) continue;
        unsigned long long v = __ldcg(&a.slots[j].next);
        if (pk_tile(v) < pk_ntiles(v)) atomicMin(&sm.cand, k);
    }
    __syncthreads();
    if (sm.cand == INT_MAX) return false;
    const int j = (cur + sm.cand) % P;
    PoolSlot *slot = a.slots + j;
    if (tid == 0) {
        sm.claimed = -1;
        for (int attempt = 0; attempt < 16; ++attempt) {
            unsigned long long v = ld_acquire_u64(&slot->next);
            if (pk_tile(v) >= pk_ntiles(v)) break;
            if (atomicCAS(&slot->next, v, v + 1) == v) {
                sm.claimed = pk_tile(v);
                sm.seq = pk_seq(v);
                copy_desc(sm.d, &slot->d);
                break;
            }
        }
        sm.cursor = j;  // stay with this slot while it has work
    }
    __syncthreads();
    const int t = sm.claimed;
    if (t < 0) return false;  // lost every CAS: no progress made
    pool_tile<T>(a, slot, t, sm.seq, sm);
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        atomicAdd(&slot->done, 1);
    }
    return true;
}

// Once the two sides have met, the step's unclaimed tiles need not run: move
// the tile counter to ntiles and count them done, so the owner waits only for
// tiles already in flight.  A row job pushed later by such a tile raises
// ntiles again and is cancelled on the owner's next look.  Bounded retries.
__device__ __forceinline__ void cancel_unclaimed(PoolSlot *my)
{
    unsigned long long v = ld_acquire_u64(&my->next);
    for (int it = 0; it < 64 && pk_tile(v) < pk_ntiles(v); ++it) {
        const unsigned long long n = (unsigned long long)pk_ntiles(v);
        const unsigned long long old = atomicCAS(&my->next, v, (v & ~PK_MASK) | n);
        if (old == v) {
            atomicAdd(&my->done, (int)(n - (unsigned long long)pk_tile(v)));
            return;
        }
        v = old;
    }
}

// Publish a step of my slot, run its tiles, help others until it completes.
template <int T>
__device__ void pool_publish_and_run(const PoolArgs &a, PoolSlot *my, const PoolDesc &desc,
                                     int nvt, SmemPool<T> &sm)
{
    const int tid = threadIdx.x;
    if (tid == 0) {
        my->d = desc;
        my->done = 0;
        my->njobs = 0;
        sm.my_seq = (sm.my_seq + 1) & 0xFFFFFu;
        if (sm.my_seq == 0) sm.my_seq = 1;
        __threadfence();
        atomicExch(&my->next, pk(sm.my_seq, (unsigned long long)nvt, 0));
        __threadfence();
        *(volatile int *)(a.open + blockIdx.x) = 1;
        sm.d = desc;
    }
    __syncthreads();
    // own tiles (claimed by CAS like everyone else: the tile counter never
    // runs past ntiles, so indices that row jobs add later stay claimable)
    while (true) {
        if (tid == 0) {
            sm.claimed = -1;
            if (desc.mode == MODE_STCON && desc.dir != DIR_RESET && ld_cg(&my->tc.found))
                cancel_unclaimed(my);
            unsigned long long v = ld_acquire_u64(&my->next);
            while (pk_tile(v) < pk_ntiles(v)) {
                unsigned long long w = atomicCAS(&my->next, v, v + 1);
                if (w == v) {
                    sm.claimed = pk_tile(v);
                    break;
                }
                v = w;
            }
        }
        __syncthreads();
        const int t = sm.claimed;
        if (t < 0) break;
        pool_tile<T>(a, my, t, sm.my_seq, sm);
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            atomicAdd(&my->done, 1);
            sm.d = desc;  // a helper run may not have replaced it, but keep it exact
        }
        __syncthreads();
    }
    // wait for helpers (helping others meanwhile when OWNER_HELPS); the
    // launch's error word, set only when some wait timed out, is read every
    // 16th poll: every waiting CTA reading it each time crowds its L2 line
    if (tid == 0) sm.t_idle = global_timer_ns();
    unsigned polls = 0;
    while (true) {
        if (tid == 0) {
            if (desc.mode == MODE_STCON && desc.dir != DIR_RESET && ld_cg(&my->tc.found))
                cancel_unclaimed(my);
            int dn = ld_acquire_gpu(&my->done);
            unsigned long long v = ld_acquire_u64(&my->next);
            sm.flag = dn >= pk_ntiles(v) ? 1 : 0;
            if (!sm.flag && global_timer_ns() - sm.t_idle > POOL_IDLE_NS) {
                atomicCAS(&a.ctr[CTR_ERR], 0, FC_ERR_TIMEOUT);
                sm.flag = 2;
            }
            if (!sm.flag && (++polls & 15u) == 0 && ld_cg(&a.ctr[CTR_ERR])) sm.flag = 2;
        }
        __syncthreads();
        if (sm.flag) break;
        if (OWNER_HELPS && pool_steal<T>(a, sm)) {
            if (tid == 0) sm.t_idle = global_timer_ns();
        } else if (tid == 0) {
            __nanosleep(128);
        }
        __syncthreads();
    }
    if (tid == 0) {
        *(volatile int *)(a.open + blockIdx.x) = 0;  // every tile is done
        sm.err = sm.flag == 2;
        sm.d = desc;
    }
    __syncthreads();
}

// A step the owner runs alone.
template <int T>
__device__ __forceinline__ void pool_private_step(int mode, const GraphPair &gp, int x, int level,
                                               int other_radius, const int32_t *front, int F,
                                               uint8_t *status, int32_t *levels, int32_t *log,
                                               int cap, SmemPool<T> &sm, int variant, bool track)
{
    run_step<T>(mode, gp, x, DIR_TD, level, other_radius, front, F, 0, 1, status, levels, log, cap,
                &sm.stc.tail[x], &sm.stc.deg[x], &sm.stc.found, &sm.stc.inspected, sm.td, variant,
                track ? &sm.stc.hist[x] : nullptr);
}

// Run query q with my slot as owner.
template <int T>
__device__ void pool_query(const PoolArgs &a, PoolSlot *my, int q, uint8_t *status, int32_t *log,
                           SmemPool<T> &sm)
{
    const int tid = threadIdx.x;
    const int gidx = a.graph_idx ? a.graph_idx[q] : 0;
    const GraphPair gp = a.graphs[gidx];
    const int nv = gp.fwd.nv;
    int s = a.qs[q];
    int t = a.mode == MODE_STCON ? a.qt[q] : s;
    const int cap = a.exclusive ? nv : min(nv, a.log_cap);
    if (s < 0 || s >= nv || t < 0 || t >= nv) {
        if (tid == 0) {
            if (a.out_conn) a.out_conn[q] = 0;
            if (a.out_hops) a.out_hops[q] = -2;
            atomicExch(&a.ctr[CTR_INVALID], 1);
            __threadfence();
            atomicAdd(&a.ctr[CTR_FINISHED], 1);
        }
        __syncthreads();
        return;
    }
    if (gp.fwd.remap) {  // a renumbered copy of the graph: the caller's ids map into it
        s = __ldg(gp.fwd.remap + s);
        t = __ldg(gp.fwd.remap + t);
    }
    int32_t *levels = a.levels;
    // the degree histogram is counted only for the learned schedule and traces
    const bool track = (a.sched == FC_SCHED_LEARNED && a.mlp) || a.trace;
    // the step description lives in shared memory and only thread 0 reads or
    // writes it (it is copied to the slot when a step is published)
    PoolDesc &desc = sm.own;
    // thread 0's copy of the query counter, read a step ahead so that the
    // test for the batch's tail waits on no load of its own
    int next_seen = 0;
    if (tid == 0) {
        if (!a.exclusive) next_seen = ld_cg(&a.ctr[CTR_NEXT]);
        // the roots and the counters start in this CTA: the counters in
        // shared memory (the slot's copy is written when a step is
        // published), the roots' status and log entries read by this CTA
        // after the barrier below, or by helpers after the publishing fence
        init_roots(a.mode, gp, s, t, status, levels, log, cap, &sm.stc);
        ql_start(sm.ql, a.mode == MODE_STCON, nv, gp.fwd.ne, s, t, sm.stc.deg[0], sm.stc.deg[1]);
        sm.err = 0;
        desc.q = q;
        desc.gidx = gidx;
        desc.mode = a.mode;
        desc.cap = cap;
        desc.status = status;
        desc.levels = levels;
        desc.log = log;
        desc.nreset = 0;
        desc.split_e = a.split_e;
        desc.track_hist = track;
    }
    __syncthreads();
    const int bu_cap = a.mode == MODE_BFS ? INT_MAX : LEVEL7_MAX;
    while (true) {
        if (tid < 32 && !sm.ql.done) {
            // warp 0 decides: policy, then the MLP (warp-level), then a script
            if (tid == 0) ql_decide(sm.ql, a.sched, 1, bu_cap, 1, a.force_variant);
            __syncwarp();
            const bool consult = a.sched == FC_SCHED_LEARNED && a.mlp && mlp_worth(sm.ql);
            if (a.trace || consult) {
                float f[MLP_IN];
                ql_features(sm.ql, f);
                if (consult && mlp_in_box(sm.mlp, f)) {
                    float o[MLP_OUT];
                    mlp_forward_warp(sm.mlp, f, o);
                    if (tid == 0) {
                        ql_apply_logits(sm.ql, o, 1, bu_cap);
                        if (a.force_variant >= 0) sm.ql.variant = a.force_variant;
                    }
                }
                if (tid == 0)
                    for (int i = 0; i < MLP_IN; ++i) sm.ql.feat[i] = f[i];
            }
            if (tid == 0) {
                if (a.script && sm.ql.steps < a.script_len) {
                    const unsigned char act = a.script[(size_t)q * a.script_len + sm.ql.steps];
                    if (act != 0xFF) ql_apply_script(sm.ql, act, 1, bu_cap);
                }
                const int x = sm.ql.side;
                const long long m = (long long)(sm.ql.dt[x] - sm.ql.dh[x]);
                // new claims are bounded by the entries read and by the
                // vertices not yet claimed
                const long long used = (long long)sm.ql.tail[0] + sm.ql.tail[1];
                const long long grow = m < (long long)nv - used ? m : (long long)nv - used;
                if (!a.exclusive && used + grow > cap) {
                    sm.ql.escalate = 1;  // the log could overflow: finish it in exclusive mode
                    sm.ql.done = 1;
                }
                // in the batch's tail (every query taken, idle CTAs about)
                // smaller steps are shared, in smaller tiles
                sm.tail = !a.exclusive && next_seen >= sm.nq;
                const long long priv = sm.tail ? a.private_edges / 8 : a.private_edges;
                sm.publish = sm.ql.dir == DIR_BU || m > priv;
                if (!sm.publish && a.private_variant >= 0 && a.force_variant < 0)
                    sm.ql.variant = a.private_variant;
                sm.t_step = global_timer_ns();
            }
        }
        __syncthreads();
        if (sm.ql.done) break;
        const int x = sm.ql.side;
        int F;
        const int32_t *front = ql_frontier(sm.ql, log, cap, x, &F);
        if (!sm.publish) {
            pool_private_step<T>(a.mode, gp, x, sm.ql.radius[x], sm.ql.radius[1 - x], front, F,
                                 status, levels, log, cap, sm, sm.ql.variant, track);
            __syncthreads();
        } else {
            // top-down tiles by work: frontiers of high average degree get
            // tiles of fewer vertices (down to one) so that a tile reads
            // about tile_e entries; low-degree frontiers get tiles of T
            // vertices, or of several chunks of T when there would be more
            // than about 8 tiles per CTA (fewer claims on the slot word)
            const long long m = (long long)(sm.ql.dt[x] - sm.ql.dh[x]);
            int tv = T;
            const int tile_e = sm.tail ? max(a.tile_e / 4, 2 * T) : a.tile_e;
            if (m > (long long)F * (tile_e / T)) {
                const long long want_v = (long long)tile_e * F / (m > 0 ? m : 1);
                tv = 1;
                while (tv * 2 <= want_v) tv *= 2;
            } else {
                const int chunks = (F + T - 1) / T;
                const int want = 8 * (int)gridDim.x;
                if (chunks > want) tv = T * ((chunks + want - 1) / want);
            }
            const int nvt = sm.ql.dir == DIR_TD ? (int)(((long long)F + tv - 1) / tv)
                                                : (nv + POOL_TILE_V - 1) / POOL_TILE_V;
            if (tid == 0) {
                desc.side = x;
                desc.dir = sm.ql.dir;
                desc.variant = sm.ql.variant;
                desc.level = sm.ql.radius[x];
                desc.other_radius = sm.ql.radius[1 - x];
                desc.F = F;
                desc.front_off = (int)(front - log);
                desc.tile_v = tv;
                desc.nvt = nvt;
                counters_to_slot(my, sm.stc);  // published by the fence in the call
            }
            pool_publish_and_run<T>(a, my, desc, nvt, sm);
            if (sm.err) return;
            if (tid == 0) counters_from_slot(sm.stc, my);
        }
        if (tid == 0) {
            if (!a.exclusive && next_seen < sm.nq) next_seen = ld_cg(&a.ctr[CTR_NEXT]);
            const unsigned long long ins0 = sm.ql.inspected;
            const int tail0 = sm.ql.tail[x], F0 = sm.ql.tail[x] - sm.ql.head[x];
            const int dir0 = sm.ql.dir, var0 = sm.ql.variant, step0 = sm.ql.steps;
            ql_update(sm.ql, sm.stc.found, sm.stc.tail[x], sm.stc.deg[x], sm.stc.inspected);
            if (track) {
                ql_update_hist(sm.ql, x, sm.stc.hist[x]);
            }
            if (a.trace) {
                const int k = atomicAdd(a.trace_count, 1);
                if (k < a.trace_cap) {
                    int32_t *r = a.trace + (size_t)k * TRACE_WORDS;
                    const unsigned long long cost = sm.ql.inspected - ins0;
                    const unsigned long long dt = global_timer_ns() - sm.t_step;
                    r[0] = q;
                    r[1] = step0;
                    r[2] = x;
                    r[3] = dir0;
                    r[4] = var0;
                    // bit 0: the sides met; bit 1: the step was shared as tiles
                    r[5] = (sm.ql.connected && sm.ql.done ? 1 : 0) | (sm.publish ? 2 : 0);
                    r[6] = (int32_t)(cost & 0xFFFFFFFFull);
                    r[7] = (int32_t)(cost >> 32);
                    r[8] = (int32_t)(dt & 0xFFFFFFFFull);
                    r[9] = (int32_t)(dt >> 32);
                    r[10] = sm.ql.tail[x] - tail0;
                    r[11] = F0;
                    for (int i = 0; i < MLP_IN; ++i) r[12 + i] = __float_as_int(sm.ql.feat[i]);
                }
            }
        }
        __syncthreads();
    }
    if (tid == 0) {
        if (sm.ql.escalate) {
            int k = atomicAdd(&a.ctr[CTR_SPILL], 1);
            a.spill[k] = q;
        }
        write_result(q, sm.ql, a.out_conn, a.out_hops, a.qstat, sm.ql.escalate);
        if (a.out_inspected && !sm.ql.escalate) a.out_inspected[q] = (long long)sm.ql.inspected;
    }
    // clear exactly the claimed status bytes (s-t mode), sharing big resets
    if (a.mode == MODE_STCON) {
        const int n0 = sm.ql.tail[0], n1 = sm.ql.tail[1];
        if (n0 + n1 <= 4 * POOL_TILE_R) {
            clear_claimed(status, log, cap, n0, 0, (long long)n0 + n1, tid, T);
        } else {
            const int nvt = (n0 + n1 + POOL_TILE_R - 1) / POOL_TILE_R;
            if (tid == 0) {
                desc.F = n0;
                desc.dir = DIR_RESET;
                desc.nreset = n0 + n1;
                desc.nvt = nvt;
            }
            pool_publish_and_run<T>(a, my, desc, nvt, sm);
            if (sm.err) return;
        }
    }
    // the finished count only tells idle CTAs when to leave: the answers
    // are read after the kernel ends, so no fence is needed before it
    __syncthreads();
    if (tid == 0) atomicAdd(&a.ctr[CTR_FINISHED], 1);
    __syncthreads();
}

template <int T>
__global__ void __launch_bounds__(T, 768 / T) k_pool(PoolArgs a)
{
    __shared__ SmemPool<T> sm;
    const int tid = threadIdx.x;
    PoolSlot *my = a.slots + blockIdx.x;
    const int nq = a.list_count ? ld_cg(a.list_count) : a.nlist;
    if (tid == 0) {
        sm.nq = nq;
        sm.tail = 0;
        sm.cursor = (int)((blockIdx.x * 97u) % gridDim.x);
        sm.li = 0;
        sm.err = 0;
        // continue this slot's seq numbering across launches
        sm.my_seq = pk_seq(__ldcg(&my->next));
    }
    if (a.sched == FC_SCHED_LEARNED && a.mlp)
        for (int i = tid; i < MLP_STORE; i += T) sm.mlp[i] = __ldg(a.mlp + i);
    __syncthreads();
    if (!a.exclusive || blockIdx.x == 0) {
        uint8_t *status = a.status_base + (a.exclusive ? 0 : (size_t)blockIdx.x * a.status_stride);
        int32_t *log = a.log_base + (a.exclusive ? 0 : (size_t)blockIdx.x * a.log_stride);
        while (true) {
            if (tid == 0) {
                sm.q = a.exclusive ? sm.li++ : atomicAdd(&a.ctr[CTR_NEXT], 1);
                if (ld_cg(&a.ctr[CTR_ERR])) sm.q = INT_MAX;
            }
            __syncthreads();
            const int qi = sm.q;
            if (qi >= nq) break;
            pool_query<T>(a, my, a.list ? a.list[qi] : qi, status, log, sm);
            if (sm.err) break;
        }
    }
    // help until every query is finished; an idle CTA polls the slots with a
    // growing pause (128 ns to 4 us) so that the pollers of the batch's tail
    // do not crowd the L2 lines the working CTAs claim tiles from
    if (tid == 0) {
        sm.t_idle = global_timer_ns();
        sm.backoff = 128;
    }
    __syncthreads();
    unsigned polls = 0;
    while (true) {
        if (tid == 0) {
            sm.flag = ld_acquire_gpu(&a.ctr[CTR_FINISHED]) >= nq ||
                      ((++polls & 15u) == 0 && ld_cg(&a.ctr[CTR_ERR]) != 0);
            if (!sm.flag && global_timer_ns() - sm.t_idle > POOL_IDLE_NS) {
                atomicCAS(&a.ctr[CTR_ERR], 0, FC_ERR_TIMEOUT);
                sm.flag = 1;
            }
        }
        __syncthreads();
        if (sm.flag) break;
        if (pool_steal<T>(a, sm)) {
            if (tid == 0) {
                sm.t_idle = global_timer_ns();
                sm.backoff = 128;
            }
        } else if (tid == 0) {
            __nanosleep(sm.backoff);
            if (sm.backoff < 4096) sm.backoff *= 2;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
size_t pool_slot_bytes() { return sizeof(PoolSlot); }
size_t pool_job_bytes() { return sizeof(RowJob) * POOL_JOBS; }

// The pool kernel comes in CTAs of 128 and 256 threads; a batch picks one
// (fc_opts.block), the single-query form uses 256.
static const void *pool_kernel(int block)
{
    return block == 128 ? (const void *)k_pool<128> : (const void *)k_pool<256>;
}

int pool_block(int requested) { return requested == 128 ? 128 : 256; }

int pool_grid(int sm_count, int ctas_per_sm, int block)
{
    block = pool_block(block);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pool_kernel(block), block, 0) !=
            cudaSuccess ||
        per_sm < 1)
        return 0;
    if (ctas_per_sm > 0 && ctas_per_sm < per_sm) per_sm = ctas_per_sm;
    return per_sm * sm_count;
}

int pool_max_grid(int sm_count)
{
    const int a = pool_grid(sm_count, 0, 128), b = pool_grid(sm_count, 0, 256);
    return a > b ? a : b;
}

int pool_launch(const PoolArgs &a, int grid, int block, cudaStream_t st)
{
    block = pool_block(block);
    PoolArgs args = a;
    void *kargs[] = {&args};
    FC_CUDA_TRY(cudaLaunchCooperativeKernel(pool_kernel(block), dim3(grid), dim3(block), kargs, 0,
                                            st));
    return FC_OK;
}

}  // namespace fc
