// fc_engine.cu -- traversal engines for BFS levels and s-t connectivity.
//
// Three engines share the step code of fc_step.cuh:
//
//   host-loop   one ordinary launch per expansion step; the host reads the
//               step's counters back and picks the next step.  This is the
//               plain level-synchronous form (reference shape: the per-level
//               host loop of make_stcon, S/make_stcon.c:968-1187, and of
//               cudaBFS4K, K/src/device/BFS_WorkEfficient.cu:94-116).
//   persistent  one cooperative launch; all CTAs run the level loop and meet
//               at a bounded software grid barrier after every step (reference
//               shape: BFSDispath + GlobalSync, K/.../BFS_WE_KernelDispatch.cu:
//               17-38, whose barrier spins without bound).
//   batched     one launch for many queries; each CTA pulls queries from a
//               global counter and runs them privately with __syncthreads
//               between steps (reference shape: one CTA per source in
//               BFS_4K_BLOCK, BFS_4K_BLOCK/.../BFS_WE_Block.cu:33-147).  A query
//               whose next step would exceed the CTA's work limit or log space
//               is handed to a spill list that the persistent engine finishes
//               in the same stream.
//
// s-t connectivity grows a ball from s (side 0) and from t (side 1), one side
// per step.  With both balls complete and disjoint, the first edge from the
// expanding side's frontier (radius r_x) into the other ball (radius r_y)
// proves d(s,t) = r_x + 1 + r_y: a shorter path would put a vertex in both
// balls, and any ball vertex adjacent to the frontier must sit on the other
// ball's outer level.  So the meeting step may stop early and the distance is
// still exact (the reference returns only ceil(d/2), S/make_stcon.c:1496).
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

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

// Choose the next step.  allow_bu = 0 in the batched engine (a bottom-up step
// scans every vertex, which one CTA must not do).  bu_level_cap limits
// bottom-up to levels whose status code is exact (s-t status bytes hold
// min(level, 127)).
__host__ __device__ inline void ql_decide(QLocal &q, int sched, int allow_bu, int bu_level_cap)
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
    q.variant = 0;
    if (sched != FC_SCHED_PLAIN && allow_bu && q.radius[side] + 1 <= bu_level_cap) {
        long long mf = (long long)(q.dt[side] - q.dh[side]);
        long long unexplored = q.ne - (long long)(q.dt[0] + q.dt[1]);
        long long nf = q.tail[side] - q.head[side];
        // Beamer, Asanovic & Patterson (SC'12) thresholds: alpha = 14, beta = 24
        if (mf * 14 > unexplored && nf * 24 > q.nv) q.dir = DIR_BU;
    }
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
template <int T>
__device__ void run_step(int mode, const GraphPair &gp, int side, int dir, int level,
                         int other_radius, const int32_t *frontier, int F, int team_rank,
                         int team_size, uint8_t *status, int32_t *levels, int32_t *log, int cap,
                         int *tail_ctr, unsigned long long *deg_ctr, int *found,
                         unsigned long long *bu_ins, SmemTopDown<T> &sm)
{
    const DGraph &gx = side ? gp.rev : gp.fwd;
    AppendTarget app{log, cap, side, tail_ctr, deg_ctr, gx.row_ptr};
    if (dir == DIR_TD) {
        if (mode == MODE_BFS) {
            VisitBFS vis{levels, level + 1};
            topdown_step<T>(gx.row_ptr, gx.col, frontier, F, team_rank, team_size, vis, app, sm,
                            nullptr);
        } else {
            VisitSTCON vis{status, st_code(side, level + 1), side, found};
            topdown_step<T>(gx.row_ptr, gx.col, frontier, F, team_rank, team_size, vis, app, sm,
                            found);
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
__device__ void init_roots(int mode, const GraphPair &gp, int s, int t, uint8_t *status,
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

// ---------------------------------------------------------------------------
// host-loop engine kernels
// ---------------------------------------------------------------------------
__global__ void k_init_roots(int mode, GraphPair gp, int s, int t, uint8_t *status,
                             int32_t *levels, int32_t *log, int cap, TeamCounters *tc)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) init_roots(mode, gp, s, t, status, levels, log, cap, tc);
}

struct StepArgs {
    GraphPair gp;
    int mode, side, dir, level, other_radius;
    int front_begin, F;
    uint8_t *status;
    int32_t *levels;
    int32_t *log;
    int cap;
    TeamCounters *tc;
};

template <int T>
__global__ void __launch_bounds__(T) k_step(StepArgs a)
{
    __shared__ SmemTopDown<T> sm;
    run_step<T>(a.mode, a.gp, a.side, a.dir, a.level, a.other_radius, a.log + a.front_begin, a.F,
                blockIdx.x, gridDim.x, a.status, a.levels, a.log, a.cap, &a.tc->tail[a.side],
                &a.tc->deg[a.side], &a.tc->found, &a.tc->inspected, sm);
}

// ---------------------------------------------------------------------------
// persistent engine: cooperative launch, queries run one after another, the
// whole grid on each; list/list_count select a subset (the spill list).
// ---------------------------------------------------------------------------
struct PersistArgs {
    const GraphPair *graphs;
    const int32_t *graph_idx;
    const int32_t *qs;
    const int32_t *qt;
    const int32_t *list;
    const int *list_count;
    int nlist;
    int mode, sched;
    uint8_t *status;
    int32_t *levels;
    int32_t *log;
    TeamCounters *tc;
    int32_t *out_conn;
    int32_t *out_hops;
    QueryStat *qstat;
};

template <int T>
__global__ void __launch_bounds__(T) k_persistent(PersistArgs a)
{
    __shared__ SmemTopDown<T> sm;
    __shared__ QLocal ql;
    TeamCounters *tc = a.tc;
    const int nq = a.list_count ? *(volatile const int *)a.list_count : a.nlist;
    for (int li = 0; li < nq; ++li) {
        const int q = a.list ? a.list[li] : li;
        const GraphPair gp = a.graphs[a.graph_idx ? a.graph_idx[q] : 0];
        const int nv = gp.fwd.nv;
        const int s = a.qs[q];
        const int t = a.mode == MODE_STCON ? a.qt[q] : s;
        const bool bad = s < 0 || s >= nv || t < 0 || t >= nv;
        if (bad) {  // uniform across the grid: no barrier needed to skip
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                if (a.out_conn) a.out_conn[q] = 0;
                if (a.out_hops) a.out_hops[q] = -2;
                atomicExch(&tc->invalid, 1);
            }
            continue;
        }
        if (blockIdx.x == 0 && threadIdx.x == 0)
            init_roots(a.mode, gp, s, t, a.status, a.levels, a.log, nv, tc);
        if (!grid_barrier(tc->bar, &tc->err, gridDim.x)) return;
        if (threadIdx.x == 0)
            ql_start(ql, a.mode == MODE_STCON, nv, gp.fwd.ne, s, t, ld_cg_u64(&tc->deg[0]),
                     ld_cg_u64(&tc->deg[1]));
        __syncthreads();
        while (true) {
            if (threadIdx.x == 0 && !ql.done)
                ql_decide(ql, a.sched, 1, a.mode == MODE_BFS ? 0x7fffffff : LEVEL7_MAX);
            __syncthreads();
            if (ql.done) break;
            int F;
            const int x = ql.side;
            const int32_t *front = ql_frontier(ql, a.log, nv, x, &F);
            run_step<T>(a.mode, gp, x, ql.dir, ql.radius[x], ql.radius[1 - x], front, F,
                        blockIdx.x, gridDim.x, a.status, a.levels, a.log, nv, &tc->tail[x],
                        &tc->deg[x], &tc->found, &tc->inspected, sm);
            if (!grid_barrier(tc->bar, &tc->err, gridDim.x)) return;
            if (threadIdx.x == 0)
                ql_update(ql, ld_cg(&tc->found), ld_cg(&tc->tail[x]), ld_cg_u64(&tc->deg[x]),
                          ld_cg_u64(&tc->inspected));
            __syncthreads();
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) write_result(q, ql, a.out_conn, a.out_hops, a.qstat, 0);
        if (a.mode == MODE_STCON) {
            // clear exactly the claimed vertices (the log holds each once)
            const int n0 = ql.tail[0], n1 = ql.tail[1];
            for (long long i = (long long)blockIdx.x * T + threadIdx.x; i < n0 + n1;
                 i += (long long)gridDim.x * T) {
                int v = i < n0 ? a.log[i] : a.log[nv - 1 - (i - n0)];
                a.status[v] = ST_UNVISITED;
            }
        }
        if (!grid_barrier(tc->bar, &tc->err, gridDim.x)) return;
    }
}

// ---------------------------------------------------------------------------
// batched engine: one CTA per query at a time, private slot per CTA.
// ---------------------------------------------------------------------------
struct BatchArgs {
    const GraphPair *graphs;
    const int32_t *graph_idx;
    const int32_t *qs;
    const int32_t *qt;
    int nq;
    int *ctr;  // [0] next query, [1] spill count, [2] invalid flag
    int32_t *spill;
    uint8_t *status_arena;
    size_t status_stride;
    int32_t *log_arena;
    size_t log_stride;
    int log_cap;
    long long work_limit;
    int sched;
    int32_t *out_conn;
    int32_t *out_hops;
    QueryStat *qstat;
};

template <int T>
__global__ void __launch_bounds__(T) k_batched(BatchArgs a)
{
    __shared__ SmemTopDown<T> sm;
    __shared__ QLocal ql;
    __shared__ TeamCounters tc;
    __shared__ int s_q;
    uint8_t *status = a.status_arena + (size_t)blockIdx.x * a.status_stride;
    int32_t *log = a.log_arena + (size_t)blockIdx.x * a.log_stride;
    const int cap = a.log_cap;
    while (true) {
        if (threadIdx.x == 0) s_q = atomicAdd(&a.ctr[0], 1);
        __syncthreads();
        const int q = s_q;
        if (q >= a.nq) break;
        const GraphPair gp = a.graphs[a.graph_idx ? a.graph_idx[q] : 0];
        const int nv = gp.fwd.nv;
        const int s = a.qs[q], t = a.qt[q];
        if (s < 0 || s >= nv || t < 0 || t >= nv) {
            if (threadIdx.x == 0) {
                if (a.out_conn) a.out_conn[q] = 0;
                if (a.out_hops) a.out_hops[q] = -2;
                a.ctr[2] = 1;
            }
            __syncthreads();
            continue;
        }
        if (threadIdx.x == 0) {
            init_roots(MODE_STCON, gp, s, t, status, nullptr, log, cap, &tc);
            ql_start(ql, 1, nv, gp.fwd.ne, s, t, tc.deg[0], tc.deg[1]);
        }
        __syncthreads();
        while (true) {
            if (threadIdx.x == 0 && !ql.done) {
                ql_decide(ql, a.sched, 0, LEVEL7_MAX);
                const int x = ql.side;
                long long mf = (long long)(ql.dt[x] - ql.dh[x]);
                if (mf > a.work_limit || (long long)ql.tail[0] + ql.tail[1] + mf > cap) {
                    ql.escalate = 1;
                    ql.done = 1;
                }
            }
            __syncthreads();
            if (ql.done) break;
            int F;
            const int x = ql.side;
            const int32_t *front = ql_frontier(ql, log, cap, x, &F);
            run_step<T>(MODE_STCON, gp, x, DIR_TD, ql.radius[x], ql.radius[1 - x], front, F, 0, 1,
                        status, nullptr, log, cap, &tc.tail[x], &tc.deg[x], &tc.found,
                        &tc.inspected, sm);
            __syncthreads();
            if (threadIdx.x == 0) ql_update(ql, tc.found, tc.tail[x], tc.deg[x], tc.inspected);
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            if (ql.escalate) {
                int k = atomicAdd(&a.ctr[1], 1);
                a.spill[k] = q;
            }
            write_result(q, ql, a.out_conn, a.out_hops, a.qstat, ql.escalate);
        }
        const int n0 = ql.tail[0], n1 = ql.tail[1];
        for (int i = threadIdx.x; i < n0 + n1; i += T) {
            int v = i < n0 ? log[i] : log[cap - 1 - (i - n0)];
            status[v] = ST_UNVISITED;
        }
        __syncthreads();
    }
}

// ===========================================================================
// host side
// ===========================================================================
static thread_local char g_errmsg[512];

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_errmsg, sizeof(g_errmsg), fmt, ap);
    va_end(ap);
}

}  // namespace fc

extern "C" void fc_set_last_cuda_error(cudaError_t e, const char *what, const char *file, int line)
{
    fc::set_error("%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
}

extern "C" const char *fc_last_error_message(void) { return fc::g_errmsg; }

namespace fc {

static DevCtx g_ctx[16];
static std::mutex g_ctx_mu;

DevCtx *get_ctx(int *err)
{
    int dev = 0, n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        *err = FC_ERR_NO_DEVICE;
        set_error("no CUDA device: %s", cudaGetErrorString(e));
        return nullptr;
    }
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 16) {
        *err = FC_ERR_UNSUPPORTED;
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    DevCtx *c = &g_ctx[dev];
    if (c->device < 0) {
        cudaDeviceProp p;
        if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) {
            *err = FC_ERR_CUDA;
            return nullptr;
        }
        c->sm_count = p.multiProcessorCount;
        int coop = 0;
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
        c->coop = coop;
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
            cudaEventCreate(&c->evm) != cudaSuccess ||
            cudaMalloc(&c->tc, sizeof(TeamCounters)) != cudaSuccess ||
            cudaMallocHost(&c->h_tc, sizeof(TeamCounters)) != cudaSuccess ||
            cudaMalloc(&c->b_ctr, 4 * sizeof(int)) != cudaSuccess) {
            *err = FC_ERR_CUDA;
            set_error("device context set-up failed");
            return nullptr;
        }
        cudaMemset(c->tc, 0, sizeof(TeamCounters));
        c->device = dev;
    }
    *err = FC_OK;
    return c;
}

static int ensure_ws(DevCtx *c, size_t nv)
{
    if (c->ws_nv >= nv && c->status) return FC_OK;
    cudaFree(c->status);
    cudaFree(c->levels);
    cudaFree(c->log);
    c->status = nullptr;
    c->levels = nullptr;
    c->log = nullptr;
    c->ws_nv = 0;
    size_t sbytes = (nv + 15) / 16 * 16;
    FC_CUDA_TRY(cudaMalloc(&c->status, sbytes));
    FC_CUDA_TRY(cudaMalloc(&c->levels, nv * sizeof(int32_t)));
    FC_CUDA_TRY(cudaMalloc(&c->log, nv * sizeof(int32_t)));
    FC_CUDA_TRY(cudaMemset(c->status, 0xFF, sbytes));
    c->ws_nv = nv;
    return FC_OK;
}

static int ensure_graphs(DevCtx *c, const GraphPairH *gps, int n, cudaStream_t st)
{
    if ((size_t)n > c->graphs_cap) {
        cudaFree(c->d_graphs);
        c->d_graphs = nullptr;
        c->graphs_cap = 0;
        FC_CUDA_TRY(cudaMalloc(&c->d_graphs, sizeof(GraphPair) * (size_t)n));
        c->graphs_cap = (size_t)n;
    }
    FC_CUDA_TRY(cudaMemcpyAsync(c->d_graphs, gps, sizeof(GraphPair) * (size_t)n,
                                cudaMemcpyHostToDevice, st));
    return FC_OK;
}

static inline GraphPair to_dev(const GraphPairH &h)
{
    GraphPair g;
    std::memcpy(&g, &h, sizeof(g));
    return g;
}

template <int T>
static int coop_grid(DevCtx *c)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_persistent<T>, T, 0) != cudaSuccess ||
        per_sm < 1)
        return 0;
    return per_sm * c->sm_count;
}

template <int T>
static int launch_persistent(DevCtx *c, const PersistArgs &a, cudaStream_t st)
{
    int grid = coop_grid<T>(c);
    if (grid <= 0 || !c->coop) {
        set_error("cooperative launch unavailable");
        return FC_ERR_UNSUPPORTED;
    }
    PersistArgs args = a;
    void *kargs[] = {&args};
    FC_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)k_persistent<T>, dim3(grid), dim3(T),
                                            kargs, 0, st));
    return FC_OK;
}

static int check_counters(DevCtx *c, cudaStream_t st)
{
    FC_CUDA_TRY(cudaMemcpyAsync(c->h_tc, c->tc, sizeof(TeamCounters), cudaMemcpyDeviceToHost, st));
    FC_CUDA_TRY(cudaStreamSynchronize(st));
    if (c->h_tc->err) {
        set_error("device-side wait timed out (bounded grid barrier)");
        // leave the workspace clean for the next call
        cudaMemset(c->tc, 0, sizeof(TeamCounters));
        if (c->status) cudaMemset(c->status, 0xFF, (c->ws_nv + 15) / 16 * 16);
        return FC_ERR_TIMEOUT;
    }
    return FC_OK;
}

// Host-loop engine: one launch per step; returns the final QLocal.
static int hostloop(DevCtx *c, int mode, const GraphPairH &gph, int s, int t, int sched,
                    QLocal *out, cudaStream_t st)
{
    constexpr int T = FC_BLOCK;
    const GraphPair gp = to_dev(gph);
    const int nv = gph.fwd.nv;
    k_init_roots<<<1, 32, 0, st>>>(mode, gp, s, t, c->status, c->levels, c->log, nv, c->tc);
    FC_CUDA_TRY(cudaGetLastError());
    FC_CUDA_TRY(cudaMemcpyAsync(c->h_tc, c->tc, sizeof(TeamCounters), cudaMemcpyDeviceToHost, st));
    FC_CUDA_TRY(cudaStreamSynchronize(st));
    QLocal q;
    ql_start(q, mode == MODE_STCON, nv, gph.fwd.ne, s, t, c->h_tc->deg[0], c->h_tc->deg[1]);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step<T>, T, 0);
    if (per_sm < 1) per_sm = 1;
    const int full_grid = per_sm * c->sm_count;
    while (!q.done) {
        ql_decide(q, sched, 1, mode == MODE_BFS ? 0x7fffffff : LEVEL7_MAX);
        const int x = q.side;
        StepArgs a;
        a.gp = gp;
        a.mode = mode;
        a.side = x;
        a.dir = q.dir;
        a.level = q.radius[x];
        a.other_radius = q.radius[1 - x];
        a.F = q.tail[x] - q.head[x];
        a.front_begin = x == 0 ? q.head[0] : nv - q.tail[1];
        a.status = c->status;
        a.levels = c->levels;
        a.log = c->log;
        a.cap = nv;
        a.tc = c->tc;
        int grid = q.dir == DIR_TD ? (a.F + T - 1) / T : full_grid;
        if (grid > full_grid) grid = full_grid;
        if (grid < 1) grid = 1;
        k_step<T><<<grid, T, 0, st>>>(a);
        FC_CUDA_TRY(cudaGetLastError());
        FC_CUDA_TRY(cudaMemcpyAsync(c->h_tc, c->tc, sizeof(TeamCounters), cudaMemcpyDeviceToHost, st));
        FC_CUDA_TRY(cudaStreamSynchronize(st));
        ql_update(q, c->h_tc->found, c->h_tc->tail[x], c->h_tc->deg[x], c->h_tc->inspected);
    }
    *out = q;
    return FC_OK;
}

static void fill_stats(fc_stats *st, const QLocal &q, int launches)
{
    if (!st) return;
    std::memset(st, 0, sizeof(*st));
    st->edges_inspected = (int64_t)q.inspected;
    st->visited = q.tail[0] + q.tail[1];
    st->steps = q.steps;
    st->bottom_up_steps = q.bu_steps;
    st->alg_bytes = (int64_t)q.alg_bytes;
    st->launches = launches;
}

static void from_qstat(QLocal &q, const QueryStat &h)
{
    q.inspected = (unsigned long long)h.inspected;
    q.alg_bytes = (unsigned long long)h.alg_bytes;
    q.steps = h.steps;
    q.bu_steps = h.bu_steps;
    q.tail[0] = h.visited;
    q.tail[1] = 0;
}

static int pick_engine(const fc_opts &o, int dflt)
{
    return o.engine == FC_ENGINE_AUTO ? dflt : o.engine;
}

int engine_bfs(DevCtx *c, const GraphPairH &gp, int32_t s, int32_t *h_levels, const fc_opts &o,
               fc_stats *st, cudaStream_t stream)
{
    const int nv = gp.fwd.nv;
    int rc = ensure_ws(c, (size_t)nv);
    if (rc) return rc;
    FC_CUDA_TRY(cudaMemsetAsync(c->levels, 0xFF, sizeof(int32_t) * (size_t)nv, stream));
    FC_CUDA_TRY(cudaEventRecord(c->ev0, stream));
    const int engine = pick_engine(o, FC_ENGINE_PERSISTENT);
    QLocal q;
    std::memset(&q, 0, sizeof(q));
    if (engine == FC_ENGINE_HOSTLOOP) {
        rc = hostloop(c, MODE_BFS, gp, s, s, o.sched, &q, stream);
        if (rc) return rc;
    } else {
        rc = ensure_graphs(c, &gp, 1, stream);
        if (rc) return rc;
        QueryStat *qs = nullptr;
        if (c->qstat_cap < 1) {
            FC_CUDA_TRY(cudaMalloc(&c->qstat, sizeof(QueryStat) * 1024));
            c->qstat_cap = 1024;
        }
        qs = c->qstat;
        FC_CUDA_TRY(cudaMemsetAsync(qs, 0, sizeof(QueryStat), stream));
        int32_t *d_s = nullptr;
        if (c->tmp_q_cap < 4) {
            cudaFree(c->d_tmp_q);
            c->d_tmp_q = nullptr;
            FC_CUDA_TRY(cudaMalloc(&c->d_tmp_q, sizeof(int32_t) * 4096));
            c->tmp_q_cap = 4096;
        }
        d_s = c->d_tmp_q;
        FC_CUDA_TRY(cudaMemcpyAsync(d_s, &s, sizeof(int32_t), cudaMemcpyHostToDevice, stream));
        PersistArgs a;
        std::memset(&a, 0, sizeof(a));
        a.graphs = (const GraphPair *)c->d_graphs;
        a.qs = d_s;
        a.qt = d_s;
        a.nlist = 1;
        a.mode = MODE_BFS;
        a.sched = o.sched;
        a.status = c->status;
        a.levels = c->levels;
        a.log = c->log;
        a.tc = c->tc;
        a.qstat = qs;
        rc = launch_persistent<FC_BLOCK>(c, a, stream);
        if (rc) return rc;
        rc = check_counters(c, stream);
        if (rc) return rc;
        QueryStat h;
        FC_CUDA_TRY(cudaMemcpy(&h, qs, sizeof(h), cudaMemcpyDeviceToHost));
        from_qstat(q, h);
    }
    FC_CUDA_TRY(cudaEventRecord(c->ev1, stream));
    if (h_levels)
        FC_CUDA_TRY(cudaMemcpyAsync(h_levels, c->levels, sizeof(int32_t) * (size_t)nv,
                                    cudaMemcpyDeviceToHost, stream));
    FC_CUDA_TRY(cudaStreamSynchronize(stream));
    if (st) {
        fill_stats(st, q, engine == FC_ENGINE_HOSTLOOP ? q.steps + 1 : 1);
        float ms = 0;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        st->gpu_ms = ms;
    }
    return FC_OK;
}

int engine_stcon(DevCtx *c, const GraphPairH &gp, int32_t s, int32_t t, int32_t *conn,
                 int32_t *hops, const fc_opts &o, fc_stats *st, cudaStream_t stream)
{
    const int nv = gp.fwd.nv;
    int rc = ensure_ws(c, (size_t)nv);
    if (rc) return rc;
    FC_CUDA_TRY(cudaEventRecord(c->ev0, stream));
    const int engine = pick_engine(o, FC_ENGINE_PERSISTENT);
    QLocal q;
    std::memset(&q, 0, sizeof(q));
    if (engine == FC_ENGINE_HOSTLOOP) {
        rc = hostloop(c, MODE_STCON, gp, s, t, o.sched, &q, stream);
        if (rc) return rc;
        // clear the claimed status bytes (whole array: one memset)
        FC_CUDA_TRY(cudaMemsetAsync(c->status, 0xFF, (size_t)(nv + 15) / 16 * 16, stream));
        *conn = q.connected;
        *hops = q.hops;
    } else if (engine == FC_ENGINE_PERSISTENT || engine == FC_ENGINE_BATCHED) {
        rc = ensure_graphs(c, &gp, 1, stream);
        if (rc) return rc;
        if (c->qstat_cap < 1) {
            FC_CUDA_TRY(cudaMalloc(&c->qstat, sizeof(QueryStat) * 1024));
            c->qstat_cap = 1024;
        }
        if (c->tmp_q_cap < 4) {
            cudaFree(c->d_tmp_q);
            c->d_tmp_q = nullptr;
            FC_CUDA_TRY(cudaMalloc(&c->d_tmp_q, sizeof(int32_t) * 4096));
            c->tmp_q_cap = 4096;
        }
        int32_t hq[2] = {s, t};
        FC_CUDA_TRY(cudaMemcpyAsync(c->d_tmp_q, hq, sizeof(hq), cudaMemcpyHostToDevice, stream));
        FC_CUDA_TRY(cudaMemsetAsync(c->qstat, 0, sizeof(QueryStat), stream));
        PersistArgs a;
        std::memset(&a, 0, sizeof(a));
        a.graphs = (const GraphPair *)c->d_graphs;
        a.qs = c->d_tmp_q;
        a.qt = c->d_tmp_q + 1;
        a.nlist = 1;
        a.mode = MODE_STCON;
        a.sched = o.sched;
        a.status = c->status;
        a.levels = c->levels;
        a.log = c->log;
        a.tc = c->tc;
        a.out_conn = c->d_tmp_q + 2;
        a.out_hops = c->d_tmp_q + 3;
        a.qstat = c->qstat;
        rc = launch_persistent<FC_BLOCK>(c, a, stream);
        if (rc) return rc;
        rc = check_counters(c, stream);
        if (rc) return rc;
        int32_t res[2];
        FC_CUDA_TRY(cudaMemcpy(res, c->d_tmp_q + 2, sizeof(res), cudaMemcpyDeviceToHost));
        QueryStat h;
        FC_CUDA_TRY(cudaMemcpy(&h, c->qstat, sizeof(h), cudaMemcpyDeviceToHost));
        *conn = res[0];
        *hops = res[1];
        from_qstat(q, h);
    } else {
        return FC_ERR_UNSUPPORTED;
    }
    FC_CUDA_TRY(cudaEventRecord(c->ev1, stream));
    FC_CUDA_TRY(cudaStreamSynchronize(stream));
    if (st) {
        fill_stats(st, q, engine == FC_ENGINE_HOSTLOOP ? q.steps + 1 : 1);
        float ms = 0;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        st->gpu_ms = ms;
    }
    return FC_OK;
}

// ---------------------------------------------------------------------------
// batched engine host side
// ---------------------------------------------------------------------------
static int ensure_batch_arena(DevCtx *c, size_t slots, size_t maxnv, int log_cap)
{
    size_t sstride = (maxnv + 255) / 256 * 256;
    size_t lstride = ((size_t)log_cap + 63) / 64 * 64;
    if (c->b_status && c->b_slots >= slots && c->b_status_stride >= sstride &&
        c->b_log_stride >= lstride && c->b_log_cap >= log_cap)
        return FC_OK;
    cudaFree(c->b_status);
    cudaFree(c->b_log);
    c->b_status = nullptr;
    c->b_log = nullptr;
    c->b_slots = 0;
    FC_CUDA_TRY(cudaMalloc(&c->b_status, slots * sstride));
    FC_CUDA_TRY(cudaMalloc(&c->b_log, slots * lstride * sizeof(int32_t)));
    FC_CUDA_TRY(cudaMemset(c->b_status, 0xFF, slots * sstride));
    c->b_slots = slots;
    c->b_status_stride = sstride;
    c->b_log_stride = lstride;
    c->b_log_cap = log_cap;
    return FC_OK;
}

int engine_stcon_batch(DevCtx *c, const GraphPairH *gps, int ngraphs, const int32_t *d_gi,
                       const int32_t *d_s, const int32_t *d_t, int32_t nq, int32_t *d_conn,
                       int32_t *d_hops, const fc_opts &o, fc_stats *st, cudaStream_t stream,
                       bool sync)
{
    constexpr int T = FC_BLOCK;
    if (nq <= 0) return FC_OK;
    size_t maxnv = 1;
    long long max_ne = 0;
    for (int i = 0; i < ngraphs; ++i) {
        if ((size_t)gps[i].fwd.nv > maxnv) maxnv = (size_t)gps[i].fwd.nv;
        if (gps[i].fwd.ne > max_ne) max_ne = gps[i].fwd.ne;
    }
    int rc = ensure_ws(c, maxnv);
    if (rc) return rc;
    rc = ensure_graphs(c, gps, ngraphs, stream);
    if (rc) return rc;
    if ((size_t)nq > c->qstat_cap) {
        cudaFree(c->qstat);
        c->qstat = nullptr;
        c->qstat_cap = 0;
        FC_CUDA_TRY(cudaMalloc(&c->qstat, sizeof(QueryStat) * (size_t)nq));
        c->qstat_cap = (size_t)nq;
    }
    if ((size_t)nq > c->b_spill_cap) {
        cudaFree(c->b_spill);
        c->b_spill = nullptr;
        c->b_spill_cap = 0;
        FC_CUDA_TRY(cudaMalloc(&c->b_spill, sizeof(int32_t) * (size_t)nq));
        c->b_spill_cap = (size_t)nq;
    }
    const int engine = pick_engine(o, FC_ENGINE_BATCHED);
    FC_CUDA_TRY(cudaEventRecord(c->ev0, stream));
    FC_CUDA_TRY(cudaMemsetAsync(c->qstat, 0, sizeof(QueryStat) * (size_t)nq, stream));
    FC_CUDA_TRY(cudaMemsetAsync(c->b_ctr, 0, 4 * sizeof(int), stream));
    if (engine == FC_ENGINE_BATCHED) {
        int per_sm = o.ctas_per_sm;
        if (per_sm <= 0) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batched<T>, T, 0);
            if (per_sm > 4) per_sm = 4;
        }
        if (per_sm < 1) per_sm = 1;
        size_t slots = (size_t)per_sm * (size_t)c->sm_count;
        if (o.max_slots > 0 && (size_t)o.max_slots < slots) slots = (size_t)o.max_slots;
        if (slots > (size_t)nq) slots = (size_t)nq;
        // log space per slot: enough for the CTA work limit
        const long long work_limit = 1ll << 20;
        int log_cap = (int)std::min<size_t>(maxnv, (size_t)(2 * work_limit + 1024));
        rc = ensure_batch_arena(c, slots, maxnv, log_cap);
        if (rc) return rc;
        BatchArgs b;
        b.graphs = (const GraphPair *)c->d_graphs;
        b.graph_idx = d_gi;
        b.qs = d_s;
        b.qt = d_t;
        b.nq = nq;
        b.ctr = c->b_ctr;
        b.spill = c->b_spill;
        b.status_arena = c->b_status;
        b.status_stride = c->b_status_stride;
        b.log_arena = c->b_log;
        b.log_stride = c->b_log_stride;
        b.log_cap = log_cap;
        b.work_limit = work_limit;
        b.sched = o.sched == FC_SCHED_PLAIN ? FC_SCHED_HEURISTIC : o.sched;
        b.out_conn = d_conn;
        b.out_hops = d_hops;
        b.qstat = c->qstat;
        k_batched<T><<<(unsigned)slots, T, 0, stream>>>(b);
        FC_CUDA_TRY(cudaGetLastError());
        FC_CUDA_TRY(cudaEventRecord(c->evm, stream));
        PersistArgs a;
        std::memset(&a, 0, sizeof(a));
        a.graphs = (const GraphPair *)c->d_graphs;
        a.graph_idx = d_gi;
        a.qs = d_s;
        a.qt = d_t;
        a.list = c->b_spill;
        a.list_count = c->b_ctr + 1;
        a.mode = MODE_STCON;
        a.sched = o.sched == FC_SCHED_PLAIN ? FC_SCHED_HEURISTIC : o.sched;
        a.status = c->status;
        a.levels = c->levels;
        a.log = c->log;
        a.tc = c->tc;
        a.out_conn = d_conn;
        a.out_hops = d_hops;
        a.qstat = c->qstat;
        rc = launch_persistent<T>(c, a, stream);
        if (rc) return rc;
    } else if (engine == FC_ENGINE_PERSISTENT) {
        PersistArgs a;
        std::memset(&a, 0, sizeof(a));
        a.graphs = (const GraphPair *)c->d_graphs;
        a.graph_idx = d_gi;
        a.qs = d_s;
        a.qt = d_t;
        a.nlist = nq;
        a.mode = MODE_STCON;
        a.sched = o.sched;
        a.status = c->status;
        a.levels = c->levels;
        a.log = c->log;
        a.tc = c->tc;
        a.out_conn = d_conn;
        a.out_hops = d_hops;
        a.qstat = c->qstat;
        rc = launch_persistent<T>(c, a, stream);
        if (rc) return rc;
    } else if (engine == FC_ENGINE_HOSTLOOP) {
        // the plain form: one host-driven query at a time
        std::vector<int32_t> hs(nq), ht(nq), hg(nq, 0), hc(nq), hh(nq);
        FC_CUDA_TRY(cudaMemcpyAsync(hs.data(), d_s, sizeof(int32_t) * nq, cudaMemcpyDeviceToHost, stream));
        FC_CUDA_TRY(cudaMemcpyAsync(ht.data(), d_t, sizeof(int32_t) * nq, cudaMemcpyDeviceToHost, stream));
        if (d_gi)
            FC_CUDA_TRY(cudaMemcpyAsync(hg.data(), d_gi, sizeof(int32_t) * nq, cudaMemcpyDeviceToHost, stream));
        FC_CUDA_TRY(cudaStreamSynchronize(stream));
        QLocal tot;
        std::memset(&tot, 0, sizeof(tot));
        for (int i = 0; i < nq; ++i) {
            const GraphPairH &g = gps[hg[i]];
            if (hs[i] < 0 || hs[i] >= g.fwd.nv || ht[i] < 0 || ht[i] >= g.fwd.nv) {
                hc[i] = 0;
                hh[i] = -2;
                continue;
            }
            QLocal q;
            rc = hostloop(c, MODE_STCON, g, hs[i], ht[i], o.sched, &q, stream);
            if (rc) return rc;
            FC_CUDA_TRY(cudaMemsetAsync(c->status, 0xFF, (size_t)(g.fwd.nv + 15) / 16 * 16, stream));
            hc[i] = q.connected;
            hh[i] = q.hops;
            tot.inspected += q.inspected;
            tot.alg_bytes += q.alg_bytes;
            tot.tail[0] += q.tail[0] + q.tail[1];
            tot.steps += q.steps;
            tot.bu_steps += q.bu_steps;
        }
        FC_CUDA_TRY(cudaMemcpyAsync(d_conn, hc.data(), sizeof(int32_t) * nq, cudaMemcpyHostToDevice, stream));
        FC_CUDA_TRY(cudaMemcpyAsync(d_hops, hh.data(), sizeof(int32_t) * nq, cudaMemcpyHostToDevice, stream));
        FC_CUDA_TRY(cudaEventRecord(c->ev1, stream));
        FC_CUDA_TRY(cudaStreamSynchronize(stream));
        if (st) {
            fill_stats(st, tot, tot.steps + nq);
            float ms = 0;
            cudaEventElapsedTime(&ms, c->ev0, c->ev1);
            st->gpu_ms = ms;
        }
        return FC_OK;
    } else {
        return FC_ERR_UNSUPPORTED;
    }
    FC_CUDA_TRY(cudaEventRecord(c->ev1, stream));
    if (sync || st) {
        rc = check_counters(c, stream);
        if (rc) return rc;
    }
    if (st) {
        std::vector<QueryStat> h(nq);
        FC_CUDA_TRY(cudaMemcpy(h.data(), c->qstat, sizeof(QueryStat) * nq, cudaMemcpyDeviceToHost));
        QLocal tot;
        std::memset(&tot, 0, sizeof(tot));
        long long bytes_k[2] = {0, 0};
        int esc = 0;
        for (int i = 0; i < nq; ++i) {
            tot.inspected += (unsigned long long)h[i].inspected;
            tot.alg_bytes += (unsigned long long)h[i].alg_bytes;
            tot.tail[0] += h[i].visited;
            tot.steps += h[i].steps;
            tot.bu_steps += h[i].bu_steps;
            esc += h[i].escalated;
            bytes_k[h[i].escalated ? 1 : 0] += h[i].alg_bytes;
        }
        const bool batched = engine == FC_ENGINE_BATCHED;
        fill_stats(st, tot, batched ? 2 : 1);
        st->escalated = esc;
        float ms = 0;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        st->gpu_ms = ms;
        if (batched) {
            float m0 = 0, m1 = 0;
            cudaEventElapsedTime(&m0, c->ev0, c->evm);
            cudaEventElapsedTime(&m1, c->evm, c->ev1);
            st->kernel_ms[0] = m0;
            st->kernel_ms[1] = m1;
            st->kernel_alg_bytes[0] = bytes_k[0];
            st->kernel_alg_bytes[1] = bytes_k[1];
        } else {
            st->kernel_ms[1] = ms;
            st->kernel_alg_bytes[1] = bytes_k[0] + bytes_k[1];
        }
    }
    return FC_OK;
}

}  // namespace fc
