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
//   batched     the work-sharing engine of fc_pool.cu (the default for every
//               call): each CTA owns queries, big steps are shared as tiles.
//               A query whose visit log could outgrow its slot is finished by
//               a second, exclusive launch of the same kernel in the stream.
//
// s-t connectivity grows a ball from s (side 0) and from t (side 1), one side
// per step.  With both balls complete and disjoint, the first edge from the
// expanding side's frontier (radius r_x) into the other ball (radius r_y)
// proves d(s,t) = r_x + 1 + r_y: a shorter path would put a vertex in both
// balls, and any ball vertex adjacent to the frontier must sit on the other
// ball's outer level.  So the meeting step may stop early and the distance is
// still exact (the reference returns only ceil(d/2), S/make_stcon.c:1496).
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "fc_engine.h"
#include "fc_pool.h"
#include "fc_sched.cuh"

namespace fc {

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
    int variant;
    unsigned long long *hist;  // degree-bin counters of the side (learned schedule)
    int2 *jobs;                // row jobs (rows over TEAM_SPLIT_E entries)
    int jcap;
    int tile_v;                // frontier vertices per top-down tile
};

template <int T>
__global__ void __launch_bounds__(T) k_step(StepArgs a)
{
    __shared__ SmemTopDown<T> sm;
    run_step<T>(a.mode, a.gp, a.side, a.dir, a.level, a.other_radius, a.log + a.front_begin, a.F,
                blockIdx.x, gridDim.x, a.status, a.levels, a.log, a.cap, &a.tc->tail[a.side],
                &a.tc->deg[a.side], &a.tc->found, &a.tc->inspected, sm, a.variant, a.hist,
                TeamSink{a.jobs, a.jcap, &a.tc->njobs[0], &a.tc->nok[0]}, a.tile_v);
}

// The row jobs the preceding k_step left, on the whole grid.
template <int T>
__global__ void __launch_bounds__(T) k_rowjobs(StepArgs a)
{
    __shared__ SmemTopDown<T> sm;
    const int nj = min(*(volatile const int *)&a.tc->nok[0], a.jcap);
    run_team_jobs<T>(a.mode, a.gp, a.side, a.level, a.jobs, nj, blockIdx.x, gridDim.x, a.status,
                     a.levels, a.log, a.cap, &a.tc->tail[a.side], &a.tc->deg[a.side],
                     &a.tc->found, sm, a.hist, &a.tc->inspected);
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
    int mode, sched, force_variant;
    uint8_t *status;
    int32_t *levels;
    int32_t *log;
    TeamCounters *tc;
    int32_t *out_conn;
    int32_t *out_hops;
    QueryStat *qstat;
    const float *mlp;  // learned schedule weights (nullable)
    int2 *jobs;        // row jobs of top-down steps
    int jcap;
};

// One step of k_persistent and its row jobs.
template <int T>
__device__ __forceinline__ void persist_step(const PersistArgs &a, const GraphPair &gp, const QLocal &ql,
                                          int x, const int32_t *front, int F, int par,
                                          SmemTopDown<T> &sm)
{
    TeamCounters *tc = a.tc;
    const int nv = gp.fwd.nv;
    run_step<T>(a.mode, gp, x, ql.dir, ql.radius[x], ql.radius[1 - x], front, F, blockIdx.x,
                gridDim.x, a.status, a.levels, a.log, nv, &tc->tail[x], &tc->deg[x], &tc->found,
                &tc->inspected, sm, ql.variant, a.mlp ? &tc->hist[x] : nullptr,
                TeamSink{a.jobs, a.jcap, &tc->njobs[par], &tc->nok[par]},
                team_tile_v<T>(F, (long long)(ql.dt[x] - ql.dh[x])));
}

template <int T>
__device__ __forceinline__ void persist_jobs(const PersistArgs &a, const GraphPair &gp, const QLocal &ql,
                                          int x, int nj, SmemTopDown<T> &sm)
{
    TeamCounters *tc = a.tc;
    run_team_jobs<T>(a.mode, gp, x, ql.radius[x], a.jobs, nj, blockIdx.x, gridDim.x, a.status,
                     a.levels, a.log, gp.fwd.nv, &tc->tail[x], &tc->deg[x], &tc->found, sm,
                     a.mlp ? &tc->hist[x] : nullptr, &tc->inspected);
}

template <int T>
__global__ void __launch_bounds__(T, 768 / T) k_persistent(PersistArgs a)
{
    __shared__ SmemTopDown<T> sm;
    __shared__ QLocal ql;
    TeamCounters *tc = a.tc;
    const int nq = a.list_count ? *(volatile const int *)a.list_count : a.nlist;
    for (int li = 0; li < nq; ++li) {
        const int q = a.list ? a.list[li] : li;
        const GraphPair gp = a.graphs[a.graph_idx ? a.graph_idx[q] : 0];
        const int nv = gp.fwd.nv;
        int s = a.qs[q];
        int t = a.mode == MODE_STCON ? a.qt[q] : s;
        const bool bad = s < 0 || s >= nv || t < 0 || t >= nv;
        if (bad) {  // uniform across the grid: no barrier needed to skip
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                if (a.out_conn) a.out_conn[q] = 0;
                if (a.out_hops) a.out_hops[q] = -2;
                atomicExch(&tc->invalid, 1);
            }
            continue;
        }
        if (gp.fwd.remap) {  // a renumbered copy of the graph: the caller's ids map into it
            s = __ldg(gp.fwd.remap + s);
            t = __ldg(gp.fwd.remap + t);
        }
        if (blockIdx.x == 0 && threadIdx.x == 0)
            init_roots(a.mode, gp, s, t, a.status, a.levels, a.log, nv, tc);
        // counters are read from the barrier's snapshot: fast CTAs may
        // already be claiming for the next step
        int g = grid_barrier_snap(tc->bar, &tc->err, gridDim.x, SnapTeam{tc});
        if (g < 0) return;
        if (threadIdx.x == 0)
            ql_start(ql, a.mode == MODE_STCON, nv, gp.fwd.ne, s, t,
                     ld_cg_u64(&tc->snap[g & 1].deg[0]), ld_cg_u64(&tc->snap[g & 1].deg[1]));
        __syncthreads();
        const int bu_cap = a.mode == MODE_BFS ? 0x7fffffff : LEVEL7_MAX;
        while (true) {
            if (threadIdx.x == 0 && !ql.done) {
                ql_decide(ql, a.sched, 1, bu_cap, 0, a.force_variant);
                if (a.mlp && mlp_worth(ql)) {  // every CTA computes the same decision
                    float f[MLP_IN], o[MLP_OUT];
                    ql_features(ql, f);
                    if (mlp_in_box(a.mlp, f)) {
                        mlp_forward_scalar(a.mlp, f, o);
                        ql_apply_logits(ql, o, 1, bu_cap);
                        if (a.force_variant >= 0) ql.variant = a.force_variant;
                    }
                }
            }
            __syncthreads();
            if (ql.done) break;
            int F;
            const int x = ql.side;
            const int32_t *front = ql_frontier(ql, a.log, nv, x, &F);
            // row-job counters alternate by step parity: the other parity's
            // were last read before the previous step's final barrier, so
            // clearing them now cannot race with a reader or a pusher
            const int par = ql.steps & 1;
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                tc->njobs[par ^ 1] = 0;
                tc->nok[par ^ 1] = 0;
            }
            persist_step<T>(a, gp, ql, x, front, F, par, sm);
            g = grid_barrier_snap(tc->bar, &tc->err, gridDim.x, SnapTeam{tc});
            if (g < 0) return;
            if (ql.dir == DIR_TD) {
                __shared__ int s_nj;
                if (threadIdx.x == 0) s_nj = min(ld_cg(&tc->snap[g & 1].nok[par]), a.jcap);
                __syncthreads();
                if (s_nj > 0) {  // same value in every CTA: uniform barrier
                    persist_jobs<T>(a, gp, ql, x, s_nj, sm);
                    g = grid_barrier_snap(tc->bar, &tc->err, gridDim.x, SnapTeam{tc});
                    if (g < 0) return;
                }
            }
            if (threadIdx.x == 0) {
                const TeamSnap &S = tc->snap[g & 1];
                ql_update(ql, ld_cg(&S.found), ld_cg(&S.tail[x]), ld_cg_u64(&S.deg[x]),
                          ld_cg_u64(&S.inspected));
                if (a.mlp) {
                    ql_update_hist(ql, x, ld_cg_u64(&S.hist[x]));
                }
            }
            __syncthreads();
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) write_result(q, ql, a.out_conn, a.out_hops, a.qstat, 0);
        if (a.mode == MODE_STCON) {
            // clear exactly the claimed vertices (the log holds each once)
            const int n0 = ql.tail[0], n1 = ql.tail[1];
            clear_claimed(a.status, a.log, nv, n0, 0, (long long)n0 + n1,
                          (long long)blockIdx.x * T + threadIdx.x, (long long)gridDim.x * T);
        }
        if (!grid_barrier(tc->bar, &tc->err, gridDim.x)) return;
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
            cudaMalloc(&c->b_ctr, 8 * sizeof(int)) != cudaSuccess ||
            cudaMallocHost(&c->h_bctr, 8 * sizeof(int)) != cudaSuccess) {
            *err = FC_ERR_CUDA;
            set_error("device context set-up failed");
            return nullptr;
        }
        cudaMemset(c->tc, 0, sizeof(TeamCounters));
        // set-up work runs on the legacy stream; the traversal kernels run on
        // non-blocking streams, which do not wait for it: finish it here
        cudaDeviceSynchronize();
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
    if (!c->tjobs) {
        // 2^20 jobs of 4096 entries: any step of a graph of up to 2^31 entries
        FC_CUDA_TRY(cudaMalloc(&c->tjobs, sizeof(int2) << 20));
        c->tjobs_cap = 1 << 20;
    }
    FC_CUDA_TRY(cudaMemset(c->status, 0xFF, sbytes));
    FC_CUDA_TRY(cudaDeviceSynchronize());  // before any kernel on another stream reads it
    c->ws_nv = nv;
    return FC_OK;
}

int ensure_workspace(DevCtx *c, size_t nv) { return ensure_ws(c, nv); }

static int ensure_graphs(DevCtx *c, const GraphPairH *gps, int n, cudaStream_t st)
{
    if ((size_t)n > c->graphs_cap) {
        cudaFree(c->d_graphs);
        c->d_graphs = nullptr;
        c->graphs_cap = 0;
        c->graphs_last.clear();
        FC_CUDA_TRY(cudaMalloc(&c->d_graphs, sizeof(GraphPair) * (size_t)n));
        c->graphs_cap = (size_t)n;
    }
    // repeated batches on the same graphs (the common case) skip the copy
    const size_t bytes = sizeof(GraphPair) * (size_t)n;
    if (c->graphs_last.size() == bytes && std::memcmp(c->graphs_last.data(), gps, bytes) == 0)
        return FC_OK;
    c->graphs_last.clear();
    FC_CUDA_TRY(cudaMemcpyAsync(c->d_graphs, gps, bytes, cudaMemcpyHostToDevice, st));
    c->graphs_last.assign(reinterpret_cast<const unsigned char *>(gps),
                          reinterpret_cast<const unsigned char *>(gps) + bytes);
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

// After the copy of tc to h_tc has completed.
static int counters_verdict(DevCtx *c)
{
    if (c->h_tc->err) {
        set_error("device-side wait timed out (bounded grid barrier)");
        // leave the workspace clean for the next call
        cudaMemset(c->tc, 0, sizeof(TeamCounters));
        if (c->status) cudaMemset(c->status, 0xFF, (c->ws_nv + 15) / 16 * 16);
        cudaDeviceSynchronize();
        return FC_ERR_TIMEOUT;
    }
    return FC_OK;
}

static int check_counters(DevCtx *c, cudaStream_t st)
{
    FC_CUDA_TRY(cudaMemcpyAsync(c->h_tc, c->tc, sizeof(TeamCounters), cudaMemcpyDeviceToHost, st));
    FC_CUDA_TRY(cudaStreamSynchronize(st));
    return counters_verdict(c);
}

// Host-loop engine: one launch per step; returns the final QLocal.
static int hostloop(DevCtx *c, int mode, const GraphPairH &gph, int s, int t, int sched,
                    QLocal *out, cudaStream_t st, int force_variant = -1)
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
    const int bu_cap = mode == MODE_BFS ? 0x7fffffff : LEVEL7_MAX;
    const bool learned = sched == FC_SCHED_LEARNED && c->mlp_ready;
    while (!q.done) {
        ql_decide(q, sched, 1, bu_cap, 0, force_variant);
        if (learned && mlp_worth(q)) {
            float f[MLP_IN], o[MLP_OUT];
            ql_features(q, f);
            if (mlp_in_box(c->h_mlp, f)) {
                mlp_forward_scalar(c->h_mlp, f, o);
                ql_apply_logits(q, o, 1, bu_cap);
                if (force_variant >= 0) q.variant = force_variant;
            }
        }
        const int x = q.side;
        StepArgs a;
        a.gp = gp;
        a.mode = mode;
        a.side = x;
        a.dir = q.dir;
        a.level = q.radius[x];
        a.other_radius = q.radius[1 - x];
        a.variant = q.variant;
        a.F = q.tail[x] - q.head[x];
        a.front_begin = x == 0 ? q.head[0] : nv - q.tail[1];
        a.status = c->status;
        a.levels = c->levels;
        a.log = c->log;
        a.cap = nv;
        a.tc = c->tc;
        a.hist = learned ? &c->tc->hist[x] : nullptr;
        a.jobs = c->tjobs;
        a.jcap = c->tjobs_cap;
        a.tile_v = team_tile_v<T>(a.F, (long long)(q.dt[x] - q.dh[x]));
        int grid = q.dir == DIR_TD ? (a.F + a.tile_v - 1) / a.tile_v : full_grid;
        if (grid > full_grid) grid = full_grid;
        if (grid < 1) grid = 1;
        // rows over TEAM_SPLIT_E entries become row jobs for a second,
        // full-grid launch (only possible when the frontier has that many)
        const bool jobs = q.dir == DIR_TD && q.dt[x] - q.dh[x] > (unsigned long long)TEAM_SPLIT_E;
        if (jobs) FC_CUDA_TRY(cudaMemsetAsync(c->tc->njobs, 0, 4 * sizeof(int), st));
        else a.jcap = 0;
        k_step<T><<<grid, T, 0, st>>>(a);
        FC_CUDA_TRY(cudaGetLastError());
        if (jobs) {
            k_rowjobs<T><<<full_grid, T, 0, st>>>(a);
            FC_CUDA_TRY(cudaGetLastError());
        }
        FC_CUDA_TRY(cudaMemcpyAsync(c->h_tc, c->tc, sizeof(TeamCounters), cudaMemcpyDeviceToHost, st));
        FC_CUDA_TRY(cudaStreamSynchronize(st));
        ql_update(q, c->h_tc->found, c->h_tc->tail[x], c->h_tc->deg[x], c->h_tc->inspected);
        if (learned) ql_update_hist(q, x, c->h_tc->hist[x]);
    }
    *out = q;
    return FC_OK;
}

static int forced_variant(const fc_opts &o) { return o.variant > 0 ? o.variant - 1 : -1; }

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
    st->visited_adjacency = (int64_t)(q.dt[0] + q.dt[1]);
}

static void accumulate(QLocal &tot, const QueryStat &h)
{
    tot.inspected += (unsigned long long)h.inspected;
    tot.alg_bytes += (unsigned long long)h.alg_bytes;
    tot.tail[0] += h.visited;
    tot.dt[0] += (unsigned long long)h.visited_deg;
    tot.steps += h.steps;
    tot.bu_steps += h.bu_steps;
}

static int ensure_qstat(DevCtx *c, size_t n)
{
    if (n <= c->qstat_cap && c->qstat) return FC_OK;
    cudaFree(c->qstat);
    c->qstat = nullptr;
    c->qstat_cap = 0;
    size_t cap = n < 1024 ? 1024 : n;
    FC_CUDA_TRY(cudaMalloc(&c->qstat, sizeof(QueryStat) * cap));
    c->qstat_cap = cap;
    return FC_OK;
}

int32_t *batch_staging(DevCtx *c, size_t n, int *rc)
{
    *rc = FC_OK;
    if (c->b_stage && c->b_stage_cap >= n) return c->b_stage;
    cudaFree(c->b_stage);
    c->b_stage = nullptr;
    c->b_stage_cap = 0;
    size_t cap = n < 4096 ? 4096 : n;
    cudaError_t e = cudaMalloc(&c->b_stage, sizeof(int32_t) * 5 * cap);
    if (e != cudaSuccess) {
        fc_set_last_cuda_error(e, "cudaMalloc(batch staging)", __FILE__, __LINE__);
        *rc = e == cudaErrorMemoryAllocation ? FC_ERR_OOM : FC_ERR_CUDA;
        return nullptr;
    }
    c->b_stage_cap = cap;
    return c->b_stage;
}

// One CTA in a barrier sized for two: the wait can only expire.
__global__ void k_wait_selftest(int *bar, int *err, unsigned long long timeout_ns)
{
    grid_barrier(bar, err, 2, timeout_ns);
}

int engine_selftest_wait(DevCtx *c, int timeout_ms, double *elapsed_ms, cudaStream_t stream)
{
    if (!c->selftest) FC_CUDA_TRY(cudaMalloc(&c->selftest, 4 * sizeof(int)));
    FC_CUDA_TRY(cudaMemsetAsync(c->selftest, 0, 4 * sizeof(int), stream));
    FC_CUDA_TRY(cudaEventRecord(c->ev0, stream));
    k_wait_selftest<<<1, 32, 0, stream>>>(c->selftest, c->selftest + 2,
                                          (unsigned long long)timeout_ms * 1000000ull);
    FC_CUDA_TRY(cudaGetLastError());
    FC_CUDA_TRY(cudaEventRecord(c->ev1, stream));
    int h[4];
    FC_CUDA_TRY(cudaMemcpyAsync(h, c->selftest, sizeof(h), cudaMemcpyDeviceToHost, stream));
    FC_CUDA_TRY(cudaStreamSynchronize(stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    if (elapsed_ms) *elapsed_ms = ms;
    if (h[2] == FC_ERR_TIMEOUT) {
        set_error("device-side wait expired after %.1f ms (self-test)", ms);
        return FC_ERR_TIMEOUT;
    }
    set_error("self-test: the wait did not report a timeout (flag %d)", h[2]);
    return FC_ERR_CUDA;
}

static int ensure_tmp(DevCtx *c)
{
    if (c->d_tmp_q) return FC_OK;
    FC_CUDA_TRY(cudaMalloc(&c->d_tmp_q, sizeof(int32_t) * 4096));
    c->tmp_q_cap = 4096;
    return FC_OK;
}

// per-CTA slot records of the pool engine, sized for the largest grid
static int ensure_pool(DevCtx *c)
{
    if (c->p_slots) return FC_OK;
    int grid = pool_max_grid(c->sm_count);
    if (grid <= 0 || !c->coop) {
        set_error("cooperative launch unavailable for the pool engine");
        return FC_ERR_UNSUPPORTED;
    }
    FC_CUDA_TRY(cudaMalloc(&c->p_slots, pool_slot_bytes() * (size_t)grid));
    FC_CUDA_TRY(cudaMalloc(&c->p_jobs, pool_job_bytes() * (size_t)grid));
    FC_CUDA_TRY(cudaMalloc(&c->p_open, sizeof(int) * (size_t)grid));
    FC_CUDA_TRY(cudaMemset(c->p_open, 0, sizeof(int) * (size_t)grid));
    FC_CUDA_TRY(cudaMemset(c->p_slots, 0, pool_slot_bytes() * (size_t)grid));
    FC_CUDA_TRY(cudaMemset(c->p_jobs, 0, pool_job_bytes() * (size_t)grid));
    FC_CUDA_TRY(cudaDeviceSynchronize());
    c->p_grid = grid;
    return FC_OK;
}

// After the copy of b_ctr to h_bctr has completed.
static int pool_verdict(DevCtx *c, int *invalid)
{
    const int *h = c->h_bctr;
    if (invalid) *invalid = h[4];
    if (h[3]) {
        set_error("device-side wait timed out in the pool engine");
        // leave every workspace clean for the next call
        cudaMemset(c->p_slots, 0, pool_slot_bytes() * (size_t)c->p_grid);
        cudaMemset(c->p_open, 0, sizeof(int) * (size_t)c->p_grid);
        if (c->status) cudaMemset(c->status, 0xFF, (c->ws_nv + 15) / 16 * 16);
        if (c->b_status) cudaMemset(c->b_status, 0xFF, c->b_slots * c->b_status_stride);
        cudaDeviceSynchronize();
        return FC_ERR_TIMEOUT;
    }
    return FC_OK;
}

static int check_pool(DevCtx *c, cudaStream_t st, int *invalid)
{
    FC_CUDA_TRY(cudaMemcpyAsync(c->h_bctr, c->b_ctr, 8 * sizeof(int), cudaMemcpyDeviceToHost, st));
    FC_CUDA_TRY(cudaStreamSynchronize(st));
    return pool_verdict(c, invalid);
}

int engine_finish_checks(DevCtx *c)
{
    const int e = c->deferred_engine;
    c->deferred_engine = -1;
    if (e < 0) return FC_OK;
    if (e != FC_ENGINE_PERSISTENT) {
        const int rc = pool_verdict(c, nullptr);
        if (rc) return rc;
    }
    return counters_verdict(c);
}

static long long private_edges_default(const fc_opts &o, bool)
{
    // steps reading more than 8192 entries are shared (R-MAT 24 batches on
    // the degree-ordered copy: 2K, 4K and 8K measured within 2% of each
    // other, 8K best with 16K-entry tiles); a negative setting shares every
    // step
    if (o.cta_work_k < 0) return 0;
    if (o.cta_work_k > 0) return (long long)o.cta_work_k * 1024;
    return 8192;
}

// Top-down tile and row-job sizes of the pool engine (entries): the options'
// values when set, clamped to sane ranges, else the tuned defaults.  Batches
// (many owners, claims spread over their slots) balance best with small
// tiles -- 16K entries on the degree-ordered copy, where a tile's meeting
// comes early (R-MAT 24: 0.239 -> 0.230 ms against 8K, 4K slower); one query
// on the whole grid (every claim on one slot word) with large ones.
static void pool_sizes(PoolArgs &a, const fc_opts &o, bool exclusive)
{
    a.tile_e = o.tile_entries > 0 ? std::min(std::max(o.tile_entries, 1024), 1 << 22)
                                  : (exclusive ? 65536 : 16384);
    a.split_e = o.job_entries > 0 ? std::min(std::max(o.job_entries, 1024), 1 << 22)
                                  : (exclusive ? 8192 : 2048);
}

// Device weights when the learned schedule is asked for and weights are loaded;
// without weights the learned schedule falls back to the heuristic.
static const float *learned_weights(DevCtx *c, const fc_opts &o)
{
    return (o.sched == FC_SCHED_LEARNED && c->mlp_ready) ? c->d_mlp : nullptr;
}

static PoolArgs pool_args_exclusive(DevCtx *c, int mode, const fc_opts &o)
{
    PoolArgs a;
    std::memset(&a, 0, sizeof(a));
    a.graphs = (const GraphPair *)c->d_graphs;
    a.mode = mode;
    a.sched = o.sched;
    a.force_variant = forced_variant(o);
    a.private_variant = -1;
    a.exclusive = 1;
    a.slots = (PoolSlot *)c->p_slots;
    a.open = c->p_open;
    a.jobs = (RowJob *)c->p_jobs;
    a.status_base = c->status;
    a.levels = c->levels;
    a.log_base = c->log;
    a.log_cap = (int)c->ws_nv;
    a.private_edges = private_edges_default(o, true);
    pool_sizes(a, o, true);
    a.ctr = c->b_ctr;
    a.qstat = c->qstat;
    a.mlp = learned_weights(c, o);
    return a;
}

static void apply_extras(PoolArgs &a, const BatchExtras *ex)
{
    if (!ex) return;
    a.script = ex->script;
    a.script_len = ex->script_len;
    a.trace = ex->trace;
    a.trace_cap = ex->trace_cap;
    a.trace_count = ex->trace_count;
    a.out_inspected = ex->inspected;
}

static int pick_engine(const fc_opts &o, int dflt)
{
    return o.engine == FC_ENGINE_AUTO ? dflt : o.engine;
}

// one query (BFS levels or s-t) on the persistent grid-barrier engine or the
// pool engine in exclusive mode; results land in c->d_tmp_q[2..3]
static int run_single(DevCtx *c, int mode, int engine, const GraphPairH &gp, int32_t s, int32_t t,
                      const fc_opts &o, QLocal &q, cudaStream_t stream)
{
    int rc = ensure_graphs(c, &gp, 1, stream);
    if (rc) return rc;
    if ((rc = ensure_qstat(c, 1)) || (rc = ensure_tmp(c))) return rc;
    int32_t hq[2] = {s, t};
    FC_CUDA_TRY(cudaMemcpyAsync(c->d_tmp_q, hq, sizeof(hq), cudaMemcpyHostToDevice, stream));
    FC_CUDA_TRY(cudaMemsetAsync(c->qstat, 0, sizeof(QueryStat), stream));
    if (engine == FC_ENGINE_PERSISTENT) {
        PersistArgs a;
        std::memset(&a, 0, sizeof(a));
        a.graphs = (const GraphPair *)c->d_graphs;
        a.qs = c->d_tmp_q;
        a.qt = c->d_tmp_q + 1;
        a.nlist = 1;
        a.mode = mode;
        a.sched = o.sched;
        a.force_variant = forced_variant(o);
        a.status = c->status;
        a.levels = c->levels;
        a.log = c->log;
        a.tc = c->tc;
        a.out_conn = c->d_tmp_q + 2;
        a.out_hops = c->d_tmp_q + 3;
        a.qstat = c->qstat;
        a.mlp = learned_weights(c, o);
        a.jobs = c->tjobs;
        a.jcap = c->tjobs_cap;
        rc = launch_persistent<FC_BLOCK>(c, a, stream);
        if (rc) return rc;
        rc = check_counters(c, stream);
        if (rc) return rc;
    } else {
        if ((rc = ensure_pool(c))) return rc;
        FC_CUDA_TRY(cudaMemsetAsync(c->b_ctr, 0, 8 * sizeof(int), stream));
        PoolArgs a = pool_args_exclusive(c, mode, o);
        a.qs = c->d_tmp_q;
        a.qt = c->d_tmp_q + 1;
        a.nlist = 1;
        a.out_conn = c->d_tmp_q + 2;
        a.out_hops = c->d_tmp_q + 3;
        rc = pool_launch(a, pool_grid(c->sm_count, 0, 256), 256, stream);
        if (rc) return rc;
        rc = check_pool(c, stream, nullptr);
        if (rc) return rc;
    }
    QueryStat h;
    FC_CUDA_TRY(cudaMemcpy(&h, c->qstat, sizeof(h), cudaMemcpyDeviceToHost));
    std::memset(&q, 0, sizeof(q));
    accumulate(q, h);
    return FC_OK;
}

// Levels of a search on a renumbered copy, back in the caller's numbering:
// out[v] = lev[remap[v]].
__global__ void k_levels_to_caller(const int32_t *lev, const int32_t *remap, int nv, int32_t *out)
{
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < nv;
         v += (long long)gridDim.x * blockDim.x)
        out[v] = __ldg(lev + __ldg(remap + v));
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
        rc = hostloop(c, MODE_BFS, gp, s, s, o.sched, &q, stream, forced_variant(o));
    } else {
        rc = run_single(c, MODE_BFS, engine, gp, s, s, o, q, stream);
    }
    if (rc) return rc;
    FC_CUDA_TRY(cudaEventRecord(c->ev1, stream));
    const int32_t *out = c->levels;
    if (gp.fwd.remap && h_levels) {  // the log is free once the search is done
        const int grid = (int)std::min<long long>(4096, ((long long)nv + 255) / 256);
        k_levels_to_caller<<<grid, 256, 0, stream>>>(c->levels, gp.fwd.remap, nv, c->log);
        FC_CUDA_TRY(cudaGetLastError());
        out = c->log;
    }
    if (h_levels)
        FC_CUDA_TRY(cudaMemcpyAsync(h_levels, out, sizeof(int32_t) * (size_t)nv,
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
        rc = hostloop(c, MODE_STCON, gp, s, t, o.sched, &q, stream, forced_variant(o));
        if (rc) return rc;
        // clear the claimed status bytes (whole array: one memset)
        FC_CUDA_TRY(cudaMemsetAsync(c->status, 0xFF, (size_t)(nv + 15) / 16 * 16, stream));
        *conn = q.connected;
        *hops = q.hops;
    } else {
        rc = run_single(c, MODE_STCON, engine, gp, s, t, o, q, stream);
        if (rc) return rc;
        int32_t res[2];
        FC_CUDA_TRY(cudaMemcpy(res, c->d_tmp_q + 2, sizeof(res), cudaMemcpyDeviceToHost));
        *conn = res[0];
        *hops = res[1];
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
// batches
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
    FC_CUDA_TRY(cudaDeviceSynchronize());  // the pool kernel runs on another stream
    c->b_slots = slots;
    c->b_status_stride = sstride;
    c->b_log_stride = lstride;
    c->b_log_cap = log_cap;
    return FC_OK;
}

int engine_stcon_batch(DevCtx *c, const GraphPairH *gps, int ngraphs, const int32_t *d_gi,
                       const int32_t *d_s, const int32_t *d_t, int32_t nq, int32_t *d_conn,
                       int32_t *d_hops, const fc_opts &o, fc_stats *st, cudaStream_t stream,
                       int check, const BatchExtras *ex, const BatchHostIO *hio)
{
    if (hio && pick_engine(o, FC_ENGINE_BATCHED) != FC_ENGINE_BATCHED) {
        set_error("host arrays are copied by the batched engine only");
        return FC_ERR_UNSUPPORTED;
    }
    const bool hio_checks = hio && check == BATCH_DEFER_CHECK && !st;
    constexpr int T = FC_BLOCK;
    c->deferred_engine = -1;
    if (nq <= 0) return FC_OK;
    if (ex && pick_engine(o, FC_ENGINE_BATCHED) != FC_ENGINE_BATCHED) {
        set_error("scripts and traces need the batched engine");
        return FC_ERR_UNSUPPORTED;
    }
    size_t maxnv = 1;
    for (int i = 0; i < ngraphs; ++i)
        if ((size_t)gps[i].fwd.nv > maxnv) maxnv = (size_t)gps[i].fwd.nv;
    int rc = ensure_ws(c, maxnv);
    if (rc) return rc;
    rc = ensure_graphs(c, gps, ngraphs, stream);
    if (rc) return rc;
    if ((rc = ensure_qstat(c, (size_t)nq))) return rc;
    if ((size_t)nq > c->b_spill_cap) {
        cudaFree(c->b_spill);
        c->b_spill = nullptr;
        c->b_spill_cap = 0;
        FC_CUDA_TRY(cudaMalloc(&c->b_spill, sizeof(int32_t) * (size_t)nq));
        c->b_spill_cap = (size_t)nq;
    }
    const int engine = pick_engine(o, FC_ENGINE_BATCHED);
    int launches = 0;
    int graph_use = 0;
    FC_CUDA_TRY(cudaEventRecord(c->ev0, stream));
    if (engine != FC_ENGINE_BATCHED) {
        FC_CUDA_TRY(cudaMemsetAsync(c->qstat, 0, sizeof(QueryStat) * (size_t)nq, stream));
        FC_CUDA_TRY(cudaMemsetAsync(c->b_ctr, 0, 8 * sizeof(int), stream));
    }
    if (engine == FC_ENGINE_BATCHED) {
        if ((rc = ensure_pool(c))) return rc;
        // three owner CTAs per SM (measured best on R-MAT-24 batches against 2
        // and 4); each owner costs a status array of the largest graph
        const int block = pool_block(o.block);
        int grid = pool_grid(c->sm_count, o.ctas_per_sm > 0 ? o.ctas_per_sm : 3, block);
        if (grid > c->p_grid) grid = c->p_grid;
        if (o.max_slots > 0 && o.max_slots < grid) grid = o.max_slots;
        // a slot's visit log bounds the queries it can finish itself; bigger
        // ones move to the exclusive pass below.  Full-size logs when the arena
        // fits in 40% of the free device memory (deep graphs such as grids
        // visit millions of vertices per query), otherwise as large as fits.
        size_t sstride = (maxnv + 255) / 256 * 256;
        size_t log_cap_sz = maxnv;
        if (!(c->b_status && c->b_slots >= (size_t)grid && c->b_status_stride >= sstride &&
              c->b_log_cap >= (int)maxnv)) {
            size_t free_b = 0, total_b = 0;
            cudaMemGetInfo(&free_b, &total_b);
            size_t held = c->b_slots * (c->b_status_stride + 4 * (size_t)c->b_log_cap);
            size_t budget = (size_t)(0.4 * (double)(free_b + held)) / (size_t)grid;
            size_t fit = budget > sstride ? (budget - sstride) / 4 : 0;
            if (fit < log_cap_sz) log_cap_sz = std::max<size_t>(fit, std::min<size_t>(maxnv, 1 << 16));
        }
        // a caller's cap (at least 1,024 entries) bounds the slots' logs too
        if (o.slot_log_cap > 0) log_cap_sz = std::min<size_t>(log_cap_sz, std::max(o.slot_log_cap, 1024));
        int log_cap = (int)log_cap_sz;
        rc = ensure_batch_arena(c, (size_t)grid, maxnv, log_cap);
        if (rc) return rc;
        PoolArgs a;
        std::memset(&a, 0, sizeof(a));
        a.graphs = (const GraphPair *)c->d_graphs;
        a.graph_idx = d_gi;
        a.qs = d_s;
        a.qt = d_t;
        a.nlist = nq;
        a.mode = MODE_STCON;
        a.sched = o.sched;
        a.force_variant = forced_variant(o);
        a.private_variant = o.private_variant > 0 ? o.private_variant - 1 : -1;
        a.exclusive = 0;
        a.slots = (PoolSlot *)c->p_slots;
        a.open = c->p_open;
        a.jobs = (RowJob *)c->p_jobs;
        a.status_base = c->b_status;
        a.status_stride = c->b_status_stride;
        a.log_base = c->b_log;
        a.log_stride = c->b_log_stride;
        a.log_cap = log_cap;
        a.private_edges = private_edges_default(o, false);
        pool_sizes(a, o, false);
        a.ctr = c->b_ctr;
        a.spill = c->b_spill;
        a.out_conn = d_conn;
        a.out_hops = d_hops;
        a.qstat = c->qstat;
        a.mlp = learned_weights(c, o);
        apply_extras(a, ex);
        // queries whose visit log outgrew their slot: one at a time on the
        // whole grid (grid engine over the spill list)
        PersistArgs x;
        std::memset(&x, 0, sizeof(x));
        x.graphs = (const GraphPair *)c->d_graphs;
        x.graph_idx = d_gi;
        x.qs = d_s;
        x.qt = d_t;
        x.list = c->b_spill;
        x.list_count = c->b_ctr + 2;
        x.mode = MODE_STCON;
        x.sched = o.sched;
        x.force_variant = forced_variant(o);
        x.status = c->status;
        x.levels = c->levels;
        x.log = c->log;
        x.tc = c->tc;
        x.out_conn = d_conn;
        x.out_hops = d_hops;
        x.qstat = c->qstat;
        x.mlp = learned_weights(c, o);
        x.jobs = c->tjobs;
        x.jcap = c->tjobs_cap;
        const int xgrid = coop_grid<T>(c);
        const size_t qb = sizeof(int32_t) * (size_t)nq;
        auto issue = [&](unsigned evflags) -> int {
            if (hio) {
                FC_CUDA_TRY(cudaMemcpyAsync((void *)d_s, hio->s, qb, cudaMemcpyHostToDevice, stream));
                FC_CUDA_TRY(cudaMemcpyAsync((void *)d_t, hio->t, qb, cudaMemcpyHostToDevice, stream));
                if (hio->gi)
                    FC_CUDA_TRY(cudaMemcpyAsync((void *)d_gi, hio->gi, qb, cudaMemcpyHostToDevice,
                                                stream));
            }
            FC_CUDA_TRY(cudaMemsetAsync(c->qstat, 0, sizeof(QueryStat) * (size_t)nq, stream));
            FC_CUDA_TRY(cudaMemsetAsync(c->b_ctr, 0, 8 * sizeof(int), stream));
            int r = pool_launch(a, grid, block, stream);
            if (r) return r;
            FC_CUDA_TRY(cudaEventRecordWithFlags(c->evm, stream, evflags));
            r = launch_persistent<T>(c, x, stream);
            if (r) return r;
            if (hio) {
                if (hio_checks) {  // the error words travel with the answers
                    FC_CUDA_TRY(cudaMemcpyAsync(c->h_bctr, c->b_ctr, 8 * sizeof(int),
                                                cudaMemcpyDeviceToHost, stream));
                    FC_CUDA_TRY(cudaMemcpyAsync(c->h_tc, c->tc, sizeof(TeamCounters),
                                                cudaMemcpyDeviceToHost, stream));
                }
                FC_CUDA_TRY(cudaMemcpyAsync(hio->conn, d_conn, qb, cudaMemcpyDeviceToHost, stream));
                FC_CUDA_TRY(cudaMemcpyAsync(hio->hops, d_hops, qb, cudaMemcpyDeviceToHost, stream));
            }
            return FC_OK;
        };
        if (o.use_graph) {
            // the two launches and their resets as one CUDA graph, replayed
            // while every argument (pointers, sizes, grids) stays the same
            // (the host arrays' addresses and whether the error words are
            // copied are part of the graph too)
            BatchHostIO hk;
            std::memset(&hk, 0, sizeof(hk));
            if (hio) hk = *hio;
            unsigned char key[sizeof(PoolArgs) + sizeof(PersistArgs) + 5 * sizeof(int) +
                              sizeof(BatchHostIO)];
            std::memcpy(key, &a, sizeof(PoolArgs));
            std::memcpy(key + sizeof(PoolArgs), &x, sizeof(PersistArgs));
            int tail[5] = {grid, xgrid, nq, block, (hio ? 1 : 0) | (hio_checks ? 2 : 0)};
            std::memcpy(key + sizeof(PoolArgs) + sizeof(PersistArgs), tail, sizeof(tail));
            std::memcpy(key + sizeof(PoolArgs) + sizeof(PersistArgs) + sizeof(tail), &hk,
                        sizeof(hk));
            static_assert(sizeof(key) <= sizeof(c->gkey), "graph key too large");
            if (!(c->gexec && c->gkey_len == sizeof(key) &&
                  std::memcmp(c->gkey, key, sizeof(key)) == 0)) {
                if (c->gexec) cudaGraphExecDestroy(c->gexec);
                c->gexec = nullptr;
                c->gkey_len = 0;
                FC_CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
                int r = issue(cudaEventRecordExternal);
                cudaGraph_t g = nullptr;
                cudaError_t e = cudaStreamEndCapture(stream, &g);
                if (r || e != cudaSuccess) {
                    if (g) cudaGraphDestroy(g);
                    if (!r) fc_set_last_cuda_error(e, "cudaStreamEndCapture", __FILE__, __LINE__);
                    return r ? r : FC_ERR_CUDA;
                }
                cudaGraphExec_t ge = nullptr;
                e = cudaGraphInstantiate(&ge, g, 0);
                cudaGraphDestroy(g);
                FC_CUDA_TRY(e);
                c->gexec = ge;
                std::memcpy(c->gkey, key, sizeof(key));
                c->gkey_len = sizeof(key);
                ++c->graph_captures;
                graph_use = 2;
            } else {
                ++c->graph_replays;
                graph_use = 1;
            }
            FC_CUDA_TRY(cudaGraphLaunch(c->gexec, stream));
        } else {
            rc = issue(cudaEventRecordDefault);
            if (rc) return rc;
        }
        launches = 2;
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
        a.force_variant = forced_variant(o);
        a.status = c->status;
        a.levels = c->levels;
        a.log = c->log;
        a.tc = c->tc;
        a.out_conn = d_conn;
        a.out_hops = d_hops;
        a.qstat = c->qstat;
        a.mlp = learned_weights(c, o);
        a.jobs = c->tjobs;
        a.jcap = c->tjobs_cap;
        rc = launch_persistent<T>(c, a, stream);
        if (rc) return rc;
        FC_CUDA_TRY(cudaEventRecord(c->evm, stream));
        launches = 1;
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
            rc = hostloop(c, MODE_STCON, g, hs[i], ht[i], o.sched, &q, stream, forced_variant(o));
            if (rc) return rc;
            FC_CUDA_TRY(cudaMemsetAsync(c->status, 0xFF, (size_t)(g.fwd.nv + 15) / 16 * 16, stream));
            hc[i] = q.connected;
            hh[i] = q.hops;
            tot.inspected += q.inspected;
            tot.alg_bytes += q.alg_bytes;
            tot.tail[0] += q.tail[0] + q.tail[1];
            tot.dt[0] += q.dt[0] + q.dt[1];
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
            st->kernel_ms[0] = ms;
            st->kernel_alg_bytes[0] = (int64_t)tot.alg_bytes;
        }
        return FC_OK;
    } else {
        return FC_ERR_UNSUPPORTED;
    }
    FC_CUDA_TRY(cudaEventRecord(c->ev1, stream));
    if (hio_checks) {  // queued with the answers
        c->deferred_engine = engine;
        return FC_OK;
    }
    if (check == BATCH_DEFER_CHECK && !st) {
        if (engine != FC_ENGINE_PERSISTENT)
            FC_CUDA_TRY(cudaMemcpyAsync(c->h_bctr, c->b_ctr, 8 * sizeof(int),
                                        cudaMemcpyDeviceToHost, stream));
        FC_CUDA_TRY(cudaMemcpyAsync(c->h_tc, c->tc, sizeof(TeamCounters), cudaMemcpyDeviceToHost,
                                    stream));
        c->deferred_engine = engine;
        return FC_OK;
    }
    if (check || st) {
        rc = engine == FC_ENGINE_PERSISTENT ? check_counters(c, stream) : check_pool(c, stream, nullptr);
        if (rc) return rc;
        if (engine == FC_ENGINE_BATCHED && (rc = check_counters(c, stream))) return rc;
    }
    if (st) {
        std::vector<QueryStat> h(nq);
        FC_CUDA_TRY(cudaMemcpy(h.data(), c->qstat, sizeof(QueryStat) * nq, cudaMemcpyDeviceToHost));
        QLocal tot;
        std::memset(&tot, 0, sizeof(tot));
        long long bytes_k[2] = {0, 0};
        int esc = 0;
        for (int i = 0; i < nq; ++i) {
            accumulate(tot, h[i]);
            esc += h[i].escalated;
            bytes_k[h[i].escalated ? 1 : 0] += h[i].alg_bytes;
        }
        fill_stats(st, tot, launches);
        st->escalated = esc;
        st->graph = graph_use;
        float ms = 0, m0 = 0, m1 = 0;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        cudaEventElapsedTime(&m0, c->ev0, c->evm);
        cudaEventElapsedTime(&m1, c->evm, c->ev1);
        st->gpu_ms = ms;
        st->kernel_ms[0] = m0;
        st->kernel_ms[1] = m1;
        st->kernel_alg_bytes[0] = bytes_k[0];
        st->kernel_alg_bytes[1] = bytes_k[1];
    }
    return FC_OK;
}

}  // namespace fc
