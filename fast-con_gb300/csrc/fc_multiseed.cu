// fc_multiseed.cu -- s~t connectivity by multi-seed region growth and a
// device union-find of region meetings (the BFS_4K_MULTI fork's semantics).
//
// The reference (KM/src/device/BFS_WorkEfficient.cu:9-233) grows BFS regions
// from NUM_SOURCES seeds at once -- seed 0 = s, seed 1 = t, the rest random --
// tags each vertex with the id of the region that reached it first, records
// a meeting in a bool[NUM_SOURCES^2] matrix whenever an edge joins two
// regions, and closes the matrix on the host side by repeated relaxation
// (AdjAnalysis, KM/.../BFS_WE_AdjMatrixAnalysis.cu:4-35) until s's and t's
// regions are linked.  Here the meetings go straight into a union-find over
// the region ids (lock-free hooking by atomicCAS, smaller root wins, path
// halving), so the closure is always current and the host reads one flag.
//
// Exactness.  Every edge between two labelled vertices of different regions
// is examined when the earlier-labelled endpoint is expanded, so at the end
// of the growth the union-find joins exactly the regions of each connected
// component that holds a seed; s~t is decided when the two roots agree (an
// early, exact yes) or when growth stops without that (an exact no).  Only
// undirected graphs: on a directed graph two regions meeting says nothing
// about a path from s to t.
//
// One level = one launch over the level's frontier (thread per vertex; rows
// over MS_SPLIT entries become jobs walked by whole warps in a second
// launch).  The frontier is a segment of an append-only visit log.
#include <climits>
#include <cstring>
#include <vector>

#include "fc_engine.h"
#include "fc_sched.cuh"

namespace fc {

constexpr int MS_BLOCK = 256;
constexpr int MS_SPLIT = 1024;     // rows longer than this become warp jobs
constexpr int MS_MAX_SEEDS = 4096;
constexpr int UF_MAX_STEPS = 1 << 20;  // bound on the lock-free retry loops

struct MsCounters {
    int tail;       // visit-log length
    int njobs;      // jobs of the current level
    int nok;        // jobs written
    int err;        // a union-find loop ran past its bound
    unsigned long long inspected;
};

__device__ __forceinline__ int uf_find(int *uf, int x, int *err)
{
    for (int it = 0; it < UF_MAX_STEPS; ++it) {
        const int p = ld_cg(uf + x);
        if (p == x) return x;
        const int gp = ld_cg(uf + p);
        if (gp != p) atomicCAS(uf + x, p, gp);  // path halving
        x = p;
    }
    atomicExch(err, 1);
    return x;
}

__device__ __forceinline__ void uf_union(int *uf, int a, int b, int *err)
{
    for (int it = 0; it < UF_MAX_STEPS; ++it) {
        a = uf_find(uf, a, err);
        b = uf_find(uf, b, err);
        if (a == b) return;
        if (a > b) {
            const int t = a;
            a = b;
            b = t;
        }
        if (atomicCAS(uf + b, b, a) == b) return;
    }
    atomicExch(err, 1);
}

struct MsArgs {
    const int32_t *row_ptr, *col;
    int32_t *label;   // region id per vertex, -1 unreached
    int32_t *log;     // every labelled vertex once, in level order
    int head, tail;   // this level's frontier: log[head, tail)
    int *uf;          // union-find over region ids
    MsCounters *ctr;
    int4 *jobs;       // {b, e, region, 0}
    int jcap;
};

// the edge (region L) -> v
__device__ __forceinline__ void ms_visit(const MsArgs &a, int L, int v)
{
    int lv = ld_cg(a.label + v);
    if (lv < 0) {
        lv = atomicCAS(a.label + v, -1, L);
        if (lv < 0) {
            a.log[atomicAdd(&a.ctr->tail, 1)] = v;
            return;
        }
    }
    if (lv != L) uf_union(a.uf, L, lv, &a.ctr->err);
}

__global__ void __launch_bounds__(MS_BLOCK) k_ms_step(MsArgs a)
{
    unsigned long long ins = 0;
    for (int i = a.head + blockIdx.x * blockDim.x + threadIdx.x; i < a.tail;
         i += gridDim.x * blockDim.x) {
        const int u = a.log[i];
        const int L = a.label[u];
        const int b = a.row_ptr[u], e = a.row_ptr[u + 1];
        if (e - b > MS_SPLIT) {
            const int n = (e - b + MS_SPLIT - 1) / MS_SPLIT;
            const int k = atomicAdd(&a.ctr->njobs, n);
            if (k + n <= a.jcap) {
                for (int j = 0; j < n; ++j)
                    a.jobs[k + j] = make_int4(b + j * MS_SPLIT, min(e, b + (j + 1) * MS_SPLIT), L, 0);
                atomicAdd(&a.ctr->nok, n);
                continue;
            }
        }
        ins += (unsigned long long)(e - b);
        for (int j = b; j < e; j += 4) {
            int v[4], lv[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) v[k] = j + k < e ? __ldg(a.col + j + k) : -1;
#pragma unroll
            for (int k = 0; k < 4; ++k) lv[k] = v[k] >= 0 ? ld_cg(a.label + v[k]) : 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (v[k] < 0) continue;
                if (lv[k] < 0 || lv[k] != L) ms_visit(a, L, v[k]);
            }
        }
    }
    ins = warp_sum_ll((long long)ins);
    if (lane_id() == 0 && ins) atomicAdd(&a.ctr->inspected, ins);
}

// jobs of long rows: one warp per job
__global__ void __launch_bounds__(MS_BLOCK) k_ms_jobs(MsArgs a)
{
    const int nj = min(ld_cg(&a.ctr->nok), a.jcap);
    const int warps = gridDim.x * (blockDim.x / 32);
    unsigned long long ins = 0;
    for (int w = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); w < nj; w += warps) {
        const int4 J = a.jobs[w];
        if (lane_id() == 0) ins += (unsigned long long)(J.y - J.x);
        for (int j = J.x + (int)lane_id(); j < J.y; j += 32) {
            const int v = __ldg(a.col + j);
            const int lv = ld_cg(a.label + v);
            if (lv < 0 || lv != J.z) ms_visit(a, J.z, v);
        }
    }
    ins = warp_sum_ll((long long)ins);
    if (lane_id() == 0 && ins) atomicAdd(&a.ctr->inspected, ins);
}

__global__ void k_ms_init(int32_t *label, int32_t *log, int *uf, const int32_t *seeds, int k,
                          MsCounters *ctr)
{
    // one thread: seeds in order, a seed already taken by an earlier seed
    // joins that seed's region
    if (blockIdx.x || threadIdx.x) return;
    int n = 0;
    for (int i = 0; i < k; ++i) {
        uf[i] = i;
        const int v = seeds[i];
        if (label[v] < 0) {
            label[v] = i;
            log[n++] = v;
        } else {
            uf[i] = label[v];  // label[v] < i is a root at this point
        }
    }
    ctr->tail = n;
    ctr->njobs = ctr->nok = ctr->err = 0;
    ctr->inspected = 0;
}

__global__ void k_ms_same(int *uf, MsCounters *ctr, int *out)
{
    if (blockIdx.x || threadIdx.x) return;
    *out = uf_find(uf, 0, &ctr->err) == uf_find(uf, 1, &ctr->err);
}

int engine_stcon_multiseed(DevCtx *c, const GraphPairH &gp, int32_t s, int32_t t, int32_t nseeds,
                           unsigned long long seed, int32_t *connected, fc_stats *st,
                           cudaStream_t stream)
{
    const int nv = gp.fwd.nv;
    if (nseeds < 2 || nseeds > MS_MAX_SEEDS) {
        set_error("nseeds %d outside [2, %d]", nseeds, MS_MAX_SEEDS);
        return FC_ERR_INVALID;
    }
    // seeds: s, t, then a counter-based hash of (seed, i) mapped onto [0, nv)
    std::vector<int32_t> hs((size_t)nseeds);
    hs[0] = s;
    hs[1] = t;
    for (int i = 2; i < nseeds; ++i) {
        unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(i + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        hs[(size_t)i] = (int32_t)(z % (unsigned long long)nv);
    }
    // workspaces: labels in the level array, the log, the team job area
    int32_t *d = nullptr;
    const size_t extra = sizeof(int32_t) * ((size_t)nseeds * 2 + 8) + sizeof(MsCounters) + 64;
    FC_CUDA_TRY(cudaMallocAsync(&d, extra, stream));
    int32_t *d_seeds = d, *uf = d + nseeds, *d_out = d + 2 * nseeds;
    MsCounters *ctr = reinterpret_cast<MsCounters *>(
        (reinterpret_cast<uintptr_t>(d + 2 * nseeds + 8) + 15) & ~(uintptr_t)15);
    int rc = ensure_workspace(c, (size_t)nv);
    if (rc) {
        cudaFreeAsync(d, stream);
        return rc;
    }
    int levels = 0, found = 0;
    do {
        cudaError_t e;
        if ((e = cudaMemsetAsync(c->levels, 0xFF, sizeof(int32_t) * (size_t)nv, stream)) ||
            (e = cudaMemcpyAsync(d_seeds, hs.data(), sizeof(int32_t) * (size_t)nseeds,
                                 cudaMemcpyHostToDevice, stream)) ||
            (e = cudaEventRecord(c->ev0, stream))) {
            fc_set_last_cuda_error(e, "multi-seed set-up", __FILE__, __LINE__);
            rc = FC_ERR_CUDA;
            break;
        }
        k_ms_init<<<1, 1, 0, stream>>>(c->levels, c->log, uf, d_seeds, nseeds, ctr);
        MsArgs a;
        a.row_ptr = gp.fwd.row_ptr;
        a.col = gp.fwd.col;
        a.label = c->levels;
        a.log = c->log;
        a.uf = uf;
        a.ctr = ctr;
        a.jobs = reinterpret_cast<int4 *>(c->tjobs);
        a.jcap = c->tjobs_cap / 2;  // int4 jobs in the int2 area
        MsCounters h;
        int head = 0;
        const int grid = c->sm_count * 8;
        while (true) {
            k_ms_same<<<1, 1, 0, stream>>>(uf, ctr, d_out);
            int same = 0;
            if ((e = cudaMemcpyAsync(&h, ctr, sizeof(h), cudaMemcpyDeviceToHost, stream)) ||
                (e = cudaMemcpyAsync(&same, d_out, sizeof(int), cudaMemcpyDeviceToHost, stream)) ||
                (e = cudaStreamSynchronize(stream))) {
                fc_set_last_cuda_error(e, "multi-seed level", __FILE__, __LINE__);
                rc = FC_ERR_CUDA;
                break;
            }
            if (h.err) {
                set_error("multi-seed union-find ran past its bound");
                rc = FC_ERR_TIMEOUT;
                break;
            }
            if (same) {
                found = 1;
                break;
            }
            if (h.tail == head) break;  // growth over: not connected
            a.head = head;
            a.tail = h.tail;
            head = h.tail;
            if ((e = cudaMemsetAsync(&ctr->njobs, 0, 2 * sizeof(int), stream))) {
                fc_set_last_cuda_error(e, "multi-seed level", __FILE__, __LINE__);
                rc = FC_ERR_CUDA;
                break;
            }
            int g = (a.tail - a.head + MS_BLOCK - 1) / MS_BLOCK;
            k_ms_step<<<g < grid ? g : grid, MS_BLOCK, 0, stream>>>(a);
            k_ms_jobs<<<grid, MS_BLOCK, 0, stream>>>(a);
            if ((e = cudaGetLastError())) {
                fc_set_last_cuda_error(e, "multi-seed kernels", __FILE__, __LINE__);
                rc = FC_ERR_CUDA;
                break;
            }
            ++levels;
        }
        if (rc) break;
        cudaEventRecord(c->ev1, stream);
        cudaEventSynchronize(c->ev1);
        *connected = found;
        if (st) {
            std::memset(st, 0, sizeof(*st));
            st->edges_inspected = (int64_t)h.inspected;
            st->visited = h.tail;
            st->steps = levels;
            st->launches = 2 * levels + 1;
            float ms = 0;
            cudaEventElapsedTime(&ms, c->ev0, c->ev1);
            st->gpu_ms = ms;
        }
    } while (0);
    cudaFreeAsync(d, stream);
    cudaStreamSynchronize(stream);
    return rc;
}

}  // namespace fc
