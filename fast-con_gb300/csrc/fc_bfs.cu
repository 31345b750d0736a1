// fc_bfs.cu -- plain level-synchronous BFS (full level array from one source).
//
// The reference's level BFS (cudaBFS4K, K/src/device/BFS_WorkEfficient.cu:
// 81-118, with the persistent dispatch BFSDispath + GlobalSync,
// K/.../BFS_WE_KernelDispatch.cu:17-38) expands every frontier vertex's whole
// row each level and records dist[v] = level + 1 at the first visit.  This
// engine does the same top-down expansion, for the whole level array, in one
// cooperative launch with a bounded grid barrier per level; it differs in
// where the visited test is answered:
//
// * Visited bitmap.  One bit per vertex (2 MB for 2^24 vertices) holds
//   "visited"; a neighbour is probed in the bitmap and claimed with one
//   atomicOr on its word, whose returned word says whether this thread set
//   the bit.  The bitmap stays in L2 for the whole search, and a set bit
//   never clears during a search, so the probe may be served by the SM's L1
//   (ld.global.ca): a stale line can only say "not visited" for a visited
//   vertex, and then the atomicOr answers.  The level word of a vertex is
//   written once, by the thread that claimed it, and never probed.
// * Degree-ordered layout.  On graphs with skewed degrees most adjacency
//   entries of a big level point at a few hub vertices.  The engine keeps,
//   per graph, a copy of the CSR whose vertices are renumbered by descending
//   degree (built once, on the first call), so the hubs' visited bits share a
//   few dozen KB of the bitmap that stay in every SM's L1; on R-MAT 24 the
//   top 2^18 vertices receive ~85% of the entries of the largest level.  The
//   levels are mapped back to the caller's numbering in the output pass.
//   Levels do not depend on the numbering.
//
// Work per level: the frontier is the level's range of the visit queue; it is
// cut into tiles of frontier vertices sized by their degree sum and expanded
// by load-balanced search (fc_step.cuh), rows longer than TEAM_SPLIT_E
// entries being cut into row jobs that the whole grid walks after the tiles.
#include <algorithm>
#include <cstring>
#include <vector>

#include "fc_engine.h"
#include "fc_ingest.h"
#include "fc_sched.cuh"

namespace fc {

// ---------------------------------------------------------------------------
// degree-ordered copy of a graph's forward CSR
// ---------------------------------------------------------------------------
struct BfsLayout {
    int32_t nv = 0;
    long long ne = 0;
    int32_t *row_ptr = nullptr;  // renumbered CSR (rows in descending degree class)
    int32_t *col = nullptr;
    int32_t *new_id = nullptr;   // caller's id -> renumbered id
};

constexpr int LAYOUT_BUCKETS = 256;

// Degree class, descending: 8 classes per octave of the degree (the leading
// bit and the three below it), degree-0 vertices last.
__device__ __forceinline__ int degree_bucket(int d)
{
    if (d <= 0) return LAYOUT_BUCKETS - 1;
    const int e = 31 - __clz(d);
    const int m = e >= 3 ? (d >> (e - 3)) & 7 : (d << (3 - e)) & 7;
    return LAYOUT_BUCKETS - 2 - (e * 8 + m);  // e <= 30: at least 2
}

__global__ void k_layout_buckets(const int32_t *row_ptr, int nv, uint8_t *bucket,
                                 unsigned *counts)
{
    __shared__ unsigned h[LAYOUT_BUCKETS];
    for (int i = threadIdx.x; i < LAYOUT_BUCKETS; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < nv;
         v += (long long)gridDim.x * blockDim.x) {
        const int b = degree_bucket(row_ptr[v + 1] - row_ptr[v]);
        bucket[v] = (uint8_t)b;
        atomicAdd(&h[b], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < LAYOUT_BUCKETS; i += blockDim.x)
        if (h[i]) atomicAdd(&counts[i], h[i]);
}

// Block b lists the vertices of bucket b in increasing id order (a stable
// counting sort: the renumbering is deterministic).  Keys are read 16 per
// thread per round as one 16-byte load (the bucket array is padded to a
// multiple of 16 bytes; entries past nv are skipped).
constexpr int LAYOUT_T = 256;
__global__ void __launch_bounds__(LAYOUT_T) k_layout_assign(const uint8_t *bucket, int nv,
                                                            const unsigned *start,
                                                            const unsigned *counts,
                                                            int32_t *new_id, int32_t *old_id)
{
    const int b = blockIdx.x;
    if (counts[b] == 0) return;
    __shared__ int warp_tot[LAYOUT_T / 32];
    __shared__ int total;
    int base = (int)start[b];
    const uint4 *keys = reinterpret_cast<const uint4 *>(bucket);
    const long long nchunks = ((long long)nv + 15) / 16;
    for (long long c0 = 0; c0 < nchunks; c0 += LAYOUT_T) {
        const long long c = c0 + threadIdx.x;
        uint4 k4 = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
        if (c < nchunks) k4 = keys[c];
        const unsigned w[4] = {k4.x, k4.y, k4.z, k4.w};
        unsigned mask = 0;  // bit j: vertex 16c + j is in bucket b
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const long long v = c * 16 + j;
            if ((int)((w[j >> 2] >> ((j & 3) * 8)) & 0xFF) == b && v < nv) mask |= 1u << j;
        }
        const int cnt = __popc(mask);
        const int incl = block_inclusive_scan<LAYOUT_T>(cnt, warp_tot, &total);
        int pos = base + incl - cnt;
        while (mask) {
            const int j = __ffs(mask) - 1;
            mask &= mask - 1;
            const int v = (int)(c * 16 + j);
            new_id[v] = pos;
            old_id[pos] = v;
            ++pos;
        }
        base += total;
        __syncthreads();  // total is rewritten by the next round's scan
    }
}

__global__ void k_layout_degrees(const int32_t *row_ptr, const int32_t *old_id, int nv,
                                 int32_t *deg2)
{
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < nv;
         r += (long long)gridDim.x * blockDim.x) {
        const int v = old_id[r];
        deg2[r] = row_ptr[v + 1] - row_ptr[v];
    }
}

__global__ void k_layout_rowptr(const long long *off, int nv, int32_t *row_ptr2)
{
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r <= nv;
         r += (long long)gridDim.x * blockDim.x)
        row_ptr2[r] = (int32_t)off[r];
}

// One warp per renumbered row: copy the caller's row, renaming every entry.
__global__ void k_layout_cols(const int32_t *row_ptr, const int32_t *col, const int32_t *old_id,
                              const int32_t *new_id, const int32_t *row_ptr2, int nv, int32_t *col2)
{
    const int lane = threadIdx.x & 31;
    const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long r = w0; r < nv; r += nw) {
        const int v = old_id[r];
        const int b = row_ptr[v], e = row_ptr[v + 1];
        const int o = row_ptr2[r];
        for (int k = b + lane; k < e; k += 32) col2[o + (k - b)] = new_id[col[k]];
    }
}

void bfs_layout_free(BfsLayout *L)
{
    if (!L) return;
    cudaFree(L->row_ptr);
    cudaFree(L->col);
    cudaFree(L->new_id);
    delete L;
}

// Builds the layout into *out.  only_if_skewed: when no vertex has a degree of
// at least LAYOUT_HUB_DEGREE the graph has no hubs to pack, and *out is left
// NULL (FC_OK).
constexpr int LAYOUT_HUB_DEGREE = 256;
int bfs_layout_build(const GraphPairH &gp, BfsLayout **out, cudaStream_t st, int only_if_skewed)
{
    *out = nullptr;
    const int nv = gp.fwd.nv;
    const long long ne = gp.fwd.ne;
    BfsLayout *L = new BfsLayout();
    L->nv = nv;
    L->ne = ne;
    uint8_t *bucket = nullptr;
    unsigned *cnt = nullptr;  // [0, 256) counts, [256, 512) starts
    int32_t *old_id = nullptr, *deg2 = nullptr;
    long long *off = nullptr;
    int rc = FC_OK;
    auto fail = [&](cudaError_t e, const char *what) {
        fc_set_last_cuda_error(e, what, __FILE__, __LINE__);
        rc = e == cudaErrorMemoryAllocation ? FC_ERR_OOM : FC_ERR_CUDA;
    };
    const size_t kbytes = ((size_t)nv + 15) / 16 * 16;
    cudaError_t e;
    if ((e = cudaMalloc(&bucket, kbytes)) != cudaSuccess ||
        (e = cudaMalloc(&cnt, 2 * LAYOUT_BUCKETS * sizeof(unsigned))) != cudaSuccess ||
        (e = cudaMalloc(&old_id, sizeof(int32_t) * (size_t)nv)) != cudaSuccess ||
        (e = cudaMalloc(&deg2, sizeof(int32_t) * (size_t)nv)) != cudaSuccess ||
        (e = cudaMalloc(&off, sizeof(long long) * ((size_t)nv + 1))) != cudaSuccess ||
        (e = cudaMalloc(&L->new_id, sizeof(int32_t) * (size_t)nv)) != cudaSuccess ||
        (e = cudaMalloc(&L->row_ptr, sizeof(int32_t) * ((size_t)nv + 1))) != cudaSuccess ||
        (e = cudaMalloc(&L->col, sizeof(int32_t) * (size_t)std::max(1LL, ne))) != cudaSuccess) {
        fail(e, "cudaMalloc (degree-ordered layout)");
    }
    if (rc == FC_OK) {
        cudaMemsetAsync(bucket, 0xFF, kbytes, st);
        cudaMemsetAsync(cnt, 0, LAYOUT_BUCKETS * sizeof(unsigned), st);
        const int grid = (int)std::min<long long>(4096, ((long long)nv + 255) / 256);
        k_layout_buckets<<<grid, 256, 0, st>>>(gp.fwd.row_ptr, nv, bucket, cnt);
        unsigned h[LAYOUT_BUCKETS], hs[LAYOUT_BUCKETS];
        if ((e = cudaMemcpyAsync(h, cnt, sizeof(h), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess) {
            fail(e, "degree classes");
        } else {
            unsigned run = 0, hubs = 0;
            for (int i = 0; i < LAYOUT_BUCKETS; ++i) {
                hs[i] = run;
                run += h[i];
            }
            // buckets are descending: those at or below the class of
            // LAYOUT_HUB_DEGREE hold its degree or more
            static_assert(LAYOUT_HUB_DEGREE == 1 << 8, "hub class below assumes 2^8");
            for (int i = 0; i <= LAYOUT_BUCKETS - 2 - 8 * 8; ++i) hubs += h[i];
            if (only_if_skewed && hubs == 0) rc = -1;  // nothing to gain: keep the numbering
            if (rc == FC_OK &&
                (e = cudaMemcpyAsync(cnt + LAYOUT_BUCKETS, hs, sizeof(hs), cudaMemcpyHostToDevice,
                                     st)) != cudaSuccess)
                fail(e, "bucket starts");
        }
    }
    if (rc == FC_OK) {
        k_layout_assign<<<LAYOUT_BUCKETS, LAYOUT_T, 0, st>>>(bucket, nv, cnt + LAYOUT_BUCKETS, cnt,
                                                           L->new_id, old_id);
        const int grid = (int)std::min<long long>(4096, ((long long)nv + 255) / 256);
        k_layout_degrees<<<grid, 256, 0, st>>>(gp.fwd.row_ptr, old_id, nv, deg2);
        rc = scan_i32(deg2, nv, off, st);
    }
    if (rc == FC_OK) {
        const int grid = (int)std::min<long long>(4096, ((long long)nv + 256) / 256);
        k_layout_rowptr<<<grid, 256, 0, st>>>(off, nv, L->row_ptr);
        const int wgrid = (int)std::min<long long>(8192, ((long long)nv * 32 + 255) / 256);
        k_layout_cols<<<wgrid, 256, 0, st>>>(gp.fwd.row_ptr, gp.fwd.col, old_id, L->new_id,
                                             L->row_ptr, nv, L->col);
        if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaStreamSynchronize(st)) != cudaSuccess)
            fail(e, "degree-ordered layout kernels");
    }
    cudaFree(bucket);
    cudaFree(cnt);
    cudaFree(old_id);
    cudaFree(deg2);
    cudaFree(off);
    if (rc != FC_OK) {
        bfs_layout_free(L);
        return rc < 0 ? FC_OK : rc;  // -1: no hubs, numbering kept
    }
    *out = L;
    return FC_OK;
}

// ---------------------------------------------------------------------------
// the search
// ---------------------------------------------------------------------------
struct BfsSnap {  // counters as they stood at a level's last barrier
    int tail;
    int nok[2];
    int pad;
    unsigned long long deg;
    unsigned long long reads;
};

// Per-level record of the last search (the first BFS_TRACE_LEVELS levels):
// start time from %globaltimer, frontier end in the queue, entries read before
// the level.  The reference times its levels under DBG_TIME (START_TIMER /
// STOP_TIMER, S/include/header.h).
constexpr int BFS_TRACE_LEVELS = 256;
struct BfsTrace {
    unsigned long long t0;
    unsigned long long ns[BFS_TRACE_LEVELS + 1];
    long long tail[BFS_TRACE_LEVELS + 1];
    unsigned long long reads[BFS_TRACE_LEVELS + 1];
};

struct BfsCounters {
    int tail;   // vertices queued (= reached)
    int err;
    int bar[2];
    int njobs[2];
    int nok[2];
    unsigned long long deg;    // degree sum of the queued vertices
    unsigned long long reads;  // adjacency entries read
    unsigned long long root_deg;
    int levels;                // levels expanded
    int pad;
    BfsSnap snap[2];           // by barrier generation parity
    BfsTrace trace;
};

// Every CTA reads the level's counters from the barrier's snapshot: the
// fastest CTAs are already claiming the next level's vertices.
struct SnapBfs {
    BfsCounters *c;
    __device__ __forceinline__ void operator()(int p) const
    {
        BfsSnap &s = c->snap[p];
        s.tail = ld_cg(&c->tail);
        s.nok[0] = ld_cg(&c->nok[0]);
        s.nok[1] = ld_cg(&c->nok[1]);
        s.deg = ld_cg_u64(&c->deg);
        s.reads = ld_cg_u64(&c->reads);
    }
};

// Claim through the visited bitmap; the winner writes the level.
struct VisitBitmap {
    unsigned *bm;
    int32_t *lev;
    int next_level;
    __device__ __forceinline__ int probe(int v) const { return (int)__ldca(bm + (v >> 5)); }
    __device__ __forceinline__ int attempt(int v, int p) const
    {
        const unsigned bit = 1u << (v & 31);
        if ((unsigned)p & bit) return p;
        return (int)atomicOr(bm + (v >> 5), bit);
    }
    __device__ __forceinline__ int resolve(int v, int r) const
    {
        if ((unsigned)r & (1u << (v & 31))) return -1;
        lev[v] = next_level;
        return v;
    }
    __device__ __forceinline__ int visit(int v) const { return resolve(v, attempt(v, probe(v))); }
};

struct BfsArgs {
    const int32_t *row_ptr;
    const int32_t *col;
    int nv;
    unsigned *bm;
    int32_t *lev;
    int32_t *queue;
    BfsCounters *ctr;
    int2 *jobs;
    int jcap;
};

constexpr int BFS_T = 256;
constexpr int BFS_MIN_CTAS = 4;  // resident CTAs per SM the register budget allows

__global__ void k_bfs_root(BfsArgs a, int s)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    BfsCounters *c = a.ctr;
    a.bm[s >> 5] |= 1u << (s & 31);
    a.lev[s] = 0;
    a.queue[0] = s;
    c->tail = 1;
    c->err = 0;
    c->njobs[0] = c->njobs[1] = 0;
    c->nok[0] = c->nok[1] = 0;
    c->deg = (unsigned long long)(a.row_ptr[s + 1] - a.row_ptr[s]);
    c->root_deg = c->deg;
    c->reads = 0;
    c->levels = 0;
    c->bar[0] = 0;  // arrivals (a launch that gave up at a barrier may have left some)
}

template <int T>
__global__ void __launch_bounds__(T, BFS_MIN_CTAS) k_bfs_plain(BfsArgs a)
{
    __shared__ SmemTopDown<T> sm;
    __shared__ int s_nj;
    BfsCounters *c = a.ctr;
    int head = 0, tail = 1, level = 0;
    unsigned long long dprev = 0, dcur = ld_cg_u64(&c->root_deg);
    const bool tracer = blockIdx.x == 0 && threadIdx.x == 0;
    if (tracer) {
        c->trace.t0 = global_timer_ns();
        c->trace.ns[0] = 0;
        c->trace.tail[0] = 1;
        c->trace.reads[0] = 0;
    }
    while (tail > head) {
        const int F = tail - head;
        const int par = level & 1;
        // the other parity's job counters were last read before the previous
        // level's final barrier: clearing them cannot race
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            c->njobs[par ^ 1] = 0;
            c->nok[par ^ 1] = 0;
        }
        const VisitBitmap vis{a.bm, a.lev, level + 1};
        const AppendTarget app{a.queue, a.nv, 0, &c->tail, &c->deg, a.row_ptr, nullptr, &c->reads};
        topdown_step<T>(a.row_ptr, a.col, a.queue + head, F, blockIdx.x, gridDim.x, vis, app, sm,
                        nullptr, TeamSink{a.jobs, a.jcap, &c->njobs[par], &c->nok[par]},
                        team_tile_v<T>(F, (long long)(dcur - dprev)));
        int g = grid_barrier_snap(c->bar, &c->err, gridDim.x, SnapBfs{c});
        if (g < 0) return;
        if (threadIdx.x == 0) s_nj = min(ld_cg(&c->snap[g & 1].nok[par]), a.jcap);
        __syncthreads();
        if (s_nj > 0) {  // the same value in every CTA: a uniform barrier
            team_jobs<T>(a.col, a.jobs, s_nj, blockIdx.x, gridDim.x, vis, app, sm, nullptr);
            g = grid_barrier_snap(c->bar, &c->err, gridDim.x, SnapBfs{c});
            if (g < 0) return;
        }
        head = tail;
        tail = ld_cg(&c->snap[g & 1].tail);
        dprev = dcur;
        dcur = ld_cg_u64(&c->snap[g & 1].deg);
        ++level;
        if (tracer && level <= BFS_TRACE_LEVELS) {
            c->trace.ns[level] = global_timer_ns() - c->trace.t0;
            c->trace.tail[level] = tail;
            c->trace.reads[level] = ld_cg_u64(&c->snap[g & 1].reads);
        }
    }
    if (tracer) c->levels = level;
}

// Levels in the caller's numbering: -1 where the bitmap bit is clear.
__global__ void k_bfs_out(const unsigned *bm, const int32_t *lev, const int32_t *new_id, int nv,
                          int32_t *out)
{
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < nv;
         v += (long long)gridDim.x * blockDim.x) {
        const int x = new_id ? __ldg(new_id + v) : (int)v;
        const bool hit = (__ldg(bm + (x >> 5)) >> (x & 31)) & 1u;
        out[v] = hit ? __ldg(lev + x) : -1;
    }
}

static int ensure_bfs_ws(DevCtx *c, size_t nv)
{
    if (!c->bfs_ctr) {
        FC_CUDA_TRY(cudaMalloc(&c->bfs_ctr, sizeof(BfsCounters)));
        FC_CUDA_TRY(cudaMemset(c->bfs_ctr, 0, sizeof(BfsCounters)));
        FC_CUDA_TRY(cudaMallocHost(&c->h_bfs_ctr, sizeof(BfsCounters)));
        // 2^20 jobs of TEAM_SPLIT_E entries: any level of a graph of up to 2^32 entries
        FC_CUDA_TRY(cudaMalloc(&c->bfs_jobs, sizeof(int2) << 20));
        c->bfs_jcap = 1 << 20;
    }
    if (c->bfs_nv >= nv && c->bfs_bm) return FC_OK;
    cudaFree(c->bfs_bm);
    cudaFree(c->bfs_lev);
    cudaFree(c->bfs_q);
    cudaFree(c->bfs_out);
    c->bfs_bm = nullptr;
    c->bfs_lev = c->bfs_q = c->bfs_out = nullptr;
    c->bfs_nv = 0;
    const size_t words = (nv + 1023) / 1024 * 32;  // whole 128-byte lines
    FC_CUDA_TRY(cudaMalloc(&c->bfs_bm, words * sizeof(unsigned)));
    FC_CUDA_TRY(cudaMalloc(&c->bfs_lev, nv * sizeof(int32_t)));
    FC_CUDA_TRY(cudaMalloc(&c->bfs_q, nv * sizeof(int32_t)));
    FC_CUDA_TRY(cudaMalloc(&c->bfs_out, nv * sizeof(int32_t)));
    FC_CUDA_TRY(cudaDeviceSynchronize());
    c->bfs_nv = nv;
    return FC_OK;
}

static int bfs_grid(DevCtx *c)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bfs_plain<BFS_T>, BFS_T, 0) !=
            cudaSuccess ||
        per_sm < 1)
        return 0;
    return per_sm * c->sm_count;
}

int engine_bfs_plain(DevCtx *c, const GraphPairH &gp, const BfsLayout *L, int32_t s,
                     int32_t *h_levels, fc_stats *st, cudaStream_t stream)
{
    const int nv = gp.fwd.nv;
    int rc = ensure_bfs_ws(c, (size_t)nv);
    if (rc) return rc;
    if (!c->coop) {
        set_error("cooperative launch not supported on this device");
        return FC_ERR_UNSUPPORTED;
    }
    const int grid = bfs_grid(c);
    if (grid < 1) {
        set_error("k_bfs_plain cannot be resident");
        return FC_ERR_CUDA;
    }
    BfsArgs a;
    a.row_ptr = L ? L->row_ptr : gp.fwd.row_ptr;
    a.col = L ? L->col : gp.fwd.col;
    a.nv = nv;
    a.bm = c->bfs_bm;
    a.lev = c->bfs_lev;
    a.queue = c->bfs_q;
    a.ctr = (BfsCounters *)c->bfs_ctr;
    a.jobs = c->bfs_jobs;
    a.jcap = c->bfs_jcap;
    // the root in the search's numbering (one element read back)
    int32_t root = s;
    if (L)
        FC_CUDA_TRY(cudaMemcpyAsync(&root, L->new_id + s, sizeof(int32_t), cudaMemcpyDeviceToHost,
                                    stream));
    FC_CUDA_TRY(cudaStreamSynchronize(stream));
    FC_CUDA_TRY(cudaEventRecord(c->ev0, stream));
    FC_CUDA_TRY(cudaMemsetAsync(a.bm, 0, ((size_t)nv + 1023) / 1024 * 128, stream));
    k_bfs_root<<<1, 32, 0, stream>>>(a, root);
    FC_CUDA_TRY(cudaGetLastError());
    void *args[] = {&a};
    FC_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)k_bfs_plain<BFS_T>, dim3(grid),
                                            dim3(BFS_T), args, 0, stream));
    const int ogrid = (int)std::min<long long>(8 * (long long)c->sm_count, ((long long)nv + 255) / 256);
    k_bfs_out<<<ogrid, 256, 0, stream>>>(a.bm, a.lev, L ? L->new_id : nullptr, nv, c->bfs_out);
    FC_CUDA_TRY(cudaGetLastError());
    FC_CUDA_TRY(cudaEventRecord(c->ev1, stream));
    FC_CUDA_TRY(cudaMemcpyAsync(c->h_bfs_ctr, a.ctr, sizeof(BfsCounters), cudaMemcpyDeviceToHost,
                                stream));
    if (h_levels)
        FC_CUDA_TRY(cudaMemcpyAsync(h_levels, c->bfs_out, sizeof(int32_t) * (size_t)nv,
                                    cudaMemcpyDeviceToHost, stream));
    FC_CUDA_TRY(cudaStreamSynchronize(stream));
    const BfsCounters *hc = (const BfsCounters *)c->h_bfs_ctr;
    if (hc->err) {
        set_error("k_bfs_plain: a grid barrier wait expired");
        return FC_ERR_TIMEOUT;
    }
    if (st) {
        std::memset(st, 0, sizeof(*st));
        const long long reached = hc->tail;
        st->edges_inspected = (int64_t)hc->reads;
        st->visited = reached;
        st->steps = hc->levels;
        // 12 per frontier vertex + 8 per entry read + 8 per claimed vertex
        st->alg_bytes = (int64_t)(12 * reached + 8 * (long long)hc->reads + 8 * (reached - 1));
        st->launches = 4;
        st->visited_adjacency = (int64_t)hc->deg;
        float ms = 0;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        st->gpu_ms = ms;
    }
    return FC_OK;
}

int engine_bfs_trace(DevCtx *c, int32_t *nlevels, int64_t *level_ns, int64_t *frontier,
                     int64_t *entries, int32_t cap)
{
    if (!c->h_bfs_ctr) {
        *nlevels = 0;
        return FC_OK;
    }
    const BfsCounters *hc = (const BfsCounters *)c->h_bfs_ctr;
    const int n = std::min(hc->levels, BFS_TRACE_LEVELS);
    *nlevels = hc->levels;
    for (int l = 0; l < n && l < cap; ++l) {
        // level l expands queue [tail[l-1], tail[l]) -- the vertices at distance l
        const long long b = l == 0 ? 0 : hc->trace.tail[l - 1], e = hc->trace.tail[l];
        if (level_ns) level_ns[l] = (int64_t)(hc->trace.ns[l + 1] - hc->trace.ns[l]);
        if (frontier) frontier[l] = e - b;
        if (entries) entries[l] = (int64_t)(hc->trace.reads[l + 1] - hc->trace.reads[l]);
    }
    return FC_OK;
}

}  // namespace fc
