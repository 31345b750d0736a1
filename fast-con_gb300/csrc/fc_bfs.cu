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
//   degree (built once, by the first search that uses it; s-t batches and
//   the other BFS engines use the same copy), so the hubs' visited bits
//   share a few dozen KB of the bitmap that stay in every SM's L1; on R-MAT
//   24 the top 2^18 vertices receive ~85% of the entries of the largest
//   level.  Each row of the copy is sorted by the new ids (its hubs first).
//   The levels are mapped back to the caller's numbering in the output pass.
//   Levels do not depend on the numbering.
//
// Work per level, with no CTA barrier: each warp takes work from the level's
// queues on its own (its first item by its index, later ones from an atomic
// counter).  Long rows come as pieces of at most BFS_PIECE entries, walked
// with 16-byte column loads; short rows come 32 * V to a chunk, laid end to
// end by a warp prefix sum and read by load-balanced search within the warp
// (after Merrill, Garland & Grimshaw, PPoPP 2012).  Claims gather in a
// per-warp shared-memory buffer and reach the next level's queues with one
// reservation per buffer.
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
    int32_t *row_ptr = nullptr;  // renumbered CSR (rows in descending degree class,
                                 // each row's entries ascending: hubs first)
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

void bfs_layout_graph(const BfsLayout *L, DGraphH *out)
{
    out->row_ptr = L->row_ptr;
    out->col = L->col;
    out->nv = L->nv;
    out->pad_ = 0;
    out->ne = L->ne;
    out->remap = L->new_id;
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
    // every row in ascending new id, i.e. its highest-degree neighbours first:
    // an s-t step that meets the other side mostly meets it at a hub, and a
    // bottom-up check finds a frontier parent sooner, so both stop earlier
    // (R-MAT 24, 1,024 queries: 16% fewer entries read, batch 0.277 -> 0.241 ms)
    if (rc == FC_OK) rc = sort_rows_i32(off, nv, ne, L->col, st);
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
// Frontier queues, by the parity of the level they hold.  A claimed vertex
// goes, with its row range, to the short queue (1..BFS_MED entries) or, cut
// into pieces of at most BFS_PIECE entries, to the piece queue; vertices
// without neighbours are not queued.  A level reads its queues with no row
// lookup: the claimer already read the row range.
constexpr int BFS_T = 256;
constexpr int BFS_MED = 256;      // longer rows are walked in pieces
constexpr int BFS_PIECE = 2048;   // entries per piece
constexpr int BFS_VMAX = 4;       // short-queue vertices per lane in one chunk
constexpr int BFS_KMAX = 16;      // entries per lane and round, at most
constexpr int BFS_WLOG = 32 * BFS_KMAX;  // claims buffered per warp (one round's worth)

struct BfsSnap {  // the next frontier's counters as they stood at the level's last barrier
    unsigned long long qc;   // (short vertices << 32) | pieces
    unsigned long long qds;  // adjacency entries of the short vertices
    unsigned long long qdl;  // (other claimed vertices << 40) | entries of the long ones
    unsigned long long pad;
};

// Per-level record of the last search (the first BFS_TRACE_LEVELS levels):
// start time from %globaltimer, vertices and adjacency entries of the
// frontier.  The reference times its levels under DBG_TIME (START_TIMER /
// STOP_TIMER, S/include/header.h).
constexpr int BFS_TRACE_LEVELS = 256;
struct BfsTrace {
    unsigned long long t0;
    unsigned long long ns[BFS_TRACE_LEVELS + 1];
    long long frontier[BFS_TRACE_LEVELS + 1];
    unsigned long long entries[BFS_TRACE_LEVELS + 1];
};

// Counters in separate 128-byte lines: the flush reservations, the dynamic
// fetches and the barrier words (polled by every waiting CTA) do not share
// a line, so waiting CTAs do not queue behind the working ones' atomics.
struct alignas(128) BfsQueueCtr {
    unsigned long long qc[2];     // live counters of the queue pair being filled, by parity
    unsigned long long qds[2];
    unsigned long long qdl[2];
};
struct alignas(128) BfsFetchCtr {
    int fetch_s[2], fetch_p[2];   // dynamic batches taken, by level parity
};
struct alignas(128) BfsBarrier {
    int bar[2];
    int err;
};

struct BfsCounters {
    BfsQueueCtr q;
    BfsFetchCtr f;
    BfsBarrier b;
    int levels;                   // levels expanded
    int pad;
    unsigned long long init_qc, init_qds, init_qdl;  // the root's queues
    long long overflow;           // queue writes refused (never, by construction)
    unsigned long long reached;   // vertices at some distance (totals, kept by the tracer)
    unsigned long long entries;   // adjacency entries of those vertices = entries read
    BfsSnap snap[2];              // by barrier generation parity
    BfsTrace trace;
};

struct SnapBfs {
    BfsCounters *c;
    int np;  // parity of the queues the level filled
    __device__ __forceinline__ void operator()(int p) const
    {
        BfsSnap &s = c->snap[p];
        s.qc = ld_cg_u64(&c->q.qc[np]);
        s.qds = ld_cg_u64(&c->q.qds[np]);
        s.qdl = ld_cg_u64(&c->q.qdl[np]);
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
    int2 *sq[2];       // short queues
    int2 *pq[2];       // piece queues
    long long scap, pcap;
    BfsCounters *ctr;
};

struct BfsWarpSmem {
    int off[32 * BFS_VMAX + 1];  // chunk rows laid end to end
    int rbs[32 * BFS_VMAX];      // and their first entries
    int buf[BFS_WLOG];           // claimed vertices not yet queued
    int cnt;
};

// Move the warp's buffered claims into the next frontier's queues: one
// reservation per counter for the whole buffer.  Lane l owns buffer entries
// l, l + 32, ...; their row ranges are read eight at a time (loads in
// flight together) to count, then read again -- from the cache -- to write.
constexpr int BFS_FLUSH_ILP = 8;
__device__ __noinline__ void bfs_flush(const BfsArgs &a, BfsWarpSmem &w, int np)
{
    const int lane = (int)lane_id();
    const int n = w.cnt;
    if (n == 0) return;
    int ns = 0, npc = 0, nother = 0;
    long long dsh = 0, dlo = 0;
    for (int i0 = 0; i0 < n; i0 += 32 * BFS_FLUSH_ILP) {
        int v[BFS_FLUSH_ILP], d[BFS_FLUSH_ILP];
#pragma unroll
        for (int j = 0; j < BFS_FLUSH_ILP; ++j) {
            const int i = i0 + j * 32 + lane;
            v[j] = i < n ? w.buf[i] : -1;
        }
#pragma unroll
        for (int j = 0; j < BFS_FLUSH_ILP; ++j)
            d[j] = v[j] >= 0 ? __ldg(a.row_ptr + v[j] + 1) - __ldg(a.row_ptr + v[j]) : -1;
#pragma unroll
        for (int j = 0; j < BFS_FLUSH_ILP; ++j) {
            if (d[j] < 0) continue;
            if (d[j] > 0 && d[j] <= BFS_MED) {
                ++ns;
                dsh += d[j];
            } else {
                ++nother;
                if (d[j] > 0) {
                    npc += (d[j] + BFS_PIECE - 1) / BFS_PIECE;
                    dlo += d[j];
                }
            }
        }
    }
    const int s_incl = warp_inclusive_scan(ns), p_incl = warp_inclusive_scan(npc);
    const int s_tot = __shfl_sync(0xffffffffu, s_incl, 31);
    const int p_tot = __shfl_sync(0xffffffffu, p_incl, 31);
    dsh = warp_sum_ll(dsh);
    dlo = warp_sum_ll(dlo);
    nother = warp_sum_i(nother);
    unsigned long long base = 0;
    BfsCounters *c = a.ctr;
    if (lane == 0) {
        base = atomicAdd(&c->q.qc[np], ((unsigned long long)s_tot << 32) | (unsigned)p_tot);
        if (dsh) atomicAdd(&c->q.qds[np], (unsigned long long)dsh);
        if (nother)
            atomicAdd(&c->q.qdl[np], ((unsigned long long)nother << 40) | (unsigned long long)dlo);
    }
    base = __shfl_sync(0xffffffffu, base, 0);
    long long sb = (long long)(base >> 32) + s_incl - ns;
    long long pb = (long long)(base & 0xffffffffu) + p_incl - npc;
    int2 *sq = a.sq[np], *pq = a.pq[np];
    int refused = 0;
    for (int i0 = 0; i0 < n; i0 += 32 * BFS_FLUSH_ILP) {
        int v[BFS_FLUSH_ILP], b[BFS_FLUSH_ILP], e[BFS_FLUSH_ILP];
#pragma unroll
        for (int j = 0; j < BFS_FLUSH_ILP; ++j) {
            const int i = i0 + j * 32 + lane;
            v[j] = i < n ? w.buf[i] : -1;
        }
#pragma unroll
        for (int j = 0; j < BFS_FLUSH_ILP; ++j) {
            b[j] = v[j] >= 0 ? __ldg(a.row_ptr + v[j]) : 0;
            e[j] = v[j] >= 0 ? __ldg(a.row_ptr + v[j] + 1) : 0;
        }
#pragma unroll
        for (int j = 0; j < BFS_FLUSH_ILP; ++j) {
            const int d = e[j] - b[j];
            if (d > 0 && d <= BFS_MED) {
                if (sb < a.scap) sq[sb] = make_int2(b[j], e[j]);
                else ++refused;
                ++sb;
            } else if (d > 0) {
                for (int x = b[j]; x < e[j]; x += BFS_PIECE) {
                    if (pb < a.pcap) pq[pb] = make_int2(x, min(e[j], x + BFS_PIECE));
                    else ++refused;
                    ++pb;
                }
            }
        }
    }
    refused = warp_sum_i(refused);
    if (lane == 0 && refused) atomicAdd((unsigned long long *)&c->overflow, (unsigned long long)refused);
    __syncwarp();
    if (lane == 0) w.cnt = 0;
    __syncwarp();
}

// Buffer the claims of one round (c[k] = claimed vertex or -1); the buffer
// holds one full round, so it is flushed first when the round would not fit.
template <int K>
__device__ __forceinline__ void bfs_append(const BfsArgs &a, BfsWarpSmem &w, const int (&c)[K],
                                           int np)
{
    int cnt = 0;
#pragma unroll
    for (int k = 0; k < K; ++k) cnt += c[k] >= 0;
    if (!__any_sync(0xffffffffu, cnt > 0)) return;
    const int incl = warp_inclusive_scan(cnt);
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    int n0 = w.cnt;
    if (n0 + total > BFS_WLOG) {
        bfs_flush(a, w, np);
        n0 = 0;
    }
    int pos = n0 + incl - cnt;
#pragma unroll
    for (int k = 0; k < K; ++k)
        if (c[k] >= 0) w.buf[pos++] = c[k];
    __syncwarp();
    if (lane_id() == 0) w.cnt = n0 + total;
    __syncwarp();
}

// A piece of one long row: P 16-byte column loads per lane and round
// (128 P entries), the unaligned ends with scalar loads.
template <int P>
__device__ __noinline__ void bfs_piece(const BfsArgs &a, BfsWarpSmem &w, int2 pc,
                                       VisitBitmap vis, int np)
{
    const int lane = (int)lane_id();
    const int b = pc.x, e = pc.y;
    const int al = min((b + 3) & ~3, e);
    const int z = max(e & ~3, al);
    const int nhead = al - b, ntail = e - z;
    if (nhead + ntail > 0) {
        int c[1] = {-1};
        if (lane < nhead)
            c[0] = vis.visit(__ldg(a.col + b + lane));
        else if (lane < nhead + ntail)
            c[0] = vis.visit(__ldg(a.col + z + lane - nhead));
        bfs_append<1>(a, w, c, np);
    }
    const int4 *col4 = reinterpret_cast<const int4 *>(a.col);
    const int k_end = z >> 2;
    for (int k0 = al >> 2; k0 < k_end; k0 += P * 32) {
        int v[4 * P], c[4 * P];
#pragma unroll
        for (int h = 0; h < P; ++h) {
            const int k = k0 + h * 32 + lane;
            int4 x = make_int4(-1, -1, -1, -1);
            if (k < k_end) x = __ldg(col4 + k);
            v[4 * h + 0] = x.x;
            v[4 * h + 1] = x.y;
            v[4 * h + 2] = x.z;
            v[4 * h + 3] = x.w;
        }
        visit_k<4 * P>(vis, v, c);
        bfs_append<4 * P>(a, w, c, np);
    }
}

// A chunk of 32 * V short-queue vertices: their rows laid end to end in the
// warp's shared memory, K entries per lane and round, each entry's row found
// by binary search over the chunk's prefix (load-balanced search within one
// warp: no CTA barrier).
template <int V, int K>
__device__ __noinline__ void bfs_chunk(const BfsArgs &a, BfsWarpSmem &w, const int2 *sq, int Fs,
                                       int first, VisitBitmap vis, int np)
{
    const int lane = (int)lane_id();
    int2 r[V];
    int sum = 0;
#pragma unroll
    for (int v = 0; v < V; ++v) {
        const int i = first + lane * V + v;
        r[v] = i < Fs ? sq[i] : make_int2(0, 0);
        sum += r[v].y - r[v].x;
    }
    const int incl = warp_inclusive_scan(sum);
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    int run = incl - sum;
#pragma unroll
    for (int v = 0; v < V; ++v) {
        w.off[lane * V + v] = run;
        w.rbs[lane * V + v] = r[v].x;
        run += r[v].y - r[v].x;
    }
    __syncwarp();
    for (int base = 0; base < total; base += 32 * K) {
        int v[K], c[K];
#pragma unroll
        for (int j = 0; j < K; ++j) {
            const int e = base + j * 32 + lane;
            v[j] = -1;
            if (e < total) {
                int lo = 0;  // the last row starting at or before e
#pragma unroll
                for (int s = 16 * V; s > 0; s >>= 1)  // lo + s stays below 32 * V
                    if (w.off[lo + s] <= e) lo += s;
                v[j] = __ldg(a.col + w.rbs[lo] + (e - w.off[lo]));
            }
        }
        visit_k<K>(vis, v, c);
        bfs_append<K>(a, w, c, np);
    }
    __syncwarp();  // off / rbs are rewritten by the next chunk
}

__global__ void k_bfs_root(BfsArgs a, int s)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    BfsCounters *c = a.ctr;
    a.bm[s >> 5] |= 1u << (s & 31);
    a.lev[s] = 0;
    const int b = a.row_ptr[s], e = a.row_ptr[s + 1], d = e - b;
    unsigned long long ns = 0, np = 0, other = 1;
    if (d > 0 && d <= BFS_MED) {
        a.sq[0][0] = make_int2(b, e);
        ns = 1;
        other = 0;
    } else {
        for (int x = b; x < e; x += BFS_PIECE) a.pq[0][np++] = make_int2(x, min(e, x + BFS_PIECE));
    }
    c->init_qc = (ns << 32) | np;
    c->init_qds = ns ? (unsigned long long)d : 0;
    c->init_qdl = (other << 40) | (ns ? 0ull : (unsigned long long)d);
    for (int p = 0; p < 2; ++p) {
        c->q.qc[p] = c->q.qds[p] = c->q.qdl[p] = 0;
        c->f.fetch_s[p] = c->f.fetch_p[p] = 0;
    }
    c->b.err = 0;
    c->levels = 0;
    c->overflow = 0;
    c->reached = 0;
    c->entries = 0;
    c->b.bar[0] = 0;  // arrivals (a launch that gave up at a barrier may have left some)
}

// MINB resident CTAs per SM (the register budget) and K entries per lane and
// round go together: 4 x 8 (64 registers), 3 x 8 (80), 2 x 16 (128).  On
// R-MAT 24 the three measure within run-to-run noise of each other (1.5-1.9
// ms); more entries per round, a software-pipelined round (the next round's
// column loads issued before this round's probes) and a shared-memory copy
// of the hubs' bitmap words each measured no faster.
template <int T, int MINB, int K>
__global__ void __launch_bounds__(T, MINB) k_bfs_plain(BfsArgs args)
{
    __shared__ BfsWarpSmem wsm[T / 32];
    __shared__ BfsArgs a;  // the helpers read the arguments from shared memory
    if (threadIdx.x == 0) a = args;
    __syncthreads();
    BfsCounters *c = args.ctr;
    const int lane = (int)lane_id();
    BfsWarpSmem &w = wsm[threadIdx.x >> 5];
    if (lane == 0) w.cnt = 0;
    __syncwarp();
    const int gw = (int)((blockIdx.x * T + threadIdx.x) >> 5);
    const int nw = (int)(gridDim.x * (T / 32));
    unsigned long long qc = ld_cg_u64(&c->init_qc), qds = ld_cg_u64(&c->init_qds),
                       qdl = ld_cg_u64(&c->init_qdl);
    const bool tracer = blockIdx.x == 0 && threadIdx.x == 0;
    if (tracer) c->trace.t0 = global_timer_ns();
    int level = 0;
    while (true) {
        const int Fs = (int)(qc >> 32), Fp = (int)(qc & 0xffffffffu);
        const long long fr = (long long)Fs + (long long)(qdl >> 40);  // vertices at this distance
        if (tracer) {
            const unsigned long long en = qds + (qdl & ((1ull << 40) - 1));
            c->reached += (unsigned long long)fr;
            c->entries += en;
            if (level <= BFS_TRACE_LEVELS) {
                c->trace.ns[level] = global_timer_ns() - c->trace.t0;
                c->trace.frontier[level] = fr;
                c->trace.entries[level] = en;
            }
        }
        if (Fs == 0 && Fp == 0) {
            // a level of vertices without out-edges still counts as a level
            if (fr > 0) ++level;
            break;
        }
        const int p = level & 1, np = p ^ 1;
        // the live counters of parity p described this level's queues; every
        // CTA took them from the last barrier's snapshot, and the next level
        // refills them.  The other parity's fetch counters were last used a
        // level ago, before the last barrier.
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            c->q.qc[p] = c->q.qds[p] = c->q.qdl[p] = 0;
            c->f.fetch_s[np] = c->f.fetch_p[np] = 0;
        }
        const VisitBitmap vis{args.bm, args.lev, level + 1};
        // pieces: batch gw first without a fetch, later ones from the counter
        for (int i = gw; i < Fp;) {
            bfs_piece<K / 4>(a, w, args.pq[p][i], vis, np);
            int k = 0;
            if (lane == 0) k = atomicAdd(&c->f.fetch_p[p], 1);
            i = nw + __shfl_sync(0xffffffffu, k, 0);
        }
        // short vertices: chunks of 32 * V, V by the frontier's mean degree
        if (Fs > 0) {
            const long long avg = (long long)(qds / (unsigned long long)Fs);
            const int V = (avg >= 16 || Fs < 32 * 2 * nw) ? 1 : ((avg >= 6 || Fs < 32 * 4 * nw) ? 2 : 4);
            const int cw = 32 * V;
            const int nch = (Fs + cw - 1) / cw;
            for (int i = gw; i < nch;) {
                if (V == 1)
                    bfs_chunk<1, K>(a, w, args.sq[p], Fs, i * cw, vis, np);
                else if (V == 2)
                    bfs_chunk<2, K>(a, w, args.sq[p], Fs, i * cw, vis, np);
                else
                    bfs_chunk<4, K>(a, w, args.sq[p], Fs, i * cw, vis, np);
                int k = 0;
                if (lane == 0) k = atomicAdd(&c->f.fetch_s[p], 1);
                i = nw + __shfl_sync(0xffffffffu, k, 0);
            }
        }
        bfs_flush(a, w, np);
        const int g = grid_barrier_snap(c->b.bar, &c->b.err, gridDim.x, SnapBfs{c, np});
        if (g < 0) return;
        qc = ld_cg_u64(&c->snap[g & 1].qc);
        qds = ld_cg_u64(&c->snap[g & 1].qds);
        qdl = ld_cg_u64(&c->snap[g & 1].qdl);
        ++level;
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

static int ensure_bfs_ws(DevCtx *c, size_t nv, long long ne)
{
    if (!c->bfs_ctr) {
        FC_CUDA_TRY(cudaMalloc(&c->bfs_ctr, sizeof(BfsCounters)));
        FC_CUDA_TRY(cudaMemset(c->bfs_ctr, 0, sizeof(BfsCounters)));
        FC_CUDA_TRY(cudaMallocHost(&c->h_bfs_ctr, sizeof(BfsCounters)));
        std::memset(c->h_bfs_ctr, 0, sizeof(BfsCounters));
    }
    // pieces: at most one per long row plus one per BFS_PIECE entries
    const long long pcap = (long long)nv + ne / BFS_PIECE + 2;
    if (c->bfs_nv >= nv && c->bfs_pcap >= pcap && c->bfs_bm) return FC_OK;
    cudaFree(c->bfs_bm);
    cudaFree(c->bfs_lev);
    cudaFree(c->bfs_out);
    cudaFree(c->bfs_q);
    c->bfs_bm = nullptr;
    c->bfs_lev = c->bfs_out = nullptr;
    c->bfs_q = nullptr;
    c->bfs_nv = 0;
    c->bfs_pcap = 0;
    const size_t words = (nv + 1023) / 1024 * 32;  // whole 128-byte lines
    FC_CUDA_TRY(cudaMalloc(&c->bfs_bm, words * sizeof(unsigned)));
    FC_CUDA_TRY(cudaMalloc(&c->bfs_lev, nv * sizeof(int32_t)));
    FC_CUDA_TRY(cudaMalloc(&c->bfs_out, nv * sizeof(int32_t)));
    // two short queues of nv ranges and two piece queues of pcap ranges
    FC_CUDA_TRY(cudaMalloc(&c->bfs_q, sizeof(int2) * (2 * nv + 2 * (size_t)pcap)));
    FC_CUDA_TRY(cudaDeviceSynchronize());
    c->bfs_nv = nv;
    c->bfs_pcap = pcap;
    return FC_OK;
}

static int bfs_grid(DevCtx *c, const void *fn)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, BFS_T, 0) != cudaSuccess ||
        per_sm < 1)
        return 0;
    return per_sm * c->sm_count;
}

int engine_bfs_plain(DevCtx *c, const GraphPairH &gp, const BfsLayout *L, int32_t s,
                     int32_t *h_levels, const fc_opts &o, fc_stats *st, cudaStream_t stream)
{
    const int nv = gp.fwd.nv;
    int rc = ensure_bfs_ws(c, (size_t)nv, gp.fwd.ne);
    if (rc) return rc;
    if (!c->coop) {
        set_error("cooperative launch not supported on this device");
        return FC_ERR_UNSUPPORTED;
    }
    // resident CTAs per SM (fc_opts.ctas_per_sm): 2, 3 or 4 (the default)
    const void *fn = o.ctas_per_sm == 2   ? (const void *)k_bfs_plain<BFS_T, 2, 16>
                     : o.ctas_per_sm == 3 ? (const void *)k_bfs_plain<BFS_T, 3, 8>
                                          : (const void *)k_bfs_plain<BFS_T, 4, 8>;
    const int grid = bfs_grid(c, fn);
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
    a.scap = nv;
    a.pcap = c->bfs_pcap;
    a.sq[0] = c->bfs_q;
    a.sq[1] = c->bfs_q + nv;
    a.pq[0] = c->bfs_q + 2 * (size_t)nv;
    a.pq[1] = a.pq[0] + c->bfs_pcap;
    a.ctr = (BfsCounters *)c->bfs_ctr;
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
    FC_CUDA_TRY(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(BFS_T), args, 0, stream));
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
    if (hc->b.err) {
        set_error("k_bfs_plain: a grid barrier wait expired");
        return FC_ERR_TIMEOUT;
    }
    if (hc->overflow) {
        set_error("k_bfs_plain: %lld frontier queue writes refused", (long long)hc->overflow);
        return FC_ERR_CUDA;
    }
    if (st) {
        std::memset(st, 0, sizeof(*st));
        const long long reached = (long long)hc->reached;
        st->edges_inspected = (int64_t)hc->entries;
        st->visited = reached;
        st->steps = hc->levels;
        // 12 per frontier vertex + 8 per entry read + 8 per claimed vertex
        st->alg_bytes = (int64_t)(12 * reached + 8 * (long long)hc->entries + 8 * (reached - 1));
        st->launches = 4;
        st->visited_adjacency = (int64_t)hc->entries;
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
    *nlevels = hc->levels;
    const int n = std::min(hc->levels, BFS_TRACE_LEVELS);
    for (int l = 0; l < n && l < cap; ++l) {
        if (level_ns) level_ns[l] = (int64_t)(hc->trace.ns[l + 1] - hc->trace.ns[l]);
        if (frontier) frontier[l] = hc->trace.frontier[l];
        if (entries) entries[l] = (int64_t)hc->trace.entries[l];
    }
    return FC_OK;
}

}  // namespace fc
