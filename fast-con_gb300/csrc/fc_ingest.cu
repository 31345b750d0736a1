// fc_ingest.cu -- edge list -> canonical int32 CSR, built on the device, and
// the seeded graph generators.
//
// Ingest (replaces make_g_undirect / make_own_csr_nomulti / make_offset,
// S/make_struct.c:304-359, 553-738 and the kernels k_add_vu, k_find_duplicates,
// k_count_vert, k_degree in S/cudakernel/gstruct_kernel.cu:114-235, which run
// Thrust sorts over 2E int64 pairs):
//   1. count      per-vertex degree with atomics (both directions unless
//                 directed; self-loops dropped unless kept; src < 0 = no edge)
//   2. scan       exclusive scan of the degrees (own reduce-then-scan kernels)
//   3. scatter    each entry to its row through a per-row atomic cursor
//   4. sort       every row, by size class: warp bitonic (<= 32), CTA bitonic in
//                 shared memory (<= 8192), CTA chunk sort + merge-path merges
//   5. dedupe     warp ballot counts first occurrences, scan -> row_ptr, then a
//                 ballot-compaction writes the final column array
// The result is byte-identical to the CPU canonical CSR (rows sorted,
// duplicates and loops removed, both directions stored).
#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

#include "fc_ingest.h"
#include "fc_internal.cuh"

namespace fc {

constexpr int IB = 256;           // ingest block size
constexpr int MED_MAX = 8192;     // rows sorted in one shared-memory bitonic pass
constexpr int SCAN_TILE = IB * 8;

// ---------------------------------------------------------------------------
// counter-based hash, identical to fastcon/graphs.py
// ---------------------------------------------------------------------------
__host__ __device__ inline unsigned long long mix64(unsigned long long z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
constexpr unsigned long long GOLDEN = 0x9E3779B97F4A7C15ull;

__host__ __device__ inline unsigned long long hash_base(unsigned long long seed,
                                                        unsigned long long stream)
{
    return mix64(seed * GOLDEN + stream);
}
__host__ __device__ inline unsigned long long hash_at(unsigned long long base,
                                                      unsigned long long i)
{
    return mix64(base + (i + 1) * GOLDEN);
}
__host__ __device__ inline int scale_to(unsigned long long x32, unsigned long long n)
{
    return (int)((x32 * n) >> 32);
}

// ---------------------------------------------------------------------------
// scan (exclusive, int64 output)
// ---------------------------------------------------------------------------
template <class In>
__global__ void __launch_bounds__(IB) k_tile_reduce(const In *in, long long n, long long *sums)
{
    long long base = (long long)blockIdx.x * SCAN_TILE;
    long long acc = 0;
    for (int k = 0; k < SCAN_TILE / IB; ++k) {
        long long i = base + k * IB + threadIdx.x;
        if (i < n) acc += (long long)in[i];
    }
    acc = warp_sum_ll(acc);
    __shared__ long long ws[IB / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        long long v = threadIdx.x < IB / 32 ? ws[threadIdx.x] : 0;
        v = warp_sum_ll(v);
        if (threadIdx.x == 0) sums[blockIdx.x] = v;
    }
}

__device__ __forceinline__ long long warp_incl_ll(long long x)
{
    unsigned l = lane_id();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (l >= (unsigned)o) x += y;
    }
    return x;
}

// Each thread owns 8 consecutive elements of the tile.
template <class In>
__global__ void __launch_bounds__(IB) k_tile_scan(const In *in, long long n, long long *out,
                                                  const long long *tile_off)
{
    constexpr int PER = SCAN_TILE / IB;
    long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * PER;
    long long v[PER];
    long long s = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        long long i = base + k;
        v[k] = i < n ? (long long)in[i] : 0;
        s += v[k];
    }
    long long incl = warp_incl_ll(s);
    __shared__ long long ws[IB / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 31) ws[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        long long w = lane < IB / 32 ? ws[lane] : 0;
        long long wi = warp_incl_ll(w);
        if (lane < IB / 32) ws[lane] = wi - w;
    }
    __syncthreads();
    long long run = incl - s + ws[wid] + (tile_off ? tile_off[blockIdx.x] : 0);
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        long long i = base + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
}

// exclusive scan of n elements into out[0..n); out[n] = total.
template <class In>
static int exclusive_scan(const In *in, long long n, long long *out, cudaStream_t st)
{
    long long tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (tiles <= 1) {
        long long *tot = nullptr;
        FC_CUDA_TRY(cudaMallocAsync(&tot, sizeof(long long) * 2, st));
        k_tile_reduce<In><<<1, IB, 0, st>>>(in, n, tot);
        k_tile_scan<In><<<1, IB, 0, st>>>(in, n, out, nullptr);
        FC_CUDA_TRY(cudaMemcpyAsync(out + n, tot, sizeof(long long), cudaMemcpyDeviceToDevice, st));
        FC_CUDA_TRY(cudaFreeAsync(tot, st));
        return FC_OK;
    }
    long long *sums = nullptr;
    FC_CUDA_TRY(cudaMallocAsync(&sums, sizeof(long long) * (size_t)(2 * tiles + 1), st));
    long long *soff = sums + tiles;
    k_tile_reduce<In><<<(unsigned)tiles, IB, 0, st>>>(in, n, sums);
    int rc = exclusive_scan<long long>(sums, tiles, soff, st);
    if (rc) return rc;
    k_tile_scan<In><<<(unsigned)tiles, IB, 0, st>>>(in, n, out, soff);
    FC_CUDA_TRY(cudaMemcpyAsync(out + n, soff + tiles, sizeof(long long), cudaMemcpyDeviceToDevice, st));
    FC_CUDA_TRY(cudaFreeAsync(sums, st));
    FC_CUDA_TRY(cudaGetLastError());
    return FC_OK;
}

int scan_i32(const int32_t *in, long long n, long long *out, cudaStream_t st)
{
    return exclusive_scan<int32_t>(in, n, out, st);
}

// ---------------------------------------------------------------------------
// count / scatter
// ---------------------------------------------------------------------------
__global__ void k_count(const int32_t *src, const int32_t *dst, long long n, int nv, int flags,
                        int *deg, int *bad)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        int u = src[i], v = dst[i];
        if (u == -1) continue;  // "no edge" marker (deleted / ignored entries)
        if (u < 0 || u >= nv || v < 0 || v >= nv) {
            *bad = 1;
            continue;
        }
        if (u == v && !(flags & FC_INGEST_KEEP_LOOPS)) continue;
        atomicAdd(deg + u, 1);
        if (!(flags & FC_INGEST_DIRECTED)) atomicAdd(deg + v, 1);
    }
}

__global__ void k_scatter(const int32_t *src, const int32_t *dst, long long n, int nv, int flags,
                          unsigned long long *cursor, int32_t *tmp)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        int u = src[i], v = dst[i];
        if (u < 0 || u >= nv || v < 0 || v >= nv) continue;
        if (u == v && !(flags & FC_INGEST_KEEP_LOOPS)) continue;
        unsigned long long p = atomicAdd(cursor + u, 1ull);
        tmp[p] = v;
        if (!(flags & FC_INGEST_DIRECTED)) {
            unsigned long long q = atomicAdd(cursor + v, 1ull);
            tmp[q] = u;
        }
    }
}

// ---------------------------------------------------------------------------
// per-row sort
// ---------------------------------------------------------------------------
__global__ void k_classify(const long long *off, int nv, int *lists, int *counts)
{
    // lists: [0, nv) small, [nv, 2nv) medium, [2nv, 3nv) large
    int u = blockIdx.x * blockDim.x + threadIdx.x;
    int cls = -1;
    if (u < nv) {
        long long L = off[u + 1] - off[u];
        if (L > MED_MAX)
            cls = 2;
        else if (L > 32)
            cls = 1;
        else if (L > 1)
            cls = 0;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        unsigned m = __ballot_sync(0xffffffffu, cls == c);
        if (!m) continue;
        int base = 0;
        if (lane_id() == 0) base = atomicAdd(counts + c, __popc(m));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (cls == c) lists[(size_t)c * nv + base + __popc(m & lanemask_lt())] = u;
    }
}

__global__ void k_sort_small(const long long *off, const int *list, const int *count, int32_t *tmp)
{
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    const int n = *count;
    for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < n; w += warps) {
        int u = list[w];
        long long b = off[u];
        int L = (int)(off[u + 1] - b);
        int x = lane < L ? tmp[b + lane] : INT_MAX;
#pragma unroll
        for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
            for (int j = k >> 1; j > 0; j >>= 1) {
                int y = __shfl_xor_sync(0xffffffffu, x, j);
                bool up = (lane & k) == 0;
                bool lower = (lane & j) == 0;
                x = (lower == up) ? min(x, y) : max(x, y);
            }
        }
        if (lane < L) tmp[b + lane] = x;
    }
}

// bitonic sort of s[0, P) (P a power of two) by the whole CTA
__device__ void smem_bitonic(int *s, int P)
{
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P / 2; i += blockDim.x) {
                int lo = 2 * j * (i / j) + (i % j);
                int hi = lo + j;
                bool up = (lo & k) == 0;
                int a = s[lo], b = s[hi];
                if ((a > b) == up) {
                    s[lo] = b;
                    s[hi] = a;
                }
            }
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(IB) k_sort_medium(const long long *off, const int *list,
                                                    const int *count, int32_t *tmp)
{
    __shared__ int s[MED_MAX];
    const int n = *count;
    for (int r = blockIdx.x; r < n; r += gridDim.x) {
        int u = list[r];
        long long b = off[u];
        int L = (int)(off[u + 1] - b);
        int P = 64;
        while (P < L) P <<= 1;
        for (int i = threadIdx.x; i < P; i += blockDim.x) s[i] = i < L ? tmp[b + i] : INT_MAX;
        __syncthreads();
        smem_bitonic(s, P);
        for (int i = threadIdx.x; i < L; i += blockDim.x) tmp[b + i] = s[i];
        __syncthreads();
    }
}

// Large rows: sort 8192-chunks in shared memory, then merge runs pairwise
// (merge path: every thread finds its diagonal split by binary search and
// merges 8 outputs), ping-ponging between the row and a scratch copy.
__global__ void __launch_bounds__(IB) k_sort_large(const long long *off, const int *list,
                                                   const int *count, int32_t *tmp, int32_t *scratch)
{
    __shared__ int s[MED_MAX];
    const int n = *count;
    for (int r = blockIdx.x; r < n; r += gridDim.x) {
        int u = list[r];
        long long b = off[u];
        long long L = off[u + 1] - b;
        for (long long c0 = 0; c0 < L; c0 += MED_MAX) {
            int cl = (int)min((long long)MED_MAX, L - c0);
            for (int i = threadIdx.x; i < MED_MAX; i += blockDim.x) s[i] = i < cl ? tmp[b + c0 + i] : INT_MAX;
            __syncthreads();
            smem_bitonic(s, MED_MAX);
            for (int i = threadIdx.x; i < cl; i += blockDim.x) tmp[b + c0 + i] = s[i];
            __syncthreads();
        }
        int32_t *A = tmp + b, *B = scratch + b;
        for (long long w = MED_MAX; w < L; w <<= 1) {
            for (long long lo = 0; lo < L; lo += 2 * w) {
                long long na = min(w, L - lo);
                long long nb = min(w, max(0ll, L - lo - w));
                const int32_t *a = A + lo, *bb = A + lo + na;
                int32_t *o = B + lo;
                long long tot = na + nb;
                for (long long d0 = (long long)threadIdx.x * 8; d0 < tot; d0 += (long long)blockDim.x * 8) {
                    long long l2 = max(0ll, d0 - nb), h2 = min(d0, na);
                    while (l2 < h2) {
                        long long mid = (l2 + h2) >> 1;
                        if (a[mid] <= bb[d0 - 1 - mid])
                            l2 = mid + 1;
                        else
                            h2 = mid;
                    }
                    long long i = l2, j = d0 - l2;
                    for (int k = 0; k < 8 && d0 + k < tot; ++k) {
                        if (j >= nb || (i < na && a[i] <= bb[j]))
                            o[d0 + k] = a[i++];
                        else
                            o[d0 + k] = bb[j++];
                    }
                }
            }
            __syncthreads();
            int32_t *t = A;
            A = B;
            B = t;
        }
        if (A != tmp + b)
            for (long long i = threadIdx.x; i < L; i += blockDim.x) tmp[b + i] = A[i];
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// dedupe + compaction (warp per row)
// ---------------------------------------------------------------------------
__global__ void k_count_unique(const long long *off, int nv, const int32_t *tmp, int dedupe,
                               int *ndeg)
{
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < nv; u += warps) {
        long long b = off[u], e = off[u + 1];
        if (!dedupe) {
            if (lane == 0) ndeg[u] = (int)(e - b);
            continue;
        }
        int cnt = 0;
        for (long long j0 = b; j0 < e; j0 += 32) {
            long long j = j0 + lane;
            bool keep = j < e && (j == b || tmp[j] != tmp[j - 1]);
            cnt += __popc(__ballot_sync(0xffffffffu, keep));
        }
        if (lane == 0) ndeg[u] = cnt;
    }
}

__global__ void k_compact(const long long *off, int nv, const int32_t *tmp, int dedupe,
                          const long long *noff, int32_t *row_ptr, int32_t *col)
{
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < nv; u += warps) {
        long long b = off[u], e = off[u + 1];
        long long o = noff[u];
        if (lane == 0) row_ptr[u] = (int32_t)o;
        for (long long j0 = b; j0 < e; j0 += 32) {
            long long j = j0 + lane;
            bool keep = j < e && (!dedupe || j == b || tmp[j] != tmp[j - 1]);
            unsigned m = __ballot_sync(0xffffffffu, keep);
            if (keep) col[o + __popc(m & lanemask_lt())] = tmp[j];
            o += __popc(m);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) row_ptr[nv] = (int32_t)noff[nv];
}

// ---------------------------------------------------------------------------
// generators
// ---------------------------------------------------------------------------
struct PermParams {
    unsigned long long mask;
    unsigned long long mult[3], add[3];
    int shift;
    int on;
};

__host__ __device__ inline unsigned long long permute(unsigned long long x, const PermParams &p)
{
    for (int r = 0; r < 3; ++r) {
        x = (x * p.mult[r] + p.add[r]) & p.mask;
        x ^= x >> p.shift;
    }
    return x;
}

__global__ void k_gen_rmat(int scale, long long nedges, unsigned t1, unsigned t2, unsigned t3,
                           unsigned long long seed, PermParams pp, int32_t *src, int32_t *dst)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nedges;
         i += (long long)gridDim.x * blockDim.x) {
        unsigned long long u = 0, v = 0;
        for (int k = 0; k < scale; ++k) {
            unsigned x = (unsigned)(hash_at(hash_base(seed, (unsigned long long)(k + 1)),
                                            (unsigned long long)i) >> 32);
            unsigned long long ub = x >= t2;
            unsigned long long vb = (x >= t1 && x < t2) || x >= t3;
            u |= ub << k;
            v |= vb << k;
        }
        if (pp.on) {
            u = permute(u, pp);
            v = permute(v, pp);
        }
        src[i] = (int32_t)u;
        dst[i] = (int32_t)v;
    }
}

__global__ void k_gen_grid(int w, int h, unsigned thr, unsigned long long del_seed,
                           long long shortcuts, unsigned long long sc_seed, int32_t *src,
                           int32_t *dst)
{
    const long long nh = (long long)h * (w - 1), nvv = (long long)(h - 1) * w;
    const long long total = nh + nvv + shortcuts;
    const unsigned long long dbase = hash_base(del_seed, 0), sbase = hash_base(sc_seed, 0);
    const unsigned long long n = (unsigned long long)w * h;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        long long u, v;
        if (i < nh + nvv) {
            if (i < nh) {
                long long r = i / (w - 1), c = i % (w - 1);
                u = r * w + c;
                v = u + 1;
            } else {
                long long k = i - nh;
                long long r = k / w, c = k % w;
                u = r * w + c;
                v = u + w;
            }
            unsigned x = (unsigned)(hash_at(dbase, (unsigned long long)i) >> 32);
            if (x < thr) u = v = -1;
        } else {
            unsigned long long rr = hash_at(sbase, (unsigned long long)(i - nh - nvv));
            u = scale_to(rr & 0xFFFFFFFFull, n);
            v = scale_to(rr >> 32, n);
        }
        src[i] = (int32_t)u;
        dst[i] = (int32_t)v;
    }
}

// ---------------------------------------------------------------------------
// host drivers
// ---------------------------------------------------------------------------
static int grid_for(long long n, int block = IB)
{
    long long g = (n + block - 1) / block;
    if (g > 152 * 64) g = 152 * 64;
    if (g < 1) g = 1;
    return (int)g;
}

int sort_rows_i32(const long long *off, int nv, long long ne, int32_t *col, cudaStream_t st)
{
    int *lists = nullptr, *counts = nullptr;
    int32_t *scratch = nullptr;
    int h_counts[3] = {0, 0, 0};
    int rc = FC_OK;
    auto fail = [&](cudaError_t e, const char *what) {
        fc_set_last_cuda_error(e, what, __FILE__, __LINE__);
        rc = e == cudaErrorMemoryAllocation ? FC_ERR_OOM : FC_ERR_CUDA;
    };
    cudaError_t e;
    if ((e = cudaMalloc(&lists, sizeof(int) * (size_t)nv * 3)) != cudaSuccess ||
        (e = cudaMalloc(&counts, sizeof(int) * 4)) != cudaSuccess ||
        (e = cudaMemsetAsync(counts, 0, sizeof(int) * 4, st)) != cudaSuccess) {
        fail(e, "row sort set-up");
    } else {
        k_classify<<<(nv + IB - 1) / IB, IB, 0, st>>>(off, nv, lists, counts);
        if ((e = cudaGetLastError()) != cudaSuccess ||
            (e = cudaMemcpyAsync(h_counts, counts, sizeof(int) * 3, cudaMemcpyDeviceToHost, st)) !=
                cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            fail(e, "row classes");
    }
    if (rc == FC_OK && h_counts[2] &&
        (e = cudaMalloc(&scratch, sizeof(int32_t) * (size_t)std::max(1ll, ne))) != cudaSuccess)
        fail(e, "row sort scratch");
    if (rc == FC_OK) {
        if (h_counts[0])
            k_sort_small<<<grid_for((long long)h_counts[0] * 32), IB, 0, st>>>(off, lists, counts, col);
        if (h_counts[1])
            k_sort_medium<<<std::min(h_counts[1], 152 * 8), IB, 0, st>>>(off, lists + (size_t)nv,
                                                                         counts + 1, col);
        if (h_counts[2])
            k_sort_large<<<std::min(h_counts[2], 152 * 4), IB, 0, st>>>(off, lists + 2 * (size_t)nv,
                                                                        counts + 2, col, scratch);
        if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaStreamSynchronize(st)) != cudaSuccess)
            fail(e, "row sort kernels");
    }
    cudaFree(lists);
    cudaFree(counts);
    cudaFree(scratch);
    return rc;
}

int ingest_device_edges(const int32_t *d_src, const int32_t *d_dst, long long n, int nv, int flags,
                        int32_t **out_row_ptr, int32_t **out_col, long long *out_ne,
                        cudaStream_t st)
{
    *out_row_ptr = nullptr;
    *out_col = nullptr;
    *out_ne = 0;
    if (nv <= 0) return FC_ERR_INVALID;
    int *deg = nullptr, *bad = nullptr, *ndeg = nullptr;
    long long *off = nullptr, *noff = nullptr;
    int32_t *tmp = nullptr, *row_ptr = nullptr, *col = nullptr;
    int rc = FC_OK;
    int h_bad = 0;
    long long total = 0, ne = 0;
    const int dedupe = !(flags & FC_INGEST_KEEP_DUPS);
#define ING_TRY(expr)                                                   \
    do {                                                                \
        cudaError_t e_ = (expr);                                        \
        if (e_ != cudaSuccess) {                                        \
            fc_set_last_cuda_error(e_, #expr, __FILE__, __LINE__);      \
            rc = e_ == cudaErrorMemoryAllocation ? FC_ERR_OOM : FC_ERR_CUDA; \
            goto done;                                                  \
        }                                                               \
    } while (0)
    ING_TRY(cudaMalloc(&deg, sizeof(int) * ((size_t)nv + 1) + 16));
    bad = deg + nv + 1;
    ING_TRY(cudaMemsetAsync(deg, 0, sizeof(int) * ((size_t)nv + 1) + 16, st));
    if (n > 0) {
        k_count<<<grid_for(n), IB, 0, st>>>(d_src, d_dst, n, nv, flags, deg, bad);
        ING_TRY(cudaGetLastError());
    }
    ING_TRY(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    ING_TRY(cudaMalloc(&off, sizeof(long long) * ((size_t)nv + 1)));
    rc = exclusive_scan<int>(deg, nv, off, st);
    if (rc) goto done;
    ING_TRY(cudaMemcpyAsync(&total, off + nv, sizeof(long long), cudaMemcpyDeviceToHost, st));
    ING_TRY(cudaStreamSynchronize(st));
    if (h_bad) {
        set_error("edge list has a vertex id outside [0, %d)", nv);
        rc = FC_ERR_INVALID;
        goto done;
    }
    {
        // scatter through a cursor copy of the offsets (reuse `noff` storage)
        ING_TRY(cudaMalloc(&noff, sizeof(long long) * ((size_t)nv + 1)));
        ING_TRY(cudaMemcpyAsync(noff, off, sizeof(long long) * ((size_t)nv + 1),
                                cudaMemcpyDeviceToDevice, st));
        ING_TRY(cudaMalloc(&tmp, sizeof(int32_t) * (size_t)std::max(1ll, total)));
        if (n > 0) {
            k_scatter<<<grid_for(n), IB, 0, st>>>(d_src, d_dst, n, nv, flags,
                                                  (unsigned long long *)noff, tmp);
            ING_TRY(cudaGetLastError());
        }
        // sort rows by size class
        rc = sort_rows_i32(off, nv, total, tmp, st);
        if (rc) goto done;
        // dedupe: count, scan, compact
        ndeg = deg;  // reuse
        k_count_unique<<<grid_for((long long)nv * 32), IB, 0, st>>>(off, nv, tmp, dedupe, ndeg);
        ING_TRY(cudaGetLastError());
        rc = exclusive_scan<int>(ndeg, nv, noff, st);
        if (rc) goto done;
        ING_TRY(cudaMemcpyAsync(&ne, noff + nv, sizeof(long long), cudaMemcpyDeviceToHost, st));
        ING_TRY(cudaStreamSynchronize(st));
        if (ne > (long long)INT_MAX) {
            set_error("graph has %lld entries; the int32 CSR holds at most %d", ne, INT_MAX);
            rc = FC_ERR_OVERFLOW;
            goto done;
        }
        ING_TRY(cudaMalloc(&row_ptr, sizeof(int32_t) * ((size_t)nv + 1)));
        ING_TRY(cudaMalloc(&col, sizeof(int32_t) * (size_t)std::max(1ll, ne) + 16));
        k_compact<<<grid_for((long long)nv * 32), IB, 0, st>>>(off, nv, tmp, dedupe, noff, row_ptr, col);
        ING_TRY(cudaGetLastError());
        ING_TRY(cudaStreamSynchronize(st));
    }
done:
#undef ING_TRY
    cudaFree(deg);
    cudaFree(off);
    cudaFree(noff);
    cudaFree(tmp);
    if (rc != FC_OK) {
        cudaFree(row_ptr);
        cudaFree(col);
        return rc;
    }
    *out_row_ptr = row_ptr;
    *out_col = col;
    *out_ne = ne;
    return FC_OK;
}

static PermParams make_perm(int scale, long long perm_seed)
{
    PermParams p;
    std::memset(&p, 0, sizeof(p));
    p.on = perm_seed >= 0;
    p.mask = scale >= 64 ? ~0ull : ((1ull << scale) - 1);
    for (int r = 0; r < 3; ++r) {
        unsigned long long h = hash_at(hash_base((unsigned long long)perm_seed, 0x5EED0ull + r), 0);
        p.mult[r] = (h | 1ull) & p.mask;
        p.add[r] = (h >> 32) & p.mask;
    }
    p.shift = scale / 2 + 1;
    return p;
}

int gen_rmat_device(int scale, long long nedges, double a, double b, double c,
                    unsigned long long seed, long long perm_seed, int32_t *d_src, int32_t *d_dst,
                    cudaStream_t st)
{
    unsigned t1 = (unsigned)(a * 4294967296.0);
    unsigned t2 = (unsigned)((a + b) * 4294967296.0);
    unsigned t3 = (unsigned)((a + b + c) * 4294967296.0);
    PermParams pp = make_perm(scale, perm_seed);
    if (nedges > 0)
        k_gen_rmat<<<grid_for(nedges), IB, 0, st>>>(scale, nedges, t1, t2, t3, seed, pp, d_src, d_dst);
    FC_CUDA_TRY(cudaGetLastError());
    return FC_OK;
}

long long grid_edge_slots(int w, int h, long long shortcuts)
{
    return (long long)h * (w - 1) + (long long)(h - 1) * w + shortcuts;
}

int gen_grid_device(int w, int h, double p_del, unsigned long long del_seed, long long shortcuts,
                    unsigned long long sc_seed, int32_t *d_src, int32_t *d_dst, cudaStream_t st)
{
    unsigned thr = (unsigned)(p_del * 4294967296.0);
    long long total = grid_edge_slots(w, h, shortcuts);
    if (total > 0)
        k_gen_grid<<<grid_for(total), IB, 0, st>>>(w, h, thr, del_seed, shortcuts, sc_seed, d_src, d_dst);
    FC_CUDA_TRY(cudaGetLastError());
    return FC_OK;
}

}  // namespace fc
