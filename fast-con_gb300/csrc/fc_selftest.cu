// fc_selftest.cu -- the library's scan, compaction and search primitives run
// on caller data, so that tests can compare them element by element with
// plain restatements (the reference takes these from Thrust and CUB: the
// frontier-degree scan and its check check_queue_off, S/mythrustlib.cu:25-34,
// S/test/gputestfunc.cu:225-258; the queue compaction, S/mythrustlib.cu:
// 175-185; CUB's warp scan in K/src/device/Util/GlobalWrite.cu).
#include <algorithm>
#include <vector>

#include "fc_engine.h"
#include "fc_step.cuh"

namespace fc {

constexpr int ST_T = 256;

// 0: warp_inclusive_scan per group of 32; 1: block_inclusive_scan per group
// of ST_T, aux[g] = the group's total.
__global__ void __launch_bounds__(ST_T) k_selftest_scan(int which, const int32_t *in, int n,
                                                        int32_t *out, int32_t *aux)
{
    __shared__ int warp_tot[ST_T / 32];
    __shared__ int total;
    const long long i = (long long)blockIdx.x * ST_T + threadIdx.x;
    const int x = i < n ? in[i] : 0;
    if (which == 0) {
        const int r = warp_inclusive_scan(x);
        if (i < n) out[i] = r;
    } else {
        const int r = block_inclusive_scan<ST_T>(x, warp_tot, &total);
        if (i < n) out[i] = r;
        if (threadIdx.x == 0) aux[blockIdx.x] = total;
    }
}

// 2: load-balanced search.  Group g of ST_T row lengths is one tile; the tile's
// rows are laid end to end (exclusive prefix by the block scan) and every
// entry e of the concatenation gets lb_row(e), written at out[base_g + e]
// (base_g = entries of the earlier tiles, from the host).
__global__ void __launch_bounds__(ST_T) k_selftest_lb(const int32_t *len, int n,
                                                      const long long *tile_base, int32_t *out)
{
    __shared__ int warp_tot[ST_T / 32];
    __shared__ int total;
    __shared__ int off[ST_T];
    const long long i = (long long)blockIdx.x * ST_T + threadIdx.x;
    const int d = i < n ? len[i] : 0;
    const int incl = block_inclusive_scan<ST_T>(d, warp_tot, &total);
    off[threadIdx.x] = incl - d;
    __syncthreads();
    const long long base = tile_base[blockIdx.x];
    for (int e = threadIdx.x; e < total; e += ST_T) out[base + e] = lb_row<ST_T>(off, e);
}

// 3: claim compaction.  One CTA; every thread offers GATHER_PER_THREAD values
// per round (-1 = none); the offered values are appended to the log through
// the per-warp shared-memory buffers (warp_append / warp_flush), exactly as
// the expansion steps append claimed vertices.  aux[0] = log length.
__global__ void __launch_bounds__(ST_T) k_selftest_append(const int32_t *in, int n,
                                                          const int32_t *row_ptr, int32_t *log,
                                                          int *tail, unsigned long long *deg)
{
    constexpr int K = GATHER_PER_THREAD;
    __shared__ int wcnt[ST_T / 32];
    __shared__ int wlog[ST_T / 32][WARP_LOG];
    AppendTarget app{log, n, 0, tail, deg, row_ptr, nullptr, nullptr};
    app.wlog = &wlog[0][0];
    app.wcnt = wcnt;
    if (lane_id() == 0) wcnt[threadIdx.x >> 5] = 0;
    __syncwarp();
    for (int base = 0; base < n; base += ST_T * K) {
        int c[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int i = base + k * ST_T + threadIdx.x;
            c[k] = i < n ? in[i] : -1;
        }
        warp_append<K>(c, app);
    }
    warp_flush(app);
}

int engine_selftest_primitives(DevCtx *c, int which, const int32_t *h_in, int n, int32_t *h_out,
                               int32_t *h_aux, cudaStream_t st)
{
    int32_t *d_in = nullptr, *d_out = nullptr, *d_aux = nullptr, *d_rp = nullptr;
    long long *d_base = nullptr;
    unsigned long long *d_deg = nullptr;
    int rc = FC_OK;
    const int groups = (n + ST_T - 1) / ST_T;
    auto fail = [&](cudaError_t e, const char *what) {
        fc_set_last_cuda_error(e, what, __FILE__, __LINE__);
        rc = e == cudaErrorMemoryAllocation ? FC_ERR_OOM : FC_ERR_CUDA;
    };
    cudaError_t e = cudaMalloc(&d_in, sizeof(int32_t) * (size_t)std::max(1, n));
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_in, h_in, sizeof(int32_t) * (size_t)n,
                                              cudaMemcpyHostToDevice, st);
    long long out_n = n;
    std::vector<long long> base;
    if (which == 2) {  // entries of the earlier tiles
        base.assign((size_t)groups + 1, 0);
        for (int g = 0; g < groups; ++g) {
            long long s = 0;
            for (int i = g * ST_T; i < std::min(n, (g + 1) * ST_T); ++i) s += h_in[i];
            base[(size_t)g + 1] = base[(size_t)g] + s;
        }
        out_n = base[(size_t)groups];
    }
    if (e == cudaSuccess) e = cudaMalloc(&d_out, sizeof(int32_t) * (size_t)std::max(1LL, out_n));
    if (e == cudaSuccess) e = cudaMalloc(&d_aux, sizeof(int32_t) * (size_t)std::max(1, groups));
    if (e != cudaSuccess) fail(e, "self-test buffers");
    if (rc == FC_OK) {
        if (which == 0 || which == 1) {
            k_selftest_scan<<<std::max(1, groups), ST_T, 0, st>>>(which, d_in, n, d_out, d_aux);
        } else if (which == 2) {
            if ((e = cudaMalloc(&d_base, sizeof(long long) * base.size())) != cudaSuccess ||
                (e = cudaMemcpyAsync(d_base, base.data(), sizeof(long long) * base.size(),
                                     cudaMemcpyHostToDevice, st)) != cudaSuccess)
                fail(e, "self-test tile bases");
            else
                k_selftest_lb<<<std::max(1, groups), ST_T, 0, st>>>(d_in, n, d_base, d_out);
        } else {
            int maxv = 0;
            for (int i = 0; i < n; ++i) maxv = std::max(maxv, h_in[i]);
            if ((e = cudaMalloc(&d_rp, sizeof(int32_t) * ((size_t)maxv + 2))) != cudaSuccess ||
                (e = cudaMemsetAsync(d_rp, 0, sizeof(int32_t) * ((size_t)maxv + 2), st)) != cudaSuccess ||
                (e = cudaMalloc(&d_deg, sizeof(unsigned long long))) != cudaSuccess ||
                (e = cudaMemsetAsync(d_deg, 0, sizeof(unsigned long long), st)) != cudaSuccess ||
                (e = cudaMemsetAsync(d_aux, 0, sizeof(int32_t), st)) != cudaSuccess)
                fail(e, "self-test append buffers");
            else
                k_selftest_append<<<1, ST_T, 0, st>>>(d_in, n, d_rp, d_out, d_aux, d_deg);
        }
    }
    if (rc == FC_OK && (e = cudaGetLastError()) != cudaSuccess) fail(e, "self-test launch");
    if (rc == FC_OK) {
        if ((e = cudaMemcpyAsync(h_out, d_out, sizeof(int32_t) * (size_t)out_n,
                                 cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (h_aux && (e = cudaMemcpyAsync(h_aux, d_aux,
                                           sizeof(int32_t) * (size_t)(which == 3 ? 1 : groups),
                                           cudaMemcpyDeviceToHost, st)) != cudaSuccess) ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            fail(e, "self-test results");
    }
    cudaStreamSynchronize(st);
    cudaFree(d_in);
    cudaFree(d_out);
    cudaFree(d_aux);
    cudaFree(d_rp);
    cudaFree(d_base);
    cudaFree(d_deg);
    return rc;
}

}  // namespace fc
