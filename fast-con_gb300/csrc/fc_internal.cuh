// fc_internal.cuh -- shared device/host definitions of the fastcon library.
//
// Layout of one graph in HBM (built by fc_ingest.cu):
//   row_ptr  int32[nv + 1]   offsets, 256-byte aligned allocation
//   col      int32[ne]       neighbours, rows sorted ascending, deduplicated
//
// Traversal state of one query slot:
//   status   uint8[nv, padded to 16]   0xFF = unvisited, else side<<7 | min(level,126)
//   log      int32[nv]                 every claimed vertex exactly once; side 0
//                                      appends upward from log[0], side 1 downward
//                                      from log[nv-1], so a side's frontier is always
//                                      one contiguous range of the log
// A full BFS (level-array output) uses int32 levels (-1 = unvisited) in place of
// the status bytes and only side 0 of the log.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fastcon.h"

#ifndef FC_BLOCK
#define FC_BLOCK 256
#endif

namespace fc {

constexpr uint8_t ST_UNVISITED = 0xFF;
// Levels are stored clamped to 126, so side 1's largest code is 0xFE and never
// equals ST_UNVISITED.  Bottom-up compares exact frontier codes, so it is used
// only while level + 1 <= 125 (below the clamp).
constexpr int LEVEL_CLAMP = 126;
constexpr int LEVEL7_MAX = 125;

__host__ __device__ inline uint8_t st_code(int side, int level)
{
    return (uint8_t)((side << 7) | (level < LEVEL_CLAMP ? level : LEVEL_CLAMP));
}

struct DGraph {
    const int32_t *row_ptr;
    const int32_t *col;
    int32_t nv;
    int32_t pad_;
    int64_t ne;
    const int32_t *remap;  // nullable: caller's vertex id -> id in this CSR
};

// ---------------------------------------------------------------------------
// warp helpers (hand-written PTX only for the special registers)
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned lane_id()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%laneid;" : "=r"(r));
    return r;
}

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
    return r;
}

__device__ __forceinline__ unsigned long long global_timer_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ int warp_inclusive_scan(int x)
{
    unsigned l = lane_id();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (l >= (unsigned)o) x += y;
    }
    return x;
}

__device__ __forceinline__ long long warp_sum_ll(long long x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

__device__ __forceinline__ int warp_sum_i(int x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// Loads that bypass L1: status, log and counters are written by other SMs
// during the same kernel, and L1 is not coherent across SMs.
__device__ __forceinline__ int ld_cg(const int *p) { return __ldcg(p); }
__device__ __forceinline__ long long ld_cg(const long long *p) { return __ldcg(p); }
__device__ __forceinline__ unsigned long long ld_cg_u64(const unsigned long long *p)
{
    return __ldcg(p);
}
__device__ __forceinline__ uint8_t ld_cg_u8(const uint8_t *p)
{
    return (uint8_t)__ldcg((const unsigned char *)p);
}

__device__ __forceinline__ int ld_acquire_gpu(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_gpu(int *p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// ---------------------------------------------------------------------------
// Software grid barrier for cooperative launches.  Every wait is bounded by
// an iteration count and by %globaltimer; on expiry the barrier records
// FC_ERR_TIMEOUT in *err and returns false, and the caller returns.
// bar[0] = arrival count, bar[1] = generation.
// ---------------------------------------------------------------------------
constexpr unsigned long long BARRIER_TIMEOUT_NS = 2000000000ull;  // 2 s
constexpr long long BARRIER_MAX_SPINS = 1ll << 25;

// grid_barrier_snap: the same barrier; in addition the last CTA to arrive
// calls snap(gen & 1) -- every CTA's writes before the barrier are visible to
// it -- before it releases the others.  A team whose CTAs read shared
// counters after a barrier while faster CTAs already update them for the next
// step reads the snapshot instead: the copy for generation g is rewritten at
// generation g + 2, after every CTA has passed g + 1.  Returns the generation
// waited on, or -1 when the wait expired.
struct NoSnap {
    __device__ __forceinline__ void operator()(int) const {}
};

template <class Snap>
__device__ __forceinline__ int grid_barrier_snap(int *bar, int *err, int nblocks, const Snap &snap,
                                                 unsigned long long timeout_ns = BARRIER_TIMEOUT_NS)
{
    __syncthreads();
    __shared__ int s_gen;
    if (threadIdx.x == 0) {
        int ok = 1;
        int gen = ld_acquire_gpu(bar + 1);
        __threadfence();
        int arrived = atomicAdd(bar, 1) + 1;
        if (arrived == nblocks) {
            __threadfence();
            snap(gen & 1);
            __threadfence();
            atomicExch(bar, 0);
            __threadfence();
            st_release_gpu(bar + 1, gen + 1);
        } else {
            // pollers back off (64 ns doubling to 512 ns): hundreds of CTAs
            // polling one word at a fixed short interval load its L2 slice
            // enough to slow the atomics of the CTAs still working
            unsigned long long t0 = global_timer_ns();
            long long spins = 0;
            unsigned pause = 64;
            while (ld_acquire_gpu(bar + 1) == gen) {
                if (++spins > BARRIER_MAX_SPINS ||
                    ((spins & 63) == 0 && global_timer_ns() - t0 > timeout_ns)) {
                    atomicCAS(err, 0, FC_ERR_TIMEOUT);
                    ok = 0;
                    break;
                }
                __nanosleep(pause);
                if (pause < 512) pause <<= 1;
            }
        }
        if (ok && ld_acquire_gpu(err) != 0) ok = 0;
        s_gen = ok ? (gen & 0x7fffffff) : -1;
    }
    __syncthreads();
    return s_gen;
}

__device__ __forceinline__ bool grid_barrier(int *bar, int *err, int nblocks,
                                             unsigned long long timeout_ns = BARRIER_TIMEOUT_NS)
{
    return grid_barrier_snap(bar, err, nblocks, NoSnap{}, timeout_ns) >= 0;
}

}  // namespace fc

// ---------------------------------------------------------------------------
// host-side helpers
// ---------------------------------------------------------------------------
#define FC_CUDA_TRY(expr)                                   \
    do {                                                    \
        cudaError_t e_ = (expr);                            \
        if (e_ != cudaSuccess) {                            \
            fc_set_last_cuda_error(e_, #expr, __FILE__, __LINE__); \
            return e_ == cudaErrorMemoryAllocation ? FC_ERR_OOM : FC_ERR_CUDA; \
        }                                                   \
    } while (0)

extern "C" void fc_set_last_cuda_error(cudaError_t e, const char *what, const char *file, int line);

namespace fc {
void set_error(const char *fmt, ...);  // thread-local message for fc_last_error_message
}
