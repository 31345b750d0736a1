// fc_noalloc.cu -- s-t connectivity for callers that must not allocate.
//
// fc_stcon_batch_noalloc answers a batch of s-t queries on a CSR the caller
// already holds in device memory, writing into output arrays the caller also
// provides, and calls no allocator at all: no cudaMalloc / cudaFree, no
// library routine that allocates.  It exists for code that cannot allocate
// device memory when it asks its queries -- for example a service that
// reserves all device memory up front for its own pool and forbids allocator
// calls afterwards (an allocation could fail, block on the device, or
// fragment the pool), or a plug-in that runs inside a host framework that
// owns the device memory.  The regular entry points grow workspaces with
// cudaMalloc on first use, so they do not fit those callers.
//
// The working memory of the queries (a status byte and a visit-log entry per
// vertex for each of NOALLOC_SLOTS CTAs) is one file-scope __device__ array of
// NOALLOC_BYTES (20 MiB).  Once the library's device code is loaded on a GPU,
// the array occupies that GPU's memory until the process exits.  Limits and
// rules:
//   * graphs of at most NOALLOC_MAX_NV (1,048,576) vertices; larger ones are
//     rejected with FC_ERR_INVALID;
//   * the array is shared by every call and keeps the previous call's
//     contents, so each call first re-initialises the part it uses; two calls
//     whose kernels overlap on the GPU (different streams, or threads racing)
//     race on the array and must be serialised by the caller;
//   * set-up happens in the first call on a device (and again if that
//     device's CUDA context was destroyed and re-created, e.g. after
//     cudaDeviceReset): with that device current it makes sure the library's
//     device code is loaded and looks up the array's device address with
//     cudaGetSymbolAddress.  Under lazy module loading (CUDA_MODULE_LOADING=
//     LAZY, the CUDA 12+ default) loading the code is what places the array
//     in device memory, so that first call may allocate: make it before the
//     caller reserves its device memory and before any stream capture begins
//     (or run with CUDA_MODULE_LOADING=EAGER).  Later calls allocate nothing;
//   * sched FC_SCHED_LEARNED runs as FC_SCHED_HEURISTIC here (the network's
//     weights live in memory the regular entry points allocate).
#include <cuda.h>  // driver types only: the entry points are fetched through the runtime

#include <mutex>

#include "fastcon.h"
#include "fc_sched.cuh"

namespace fc {
namespace {

constexpr int NOALLOC_MAX_NV = 1 << 20;
constexpr int NOALLOC_SLOTS = 4;
constexpr size_t NA_STATUS = (size_t)NOALLOC_MAX_NV;                   // bytes per slot
constexpr size_t NA_LOG = sizeof(int32_t) * (size_t)NOALLOC_MAX_NV;    // bytes per slot
constexpr size_t NA_SLOT = NA_STATUS + NA_LOG;
constexpr size_t NOALLOC_BYTES = NOALLOC_SLOTS * NA_SLOT;
static_assert(NA_STATUS % 256 == 0 && NA_SLOT % 256 == 0, "slot alignment");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

// One CTA per slot; each runs its share of the queries privately, top-down,
// with the same step code and scheduler as the other engines.
template <int T>
__global__ void __launch_bounds__(T) k_stcon_noalloc(GraphPair gp, const int32_t *qs,
                                                    const int32_t *qt, int nq, int32_t *conn,
                                                    int32_t *hops, int sched,
                                                    unsigned char *scratch)
{
    __shared__ SmemTopDown<T> sm;
    __shared__ QLocal ql;
    __shared__ TeamCounters tc;
    uint8_t *status = scratch + (size_t)blockIdx.x * NA_SLOT;
    int32_t *log = reinterpret_cast<int32_t *>(status + NA_STATUS);
    const int nv = gp.fwd.nv;
    // the array holds whatever the last call left: every vertex starts unvisited
    for (int i = threadIdx.x * 16; i < nv; i += T * 16)
        *reinterpret_cast<uint4 *>(status + i) = make_uint4(~0u, ~0u, ~0u, ~0u);
    __syncthreads();
    for (int q = blockIdx.x; q < nq; q += gridDim.x) {
        const int s = qs[q], t = qt[q];
        if (s < 0 || s >= nv || t < 0 || t >= nv) {
            if (threadIdx.x == 0) {
                conn[q] = 0;
                hops[q] = -2;
            }
            continue;
        }
        if (threadIdx.x == 0) {
            init_roots(MODE_STCON, gp, s, t, status, nullptr, log, nv, &tc);
            ql_start(ql, 1, nv, gp.fwd.ne, s, t, tc.deg[0], tc.deg[1]);
        }
        __syncthreads();
        while (true) {
            if (threadIdx.x == 0 && !ql.done) ql_decide(ql, sched, 0, LEVEL7_MAX);
            __syncthreads();
            if (ql.done) break;
            int F;
            const int x = ql.side;
            const int32_t *front = ql_frontier(ql, log, nv, x, &F);
            run_step<T>(MODE_STCON, gp, x, DIR_TD, ql.radius[x], ql.radius[1 - x], front, F, 0, 1,
                        status, nullptr, log, nv, &tc.tail[x], &tc.deg[x], &tc.found,
                        &tc.inspected, sm, ql.variant);
            __syncthreads();
            if (threadIdx.x == 0) ql_update(ql, tc.found, tc.tail[x], tc.deg[x], tc.inspected);
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            conn[q] = ql.connected;
            hops[q] = ql.hops;
        }
        const int n0 = ql.tail[0], n1 = ql.tail[1];
        for (int i = threadIdx.x; i < n0 + n1; i += T) {
            int v = i < n0 ? log[i] : log[nv - 1 - (i - n0)];
            status[v] = ST_UNVISITED;
        }
        __syncthreads();
    }
}

std::mutex g_setup_mu;
struct DeviceSetup {
    unsigned long long ctx_id;  // CUDA context the address belongs to (0: unknown)
    unsigned char *scratch;     // device address of g_noalloc_scratch
};
DeviceSetup g_setup[64];

typedef CUresult (*PfnCtxGetCurrent)(CUcontext *);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long *);

// Identifier of the current CUDA context (unique for the process's lifetime),
// or 0 when the driver cannot tell.  Driver entry points come through the
// runtime, so the library needs no link against the driver library.
unsigned long long current_context_id()
{
    static PfnCtxGetCurrent get_current = nullptr;
    static PfnCtxGetId get_id = nullptr;
    static bool resolved = false;
    if (!resolved) {
        resolved = true;
        cudaDriverEntryPointQueryResult q;
        void *f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<PfnCtxGetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<PfnCtxGetId>(f);
    }
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx ||
        get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

// Device address of the scratch array for the current device (the host-side
// symbol itself is not a device address).  Set-up runs on the first call on
// a device and again whenever that device's context has changed: it loads
// the module (cudaFuncGetAttributes), which also makes the context current,
// then looks the symbol up.
int scratch_for_device(int dev, unsigned char **out)
{
    std::lock_guard<std::mutex> lk(g_setup_mu);
    DeviceSetup &d = g_setup[dev];
    unsigned long long id = current_context_id();
    if (!d.scratch || id == 0 || id != d.ctx_id) {
        cudaFuncAttributes fa;
        cudaError_t e = cudaFuncGetAttributes(&fa, k_stcon_noalloc<FC_BLOCK>);
        if (e != cudaSuccess) {
            fc_set_last_cuda_error(e, "cudaFuncGetAttributes(k_stcon_noalloc)", __FILE__, __LINE__);
            return FC_ERR_CUDA;
        }
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            fc_set_last_cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
            return FC_ERR_CUDA;
        }
        d.scratch = static_cast<unsigned char *>(p);
        d.ctx_id = current_context_id();
    }
    *out = d.scratch;
    return FC_OK;
}

}  // namespace
}  // namespace fc

extern "C" int fc_stcon_batch_noalloc(const int32_t *d_row_ptr, const int32_t *d_col, int32_t nv,
                                      int64_t ne, const int32_t *d_rrow_ptr, const int32_t *d_rcol,
                                      const int32_t *d_s, const int32_t *d_t, int32_t nq,
                                      int32_t *d_connected, int32_t *d_hops, int32_t sched,
                                      void *stream)
{
    using namespace fc;
    if (nq < 0 || ne < 0) {
        set_error("fc_stcon_batch_noalloc: negative size");
        return FC_ERR_INVALID;
    }
    if (nv < 1 || nv > NOALLOC_MAX_NV) {
        set_error("fc_stcon_batch_noalloc: %d vertices; this entry point handles 1 to %d "
                  "(its working memory is a fixed %zu-byte device array)",
                  nv, NOALLOC_MAX_NV, NOALLOC_BYTES);
        return FC_ERR_INVALID;
    }
    if (sched != FC_SCHED_PLAIN && sched != FC_SCHED_HEURISTIC && sched != FC_SCHED_LEARNED) {
        set_error("fc_stcon_batch_noalloc: sched %d is not an FC_SCHED_* value", sched);
        return FC_ERR_INVALID;
    }
    if (nq == 0) return FC_OK;
    if (!d_row_ptr || (ne > 0 && !d_col) || !d_s || !d_t || !d_connected || !d_hops ||
        (!d_rrow_ptr) != (!d_rcol)) {
        set_error("fc_stcon_batch_noalloc: NULL array");
        return FC_ERR_INVALID;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        fc_set_last_cuda_error(e, "cudaGetDevice", __FILE__, __LINE__);
        return FC_ERR_NO_DEVICE;
    }
    if (dev < 0 || dev >= 64) return FC_ERR_UNSUPPORTED;
    unsigned char *scratch = nullptr;
    int rc = scratch_for_device(dev, &scratch);
    if (rc) return rc;
    GraphPair gp;
    gp.fwd.row_ptr = d_row_ptr;
    gp.fwd.col = d_col;
    gp.fwd.nv = nv;
    gp.fwd.pad_ = 0;
    gp.fwd.remap = nullptr;
    gp.fwd.ne = ne;
    gp.rev = gp.fwd;
    if (d_rrow_ptr) {
        gp.rev.row_ptr = d_rrow_ptr;
        gp.rev.col = d_rcol;
    }
    // the learned schedule needs weights from allocated memory: heuristic here
    const int run_sched = sched == FC_SCHED_LEARNED ? FC_SCHED_HEURISTIC : sched;
    k_stcon_noalloc<FC_BLOCK><<<NOALLOC_SLOTS, FC_BLOCK, 0, (cudaStream_t)stream>>>(
        gp, d_s, d_t, nq, d_connected, d_hops, run_sched, scratch);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        fc_set_last_cuda_error(e, "k_stcon_noalloc launch", __FILE__, __LINE__);
        return FC_ERR_CUDA;
    }
    return FC_OK;
}
