// fc_api.cu -- the extern "C" boundary (include/fastcon.h): graph handles,
// edge-list files, argument checks, dispatch to the engines.
#include <algorithm>
#include <cerrno>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "fastcon.h"
#include "fc_engine.h"
#include "fc_ingest.h"
#include "fc_internal.cuh"
#include "fc_parse.h"

struct fc_graph {
    int device;
    int32_t nv;
    int64_t ne;
    int directed;
    int32_t *row_ptr, *col;    // forward CSR
    int32_t *rrow_ptr, *rcol;  // reverse CSR (same pointers when undirected)
    // degree-ordered copy for the plain BFS engine: built on first use;
    // layout_state 0 = not decided, 1 = built, 2 = the graph keeps its numbering
    fc::BfsLayout *bfs_layout;
    int layout_state;
};

namespace {

using fc::set_error;

int validate_ptr(const void *p, const char *name)
{
    if (!p) {
        set_error("%s is NULL", name);
        return FC_ERR_INVALID;
    }
    return FC_OK;
}

fc::GraphPairH pair_of(const fc_graph *g)
{
    fc::GraphPairH p;
    p.fwd.row_ptr = g->row_ptr;
    p.fwd.col = g->col;
    p.fwd.nv = g->nv;
    p.fwd.pad_ = 0;
    p.fwd.ne = g->ne;
    p.fwd.remap = nullptr;
    p.rev.row_ptr = g->rrow_ptr;
    p.rev.col = g->rcol;
    p.rev.nv = g->nv;
    p.rev.pad_ = 0;
    p.rev.ne = g->ne;
    p.rev.remap = nullptr;
    return p;
}

// True when p points into page-locked host memory (cudaMallocHost,
// cudaHostRegister): only such memory may be copied inside a CUDA graph.
bool page_locked(const void *p)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();  // pageable memory of an older runtime: not an error
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

// The degree-ordered copy of g (vertices renumbered by descending degree
// class), built on first use and kept by the handle: order FC_ORDER_AUTO
// builds it only for graphs with hubs, FC_ORDER_DEGREE always, and
// FC_ORDER_GIVEN never.  The caller holds the device lock.
int ensure_layout(fc_graph *g, int order, cudaStream_t st)
{
    if (order == FC_ORDER_GIVEN) return FC_OK;
    if (g->layout_state == 0 || (g->layout_state == 2 && order == FC_ORDER_DEGREE)) {
        fc::BfsLayout *nl = nullptr;
        int rc = fc::bfs_layout_build(pair_of(g), &nl, st, order == FC_ORDER_AUTO);
        if (rc) return rc;
        g->bfs_layout = nl;
        g->layout_state = nl ? 1 : 2;
    }
    return FC_OK;
}

// The graph a search runs on.  An undirected graph with hubs is searched in
// its degree-ordered copy: the hubs' status bytes then share a few sectors of
// each query's status array, which stay in L2, instead of one sector per hub
// anywhere in it (R-MAT 24, a batch of 1,024 queries: 0.39 -> 0.26 ms), and
// each row lists its highest-degree neighbours first.  The kernels map s and t through the copy's id map; answers
// (connected, hop distance) do not depend on the numbering.  Directed graphs
// keep theirs (the copy holds no reverse CSR), and so does the host-loop
// engine, whose host side reads the ids.  by_default = 0 (a single s-t
// query) uses the copy only when asked (FC_ORDER_DEGREE): alone on the GPU
// its status array stays in L2 anyway, and on the copy the grid's claims
// crowd the few words that hold the hubs (R-MAT 24: 0.096 -> 0.106 ms per
// query); batches and full searches use it by default.  The caller holds
// the device lock.
int search_pair(fc_graph *g, const fc_opts &o, int by_default, cudaStream_t st,
                fc::GraphPairH *p)
{
    *p = pair_of(g);
    if (g->directed || o.engine == FC_ENGINE_HOSTLOOP) return FC_OK;
    if (!by_default && o.vertex_order != FC_ORDER_DEGREE) return FC_OK;
    int rc = ensure_layout(g, o.vertex_order, st);
    if (rc) return rc;
    if (o.vertex_order != FC_ORDER_GIVEN && g->bfs_layout) {
        fc::bfs_layout_graph(g->bfs_layout, &p->fwd);
        p->rev = p->fwd;
    }
    return FC_OK;
}

__global__ void k_csr_to_reverse_coo(const int32_t *row_ptr, const int32_t *col, int nv,
                                     int32_t *src, int32_t *dst)
{
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nv; u += gridDim.x * blockDim.x)
        for (int j = row_ptr[u]; j < row_ptr[u + 1]; ++j) {
            src[j] = col[j];
            dst[j] = u;
        }
}

// Reverse CSR of a directed graph, same multiset of edges.
int build_reverse(fc_graph *g, cudaStream_t st)
{
    int32_t *s = nullptr, *d = nullptr;
    FC_CUDA_TRY(cudaMalloc(&s, sizeof(int32_t) * (size_t)std::max<int64_t>(1, g->ne)));
    FC_CUDA_TRY(cudaMalloc(&d, sizeof(int32_t) * (size_t)std::max<int64_t>(1, g->ne)));
    int grid = (g->nv + 255) / 256;
    if (grid > 152 * 32) grid = 152 * 32;
    k_csr_to_reverse_coo<<<grid, 256, 0, st>>>(g->row_ptr, g->col, g->nv, s, d);
    long long ne2 = 0;
    int rc = fc::ingest_device_edges(
        s, d, g->ne, g->nv, FC_INGEST_DIRECTED | FC_INGEST_KEEP_LOOPS | FC_INGEST_KEEP_DUPS,
        &g->rrow_ptr, &g->rcol, &ne2, st);
    cudaFree(s);
    cudaFree(d);
    return rc;
}

fc_graph *new_graph(int nv, int directed)
{
    fc_graph *g = (fc_graph *)calloc(1, sizeof(fc_graph));
    if (!g) return nullptr;
    cudaGetDevice(&g->device);
    g->nv = nv;
    g->directed = directed;
    return g;
}

int finish_graph(fc_graph *g, cudaStream_t st)
{
    if (g->directed) {
        int rc = build_reverse(g, st);
        if (rc) return rc;
    } else {
        g->rrow_ptr = g->row_ptr;
        g->rcol = g->col;
    }
    return FC_OK;
}

int from_device_edges(const int32_t *d_src, const int32_t *d_dst, int64_t n, int32_t nv, int flags,
                      fc_graph **out, cudaStream_t st)
{
    fc_graph *g = new_graph(nv, (flags & FC_INGEST_DIRECTED) ? 1 : 0);
    if (!g) return FC_ERR_OOM;
    long long ne = 0;
    int rc = fc::ingest_device_edges(d_src, d_dst, n, nv, flags, &g->row_ptr, &g->col, &ne, st);
    if (rc == FC_OK) {
        g->ne = ne;
        rc = finish_graph(g, st);
    }
    if (rc != FC_OK) {
        fc_graph_free(g);
        return rc;
    }
    *out = g;
    return FC_OK;
}


struct CtxLock {
    fc::DevCtx *c = nullptr;
    int rc = FC_OK;
    std::unique_lock<std::mutex> lk;
    CtxLock()
    {
        c = fc::get_ctx(&rc);
        if (c) lk = std::unique_lock<std::mutex>(c->mu);
    }
};

cudaStream_t pick_stream(const fc_opts *o, fc::DevCtx *c)
{
    return (o && o->stream) ? (cudaStream_t)o->stream : c->stream;
}

fc_opts default_opts()
{
    fc_opts o;
    fc_opts_init(&o);
    return o;
}

}  // namespace

extern "C" {

void fc_opts_init(fc_opts *o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->sched = FC_SCHED_HEURISTIC;
    o->engine = FC_ENGINE_AUTO;
}

int fc_version(void) { return 100; }

const char *fc_strerror(int code)
{
    switch (code) {
    case FC_OK: return "ok";
    case FC_ERR_INVALID: return "invalid argument";
    case FC_ERR_CUDA: return "CUDA error";
    case FC_ERR_OOM: return "out of memory";
    case FC_ERR_IO: return "I/O error";
    case FC_ERR_FORMAT: return "malformed graph file";
    case FC_ERR_TIMEOUT: return "device-side wait timed out";
    case FC_ERR_OVERFLOW: return "graph exceeds int32 CSR limits";
    case FC_ERR_NO_DEVICE: return "no CUDA device";
    case FC_ERR_UNSUPPORTED: return "unsupported option";
    default: return "unknown error";
    }
}

int fc_device_info(int32_t *sm_count, int64_t *total_mem, int32_t *cc_major, int32_t *cc_minor)
{
    int dev = 0, n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return FC_ERR_NO_DEVICE;
    cudaGetDevice(&dev);
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) return FC_ERR_CUDA;
    if (sm_count) *sm_count = p.multiProcessorCount;
    if (total_mem) *total_mem = (int64_t)p.totalGlobalMem;
    if (cc_major) *cc_major = p.major;
    if (cc_minor) *cc_minor = p.minor;
    return FC_OK;
}

int fc_parse_edgelist(const char *path, int relabel, int nthreads, int32_t *src, int32_t *dst,
                      int64_t cap, int64_t *n, int32_t *nv, int32_t *file_directed)
{
    if (validate_ptr(path, "path") || validate_ptr(n, "n") || validate_ptr(nv, "nv") ||
        validate_ptr(file_directed, "file_directed"))
        return FC_ERR_INVALID;
    if (cap > 0 && (validate_ptr(src, "src") || validate_ptr(dst, "dst"))) return FC_ERR_INVALID;
    fc::Parsed P;
    int rc = fc::parse_edgelist_file(path, relabel, nthreads, P);
    if (rc) return rc;
    *n = (int64_t)P.src.size();
    *nv = (int32_t)P.nv;
    *file_directed = P.file_directed;
    if (cap < *n) {
        set_error("%lld pairs do not fit in %lld", (long long)*n, (long long)cap);
        return FC_ERR_OVERFLOW;
    }
    if (*n) {
        std::memcpy(src, P.src.data(), sizeof(int32_t) * (size_t)*n);
        std::memcpy(dst, P.dst.data(), sizeof(int32_t) * (size_t)*n);
    }
    return FC_OK;
}

int fc_graph_load_edgelist(const char *path, int force_dir, int relabel, fc_graph **g)
{
    if (validate_ptr(path, "path") || validate_ptr(g, "g")) return FC_ERR_INVALID;
    *g = nullptr;
    fc::Parsed P;
    int rc = fc::parse_edgelist_file(path, relabel, 0, P);
    if (rc) return rc;
    int directed = force_dir == 0 ? 1 : force_dir == 1 ? 0 : (P.file_directed == 1 ? 1 : 0);
    return fc_graph_from_edges(P.src.data(), P.dst.data(), (int64_t)P.src.size(), (int32_t)P.nv,
                               directed ? FC_INGEST_DIRECTED : 0, g);
}

int fc_graph_from_csr(const int32_t *row_ptr, int32_t nv, const int32_t *col, int64_t ne,
                      int directed, fc_graph **g)
{
    if (validate_ptr(row_ptr, "row_ptr") || validate_ptr(g, "g")) return FC_ERR_INVALID;
    if (ne > 0 && validate_ptr(col, "col")) return FC_ERR_INVALID;
    *g = nullptr;
    if (nv <= 0 || ne < 0 || ne > INT_MAX) {
        set_error("bad sizes nv=%d ne=%lld", nv, (long long)ne);
        return FC_ERR_INVALID;
    }
    if (row_ptr[0] != 0 || (int64_t)row_ptr[nv] != ne) {
        set_error("row_ptr must start at 0 and end at ne");
        return FC_ERR_INVALID;
    }
    for (int32_t i = 0; i < nv; ++i)
        if (row_ptr[i + 1] < row_ptr[i]) {
            set_error("row_ptr decreases at %d", i);
            return FC_ERR_INVALID;
        }
    for (int64_t j = 0; j < ne; ++j)
        if (col[j] < 0 || col[j] >= nv) {
            set_error("col[%lld] = %d out of range", (long long)j, col[j]);
            return FC_ERR_INVALID;
        }
    CtxLock L;
    if (!L.c) return L.rc;
    cudaStream_t st = L.c->stream;
    fc_graph *gg = new_graph(nv, directed ? 1 : 0);
    if (!gg) return FC_ERR_OOM;
    gg->ne = ne;
    int rc = FC_OK;
    if (cudaMalloc(&gg->row_ptr, sizeof(int32_t) * ((size_t)nv + 1)) != cudaSuccess ||
        cudaMalloc(&gg->col, sizeof(int32_t) * (size_t)std::max<int64_t>(1, ne) + 16) != cudaSuccess) {
        fc_graph_free(gg);
        set_error("cudaMalloc failed for the CSR");
        return FC_ERR_OOM;
    }
    if (cudaMemcpy(gg->row_ptr, row_ptr, sizeof(int32_t) * ((size_t)nv + 1), cudaMemcpyHostToDevice) != cudaSuccess ||
        (ne > 0 && cudaMemcpy(gg->col, col, sizeof(int32_t) * (size_t)ne, cudaMemcpyHostToDevice) != cudaSuccess)) {
        fc_graph_free(gg);
        set_error("copy of the CSR failed");
        return FC_ERR_CUDA;
    }
    // the copies above ran on the legacy stream; later kernels use others
    if (cudaDeviceSynchronize() != cudaSuccess) {
        fc_graph_free(gg);
        set_error("copy of the CSR failed");
        return FC_ERR_CUDA;
    }
    rc = finish_graph(gg, st);
    if (rc) {
        fc_graph_free(gg);
        return rc;
    }
    cudaStreamSynchronize(st);
    *g = gg;
    return FC_OK;
}

int fc_graph_from_edges(const int32_t *src, const int32_t *dst, int64_t n, int32_t nv, int flags,
                        fc_graph **g)
{
    if (validate_ptr(g, "g")) return FC_ERR_INVALID;
    if (n > 0 && (validate_ptr(src, "src") || validate_ptr(dst, "dst"))) return FC_ERR_INVALID;
    *g = nullptr;
    if (nv <= 0 || n < 0) {
        set_error("bad sizes nv=%d n=%lld", nv, (long long)n);
        return FC_ERR_INVALID;
    }
    CtxLock L;
    if (!L.c) return L.rc;
    cudaStream_t st = L.c->stream;
    int32_t *ds = nullptr, *dd = nullptr;
    size_t bytes = sizeof(int32_t) * (size_t)std::max<int64_t>(1, n);
    if (cudaMalloc(&ds, bytes) != cudaSuccess || cudaMalloc(&dd, bytes) != cudaSuccess) {
        cudaFree(ds);
        set_error("cudaMalloc failed for the edge list");
        return FC_ERR_OOM;
    }
    int rc = FC_OK;
    if (n > 0 && (cudaMemcpyAsync(ds, src, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
                  cudaMemcpyAsync(dd, dst, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st) != cudaSuccess))
        rc = FC_ERR_CUDA;
    if (rc == FC_OK) rc = from_device_edges(ds, dd, n, nv, flags, g, st);
    cudaStreamSynchronize(st);
    cudaFree(ds);
    cudaFree(dd);
    return rc;
}

int fc_graph_from_device_edges(const int32_t *d_src, const int32_t *d_dst, int64_t n, int32_t nv,
                               int flags, fc_graph **g)
{
    if (validate_ptr(g, "g")) return FC_ERR_INVALID;
    *g = nullptr;
    if (nv <= 0 || n < 0) return FC_ERR_INVALID;
    CtxLock L;
    if (!L.c) return L.rc;
    int rc = from_device_edges(d_src, d_dst, n, nv, flags, g, L.c->stream);
    cudaStreamSynchronize(L.c->stream);
    return rc;
}

int fc_graph_generate_rmat(int32_t scale, int64_t nedges, double a, double b, double c,
                           uint64_t seed, int64_t perm_seed, fc_graph **g)
{
    if (validate_ptr(g, "g")) return FC_ERR_INVALID;
    *g = nullptr;
    if (scale < 1 || scale > 30 || nedges < 0 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0) {
        set_error("bad R-MAT parameters");
        return FC_ERR_INVALID;
    }
    CtxLock L;
    if (!L.c) return L.rc;
    cudaStream_t st = L.c->stream;
    int32_t *ds = nullptr, *dd = nullptr;
    size_t bytes = sizeof(int32_t) * (size_t)std::max<int64_t>(1, nedges);
    if (cudaMalloc(&ds, bytes) != cudaSuccess || cudaMalloc(&dd, bytes) != cudaSuccess) {
        cudaFree(ds);
        set_error("cudaMalloc failed for the R-MAT edge list");
        return FC_ERR_OOM;
    }
    int rc = fc::gen_rmat_device(scale, nedges, a, b, c, seed, perm_seed, ds, dd, st);
    if (rc == FC_OK) rc = from_device_edges(ds, dd, nedges, 1 << scale, 0, g, st);
    cudaStreamSynchronize(st);
    cudaFree(ds);
    cudaFree(dd);
    return rc;
}

int fc_graph_generate_graph500(int32_t scale, int64_t nedges, uint64_t seed1, uint64_t seed2,
                               const double *initiator, fc_graph **g)
{
    if (validate_ptr(g, "g")) return FC_ERR_INVALID;
    *g = nullptr;
    static const double graph500_default[4] = {.57, .19, .19, .05};
    CtxLock L;
    if (!L.c) return L.rc;
    cudaStream_t st = L.c->stream;
    int32_t *ds = nullptr, *dd = nullptr;
    int rc = fc::gen_graph500_device(scale, nedges, seed1, seed2,
                                     initiator ? initiator : graph500_default, &ds, &dd, st);
    if (rc == FC_OK) rc = from_device_edges(ds, dd, nedges, 1 << scale, 0, g, st);
    cudaStreamSynchronize(st);
    cudaFree(ds);
    cudaFree(dd);
    return rc;
}

int fc_graph_generate_graph500_edges(int32_t scale, int64_t nedges, uint64_t seed1,
                                     uint64_t seed2, const double *initiator, int32_t *src,
                                     int32_t *dst)
{
    if (validate_ptr(src, "src") || validate_ptr(dst, "dst")) return FC_ERR_INVALID;
    static const double graph500_default[4] = {.57, .19, .19, .05};
    CtxLock L;
    if (!L.c) return L.rc;
    cudaStream_t st = L.c->stream;
    int32_t *ds = nullptr, *dd = nullptr;
    int rc = fc::gen_graph500_device(scale, nedges, seed1, seed2,
                                     initiator ? initiator : graph500_default, &ds, &dd, st);
    if (rc == FC_OK) {
        FC_CUDA_TRY(cudaMemcpy(src, ds, sizeof(int32_t) * (size_t)nedges, cudaMemcpyDeviceToHost));
        FC_CUDA_TRY(cudaMemcpy(dst, dd, sizeof(int32_t) * (size_t)nedges, cudaMemcpyDeviceToHost));
    }
    cudaFree(ds);
    cudaFree(dd);
    return rc;
}

int fc_graph_generate_grid(int32_t w, int32_t h, double p_del, uint64_t del_seed, int64_t shortcuts,
                           uint64_t sc_seed, fc_graph **g)
{
    if (validate_ptr(g, "g")) return FC_ERR_INVALID;
    *g = nullptr;
    if (w < 2 || h < 2 || (long long)w * h > INT_MAX || p_del < 0 || p_del > 1 || shortcuts < 0) {
        set_error("bad grid parameters");
        return FC_ERR_INVALID;
    }
    CtxLock L;
    if (!L.c) return L.rc;
    cudaStream_t st = L.c->stream;
    long long slots = fc::grid_edge_slots(w, h, shortcuts);
    int32_t *ds = nullptr, *dd = nullptr;
    size_t bytes = sizeof(int32_t) * (size_t)std::max<long long>(1, slots);
    if (cudaMalloc(&ds, bytes) != cudaSuccess || cudaMalloc(&dd, bytes) != cudaSuccess) {
        cudaFree(ds);
        set_error("cudaMalloc failed for the grid edge list");
        return FC_ERR_OOM;
    }
    int rc = fc::gen_grid_device(w, h, p_del, del_seed, shortcuts, sc_seed, ds, dd, st);
    if (rc == FC_OK) rc = from_device_edges(ds, dd, slots, w * h, 0, g, st);
    cudaStreamSynchronize(st);
    cudaFree(ds);
    cudaFree(dd);
    return rc;
}

int fc_graph_info(const fc_graph *g, int32_t *nv, int64_t *ne, int32_t *directed)
{
    if (validate_ptr(g, "g")) return FC_ERR_INVALID;
    if (nv) *nv = g->nv;
    if (ne) *ne = g->ne;
    if (directed) *directed = g->directed;
    return FC_OK;
}

int fc_graph_get_csr(const fc_graph *g, int32_t *row_ptr, int32_t *col)
{
    if (validate_ptr(g, "g")) return FC_ERR_INVALID;
    if (row_ptr)
        FC_CUDA_TRY(cudaMemcpy(row_ptr, g->row_ptr, sizeof(int32_t) * ((size_t)g->nv + 1),
                               cudaMemcpyDeviceToHost));
    if (col && g->ne > 0)
        FC_CUDA_TRY(cudaMemcpy(col, g->col, sizeof(int32_t) * (size_t)g->ne, cudaMemcpyDeviceToHost));
    return FC_OK;
}

void fc_graph_free(fc_graph *g)
{
    if (!g) return;
    fc::bfs_layout_free(g->bfs_layout);
    if (g->rrow_ptr && g->rrow_ptr != g->row_ptr) cudaFree(g->rrow_ptr);
    if (g->rcol && g->rcol != g->col) cudaFree(g->rcol);
    cudaFree(g->row_ptr);
    cudaFree(g->col);
    free(g);
}

int fc_bfs_levels_ex(fc_graph *g, int32_t s, int32_t *levels, const fc_opts *opts, fc_stats *stats)
{
    if (validate_ptr(g, "g")) return FC_ERR_INVALID;
    if (s < 0 || s >= g->nv) {
        set_error("source %d outside [0, %d)", s, g->nv);
        return FC_ERR_INVALID;
    }
    fc_opts o = opts ? *opts : default_opts();
    CtxLock L;
    if (!L.c) return L.rc;
    if (o.engine == FC_ENGINE_AUTO && o.sched == FC_SCHED_PLAIN) {
        // the visited-bitmap engine; degree-ordered numbering unless the
        // caller asks for the graph's own, or (auto) the graph has no hubs
        const fc::BfsLayout *lay = nullptr;
        if (o.vertex_order != FC_ORDER_GIVEN) {
            int rc = ensure_layout(g, o.vertex_order, pick_stream(opts, L.c));
            if (rc) return rc;
            lay = g->bfs_layout;
        }
        return fc::engine_bfs_plain(L.c, pair_of(g), lay, s, levels, o, stats,
                                    pick_stream(opts, L.c));
    }
    // the other schedules search the degree-ordered copy like batches do
    // (R-MAT 24, direction-optimising: about 1.5 -> 1.1 ms); the levels come
    // back in the caller's numbering
    fc::GraphPairH p;
    int rc = search_pair(g, o, 1, pick_stream(opts, L.c), &p);
    if (rc) return rc;
    return fc::engine_bfs(L.c, p, s, levels, o, stats, pick_stream(opts, L.c));
}

int fc_bfs_trace(int32_t *nlevels, int64_t *level_ns, int64_t *frontier, int64_t *entries,
                 int32_t cap)
{
    if (validate_ptr(nlevels, "nlevels")) return FC_ERR_INVALID;
    CtxLock L;
    if (!L.c) return L.rc;
    return fc::engine_bfs_trace(L.c, nlevels, level_ns, frontier, entries, cap);
}

int fc_bfs_levels(fc_graph *g, int32_t s, int32_t *levels)
{
    if (validate_ptr(levels, "levels")) return FC_ERR_INVALID;
    return fc_bfs_levels_ex(g, s, levels, nullptr, nullptr);
}

int fc_stcon_ex(fc_graph *g, int32_t s, int32_t t, int32_t *connected, int32_t *hops,
                const fc_opts *opts, fc_stats *stats)
{
    if (validate_ptr(g, "g") || validate_ptr(connected, "connected") || validate_ptr(hops, "hops"))
        return FC_ERR_INVALID;
    if (s < 0 || s >= g->nv || t < 0 || t >= g->nv) {
        set_error("query (%d, %d) outside [0, %d)", s, t, g->nv);
        return FC_ERR_INVALID;
    }
    fc_opts o = opts ? *opts : default_opts();
    CtxLock L;
    if (!L.c) return L.rc;
    fc::GraphPairH p;
    int rc = search_pair(g, o, 0, pick_stream(opts, L.c), &p);
    if (rc) return rc;
    return fc::engine_stcon(L.c, p, s, t, connected, hops, o, stats, pick_stream(opts, L.c));
}

int fc_stcon(fc_graph *g, int32_t s, int32_t t, int32_t *connected, int32_t *hops)
{
    return fc_stcon_ex(g, s, t, connected, hops, nullptr, nullptr);
}

int fc_stcon_depth(fc_graph *g, int32_t s, int32_t t, int32_t *depth)
{
    if (validate_ptr(depth, "depth")) return FC_ERR_INVALID;
    int32_t c = 0, h = -1;
    int rc = fc_stcon(g, s, t, &c, &h);
    if (rc) return rc;
    *depth = c ? (h + 1) / 2 : -1;
    return FC_OK;
}

int fc_stcon_batch_device(fc_graph *const *gs, int32_t ngraphs, const int32_t *d_graph_idx,
                          const int32_t *d_s, const int32_t *d_t, int32_t nq, int32_t *d_connected,
                          int32_t *d_hops, const fc_opts *opts, fc_stats *stats)
{
    if (validate_ptr(gs, "gs")) return FC_ERR_INVALID;
    if (nq < 0 || ngraphs < 1) return FC_ERR_INVALID;
    if (nq == 0) return FC_OK;
    if (validate_ptr(d_s, "s") || validate_ptr(d_t, "t") || validate_ptr(d_connected, "connected") ||
        validate_ptr(d_hops, "hops"))
        return FC_ERR_INVALID;
    for (int i = 0; i < ngraphs; ++i)
        if (!gs[i]) return FC_ERR_INVALID;
    fc_opts o = opts ? *opts : default_opts();
    CtxLock L;
    if (!L.c) return L.rc;
    std::vector<fc::GraphPairH> pairs((size_t)ngraphs);
    for (int i = 0; i < ngraphs; ++i) {
        int rc = search_pair(gs[i], o, 1, pick_stream(opts, L.c), &pairs[(size_t)i]);
        if (rc) return rc;
    }
    return fc::engine_stcon_batch(L.c, pairs.data(), ngraphs, d_graph_idx, d_s, d_t, nq, d_connected,
                                  d_hops, o, stats, pick_stream(opts, L.c), stats != nullptr);
}

// Autotuner: every candidate runs the caller's sample batch `reps` times
// after one warm-up run; the median kernel time picks the winner.  The
// candidates are the knobs the batched engine measured sensitive to on
// R-MAT and grid workloads: resident owner CTAs per SM, the private-step
// threshold and the shared tile size.
int fc_autotune_batch(fc_graph *const *gs, int32_t ngraphs, const int32_t *d_graph_idx,
                      const int32_t *d_s, const int32_t *d_t, int32_t nq, int32_t reps,
                      fc_opts *inout, double *best_ms)
{
    if (validate_ptr(gs, "gs") || validate_ptr(d_s, "s") || validate_ptr(d_t, "t") ||
        validate_ptr(inout, "opts"))
        return FC_ERR_INVALID;
    if (nq <= 0 || ngraphs < 1 || reps < 1 || reps > 100) {
        set_error("autotune: nq %d, ngraphs %d, reps %d", nq, ngraphs, reps);
        return FC_ERR_INVALID;
    }
    for (int i = 0; i < ngraphs; ++i)
        if (!gs[i]) return FC_ERR_INVALID;
    CtxLock L;
    if (!L.c) return L.rc;
    cudaStream_t st = pick_stream(inout, L.c);
    std::vector<fc::GraphPairH> pairs((size_t)ngraphs);
    {
        fc_opts ob = *inout;
        ob.engine = FC_ENGINE_BATCHED;
        for (int i = 0; i < ngraphs; ++i) {
            int rc = search_pair(gs[i], ob, 1, st, &pairs[(size_t)i]);
            if (rc) return rc;
        }
    }
    int32_t *dc = nullptr;
    FC_CUDA_TRY(cudaMallocAsync(&dc, sizeof(int32_t) * 2 * (size_t)nq, st));
    const int ctas[] = {2, 3, 4};
    const int workk[] = {2, 4, 8};
    const int tiles[] = {4096, 8192, 16384};
    fc_opts best = *inout;
    double best_t = -1;
    int rc = FC_OK;
    for (int a : ctas)
        for (int w : workk)
            for (int te : tiles) {
                fc_opts o = *inout;
                o.engine = FC_ENGINE_BATCHED;
                o.use_graph = 0;
                o.ctas_per_sm = a;
                o.cta_work_k = w;
                o.tile_entries = te;
                std::vector<double> ts;
                for (int r = 0; r <= reps && rc == FC_OK; ++r) {
                    fc_stats s;
                    rc = fc::engine_stcon_batch(L.c, pairs.data(), ngraphs, d_graph_idx, d_s, d_t,
                                                nq, dc, dc + nq, o, &s, st, true);
                    if (r) ts.push_back(s.kernel_ms[0] + s.kernel_ms[1]);
                }
                if (rc) break;
                std::sort(ts.begin(), ts.end());
                const double med = ts[ts.size() / 2];
                if (best_t < 0 || med < best_t) {
                    best_t = med;
                    best = o;
                }
            }
    cudaFreeAsync(dc, st);
    cudaStreamSynchronize(st);
    if (rc) return rc;
    best.use_graph = inout->use_graph;
    *inout = best;
    if (best_ms) *best_ms = best_t;
    return FC_OK;
}

int fc_stcon_batch_scripted(fc_graph *g, const int32_t *d_s, const int32_t *d_t, int32_t nq,
                            const uint8_t *d_script, int32_t script_len, const fc_opts *opts,
                            int32_t *d_hops, int64_t *d_inspected, int32_t *d_trace,
                            int32_t trace_cap, int32_t *d_trace_count)
{
    if (validate_ptr(g, "g") || validate_ptr(d_s, "s") || validate_ptr(d_t, "t") ||
        validate_ptr(d_hops, "hops"))
        return FC_ERR_INVALID;
    if (nq < 0 || script_len < 0 || (d_script && script_len == 0) || (d_trace && !d_trace_count) ||
        trace_cap < 0)
        return FC_ERR_INVALID;
    if (nq == 0) return FC_OK;
    fc_opts o = opts ? *opts : default_opts();
    o.engine = FC_ENGINE_BATCHED;
    CtxLock L;
    if (!L.c) return L.rc;
    cudaStream_t st = pick_stream(opts, L.c);
    int32_t *dc = nullptr;
    FC_CUDA_TRY(cudaMallocAsync(&dc, sizeof(int32_t) * (size_t)nq, st));
    if (d_trace_count) FC_CUDA_TRY(cudaMemsetAsync(d_trace_count, 0, sizeof(int32_t), st));
    fc::BatchExtras ex;
    ex.script = d_script;
    ex.script_len = d_script ? script_len : 0;
    ex.trace = d_trace;
    ex.trace_cap = trace_cap;
    ex.trace_count = d_trace_count;
    ex.inspected = reinterpret_cast<long long *>(d_inspected);
    fc::GraphPairH p;
    int rc = search_pair(g, o, 1, st, &p);
    if (rc) {
        cudaFreeAsync(dc, st);
        return rc;
    }
    rc = fc::engine_stcon_batch(L.c, &p, 1, nullptr, d_s, d_t, nq, dc, d_hops, o, nullptr, st,
                                true, &ex);
    cudaFreeAsync(dc, st);
    cudaStreamSynchronize(st);
    return rc;
}

int fc_bfs_parents(fc_graph *g, int32_t s, int32_t *parents, int32_t *levels)
{
    if (validate_ptr(g, "g") || validate_ptr(parents, "parents")) return FC_ERR_INVALID;
    if (s < 0 || s >= g->nv) {
        set_error("source %d outside [0, %d)", s, g->nv);
        return FC_ERR_INVALID;
    }
    CtxLock L;
    if (!L.c) return L.rc;
    return fc::engine_bfs_parents(L.c, pair_of(g), s, parents, levels, default_opts(), L.c->stream);
}

int fc_stcon_path(fc_graph *g, int32_t s, int32_t t, int32_t *path, int32_t cap, int32_t *len)
{
    if (validate_ptr(g, "g") || validate_ptr(len, "len") || (cap > 0 && validate_ptr(path, "path")))
        return FC_ERR_INVALID;
    if (cap < 0 || s < 0 || s >= g->nv || t < 0 || t >= g->nv) {
        set_error("query (%d, %d) outside [0, %d) or cap %d < 0", s, t, g->nv, cap);
        return FC_ERR_INVALID;
    }
    CtxLock L;
    if (!L.c) return L.rc;
    return fc::engine_stcon_path(L.c, pair_of(g), s, t, path, cap, len, default_opts(), L.c->stream);
}

int fc_validate_bfs(fc_graph *g, int32_t root, const int32_t *parents, int64_t *errors)
{
    if (validate_ptr(g, "g") || validate_ptr(parents, "parents") || validate_ptr(errors, "errors"))
        return FC_ERR_INVALID;
    if (root < 0 || root >= g->nv) {
        set_error("root %d outside [0, %d)", root, g->nv);
        return FC_ERR_INVALID;
    }
    CtxLock L;
    if (!L.c) return L.rc;
    return fc::engine_validate_bfs(L.c, pair_of(g), g->directed, root, parents, errors, L.c->stream);
}

int fc_stcon_multiseed(fc_graph *g, int32_t s, int32_t t, int32_t nseeds, uint64_t seed,
                       int32_t *connected, fc_stats *stats)
{
    if (validate_ptr(g, "g") || validate_ptr(connected, "connected")) return FC_ERR_INVALID;
    if (s < 0 || s >= g->nv || t < 0 || t >= g->nv) {
        set_error("query (%d, %d) outside [0, %d)", s, t, g->nv);
        return FC_ERR_INVALID;
    }
    if (g->directed) {
        set_error("multi-seed connectivity needs an undirected graph");
        return FC_ERR_UNSUPPORTED;
    }
    CtxLock L;
    if (!L.c) return L.rc;
    return fc::engine_stcon_multiseed(L.c, pair_of(g), s, t, nseeds, seed, connected, stats,
                                      L.c->stream);
}

int fc_selftest_primitives(int32_t which, const int32_t *in, int32_t n, int32_t *out,
                           int32_t *aux)
{
    if (which < 0 || which > 3 || n < 0 || (n > 0 && (!in || !out))) {
        set_error("fc_selftest_primitives: which %d, n %d", which, n);
        return FC_ERR_INVALID;
    }
    if (which == 3)
        for (int32_t i = 0; i < n; ++i)
            if (in[i] < -1) {
                set_error("fc_selftest_primitives: value %d below -1", in[i]);
                return FC_ERR_INVALID;
            }
    if (which == 2)
        for (int32_t i = 0; i < n; ++i)
            if (in[i] < 0) {
                set_error("fc_selftest_primitives: negative row length");
                return FC_ERR_INVALID;
            }
    if (n == 0) return FC_OK;
    CtxLock L;
    if (!L.c) return L.rc;
    return fc::engine_selftest_primitives(L.c, which, in, n, out, aux, L.c->stream);
}

int fc_selftest_wait(int32_t timeout_ms, double *elapsed_ms)
{
    if (timeout_ms < 1 || timeout_ms > 2000) {
        set_error("timeout_ms %d outside [1, 2000]", timeout_ms);
        return FC_ERR_INVALID;
    }
    CtxLock L;
    if (!L.c) return L.rc;
    return fc::engine_selftest_wait(L.c, timeout_ms, elapsed_ms, L.c->stream);
}

int fc_stcon_batch(fc_graph *const *gs, int32_t ngraphs, const int32_t *graph_idx, const int32_t *s,
                   const int32_t *t, int32_t nq, int32_t *connected, int32_t *hops,
                   const fc_opts *opts, fc_stats *stats)
{
    if (validate_ptr(gs, "gs")) return FC_ERR_INVALID;
    if (nq < 0 || ngraphs < 1) return FC_ERR_INVALID;
    if (nq == 0) return FC_OK;
    if (validate_ptr(s, "s") || validate_ptr(t, "t") || validate_ptr(connected, "connected") ||
        validate_ptr(hops, "hops"))
        return FC_ERR_INVALID;
    for (int i = 0; i < ngraphs; ++i)
        if (!gs[i]) return FC_ERR_INVALID;
    for (int32_t i = 0; i < nq; ++i) {
        int gi = graph_idx ? graph_idx[i] : 0;
        if (gi < 0 || gi >= ngraphs) {
            set_error("graph_idx[%d] = %d outside [0, %d)", i, gi, ngraphs);
            return FC_ERR_INVALID;
        }
        if (s[i] < 0 || s[i] >= gs[gi]->nv || t[i] < 0 || t[i] >= gs[gi]->nv) {
            set_error("query %d (%d, %d) outside [0, %d)", i, s[i], t[i], gs[gi]->nv);
            return FC_ERR_INVALID;
        }
    }
    CtxLock L;
    if (!L.c) return L.rc;
    cudaStream_t st = pick_stream(opts, L.c);
    int rc = FC_OK;
    size_t k = (size_t)nq;
    int32_t *buf = fc::batch_staging(L.c, k, &rc);
    if (!buf) return rc;
    int32_t *ds = buf, *dt = buf + k, *dg = buf + 2 * k, *dc = buf + 3 * k, *dh = buf + 4 * k;
    fc_opts o = opts ? *opts : default_opts();
    std::vector<fc::GraphPairH> pairs((size_t)ngraphs);
    for (int i = 0; i < ngraphs; ++i) {
        rc = search_pair(gs[i], o, 1, st, &pairs[(size_t)i]);
        if (rc) return rc;
    }
    // Page-locked arrays on the batched engine: the engine queues the copies
    // in and out with its kernels (in its CUDA graph when opts.use_graph is
    // set).  Otherwise the copies are queued here.  Either way the answers'
    // copies and the engine's error words travel together and the call
    // waits once.
    const bool batched = o.engine == FC_ENGINE_AUTO || o.engine == FC_ENGINE_BATCHED;
    const bool locked = batched && page_locked(s) && page_locked(t) &&
                        (!graph_idx || page_locked(graph_idx)) && page_locked(connected) &&
                        page_locked(hops);
    if (locked) {
        const fc::BatchHostIO hio{s, t, graph_idx, connected, hops};
        rc = fc::engine_stcon_batch(L.c, pairs.data(), ngraphs, graph_idx ? dg : nullptr, ds, dt,
                                    nq, dc, dh, o, stats, st, fc::BATCH_DEFER_CHECK, nullptr, &hio);
    } else {
        FC_CUDA_TRY(cudaMemcpyAsync(ds, s, sizeof(int32_t) * k, cudaMemcpyHostToDevice, st));
        FC_CUDA_TRY(cudaMemcpyAsync(dt, t, sizeof(int32_t) * k, cudaMemcpyHostToDevice, st));
        if (graph_idx)
            FC_CUDA_TRY(cudaMemcpyAsync(dg, graph_idx, sizeof(int32_t) * k, cudaMemcpyHostToDevice, st));
        rc = fc::engine_stcon_batch(L.c, pairs.data(), ngraphs, graph_idx ? dg : nullptr, ds, dt,
                                    nq, dc, dh, o, stats, st, fc::BATCH_DEFER_CHECK);
        if (rc == FC_OK) {
            FC_CUDA_TRY(cudaMemcpyAsync(connected, dc, sizeof(int32_t) * k, cudaMemcpyDeviceToHost, st));
            FC_CUDA_TRY(cudaMemcpyAsync(hops, dh, sizeof(int32_t) * k, cudaMemcpyDeviceToHost, st));
        }
    }
    // the staging buffer is reused by the next call
    cudaStreamSynchronize(st);
    const int crc = fc::engine_finish_checks(L.c);
    return rc != FC_OK ? rc : crc;
}

}  // extern "C"
