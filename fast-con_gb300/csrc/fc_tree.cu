// fc_tree.cu -- what comes after the traversal: BFS trees (predecessor maps),
// shortest s-t paths, and a GPU validation of predecessor maps.
//
// Parents.  parents[v] is the smallest-id in-neighbour u of v with
// level(u) = level(v) - 1 (rows are sorted, so it is the first hit of a
// row scan); parents[s] = s and -1 where v is unreachable.  The reference's
// predecessor arrays (h_pred, S/make_stcon.c:1189-1455) hold whichever
// vertex claimed v first; this choice is deterministic instead.
//
// Path.  The s-t path is the parent chain from t back to s, so its vertices
// are fixed by the same rule and its length is hops + 1.
//
// Validation restates validate_bfs_result (S/reference_functions.c:99-434)
// for one GPU, with the depth map computed by pointer jumping instead of the
// reference's MPI exchange of depths:
//   [0] the root's parent is not the root
//   [1] a non-root vertex is its own parent, or a parent is out of range
//   [2] no graph edge from a vertex's parent to the vertex
//   [3] the parent chain of a vertex does not reach the root (a cycle, or a
//       chain through a vertex outside the tree)
//   [4] an edge leads from a tree vertex to a vertex outside the tree
//   [5] an edge's endpoint depths are too far apart (|d(u) - d(v)| > 1; on a
//       directed graph d(v) > d(u) + 1 for an edge u -> v)
//   [6] vertices in the tree (a count, not an error: the reference compares
//       it with the traversal's visit count)
#include <climits>
#include <cstring>

#include "fc_engine.h"
#include "fc_sched.cuh"

namespace fc {

constexpr int TREE_BLOCK = 256;
constexpr int NOT_IN_TREE = -1;
constexpr int BAD_PARENT = -2;

// parents from a level array; `in` is the in-neighbour CSR (the reverse
// graph; the graph itself when undirected)
__global__ void k_parents(DGraph in, const int32_t *__restrict__ lev, int32_t *par, int s)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < in.nv; v += gridDim.x * blockDim.x) {
        const int l = lev[v];
        int p = -1;
        if (v == s) {
            p = s;
        } else if (l > 0) {
            const int b = in.row_ptr[v], e = in.row_ptr[v + 1];
            for (int j = b; j < e && p < 0; j += 4) {
                int u[4], lu[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) u[k] = j + k < e ? __ldg(in.col + j + k) : -1;
#pragma unroll
                for (int k = 0; k < 4; ++k) lu[k] = u[k] >= 0 ? __ldg(lev + u[k]) : -2;
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (p < 0 && lu[k] == l - 1) p = u[k];
            }
        }
        par[v] = p;
    }
}

// one thread follows the parent chain from t: path[len-1] = t ... path[0] = s
__global__ void k_walk(const int32_t *par, int t, int32_t *path, int len)
{
    if (blockIdx.x || threadIdx.x) return;
    int cur = t;
    for (int i = len - 1; i >= 0 && cur >= 0; --i) {
        path[i] = cur;
        cur = par[cur];
    }
}

__global__ void k_val_init(const int32_t *par, int nv, int root, int32_t *anc, int32_t *dist,
                           unsigned long long *err)
{
    unsigned long long e0 = 0, e1 = 0, in_tree = 0;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
        const int p = par[v];
        int a = NOT_IN_TREE, d = 0;
        if (v == root) {
            if (p != root) ++e0;
            a = root;
            ++in_tree;
        } else if (p == -1) {
            a = NOT_IN_TREE;
        } else if (p < 0 || p >= nv || p == v) {
            ++e1;
            a = BAD_PARENT;
            ++in_tree;
        } else {
            a = p;
            d = 1;
            ++in_tree;
        }
        anc[v] = a;
        dist[v] = d;
    }
    if (e0) atomicAdd(err + 0, e0);
    if (e1) atomicAdd(err + 1, e1);
    if (in_tree) atomicAdd(err + 6, in_tree);
}

// an edge from each vertex's parent to the vertex: binary search of the
// parent in the vertex's sorted in-row
__global__ void k_val_parent_edge(DGraph in, const int32_t *par, int root,
                                  unsigned long long *err)
{
    unsigned long long e2 = 0;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < in.nv; v += gridDim.x * blockDim.x) {
        const int p = par[v];
        if (v == root || p < 0 || p >= in.nv || p == v) continue;
        int lo = in.row_ptr[v], hi = in.row_ptr[v + 1];
        while (lo < hi) {
            const int mid = lo + (hi - lo) / 2;
            if (in.col[mid] < p)
                lo = mid + 1;
            else
                hi = mid;
        }
        if (lo >= in.row_ptr[v + 1] || in.col[lo] != p) ++e2;
    }
    if (e2) atomicAdd(err + 2, e2);
}

// one pointer-jumping round: dist grows by the ancestor's distance and the
// ancestor jumps to its own ancestor; the root is its own fixed point
__global__ void k_val_jump(const int32_t *anc_in, const int32_t *dist_in, int32_t *anc_out,
                           int32_t *dist_out, int nv, int root)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
        int a = anc_in[v], d = dist_in[v];
        if (a >= 0 && a != root) {
            const int a2 = anc_in[a];
            if (a2 == NOT_IN_TREE || a2 == BAD_PARENT) {
                a = BAD_PARENT;  // the chain runs through a vertex outside the tree
            } else {
                d += dist_in[a];
                a = a2;
            }
        }
        anc_out[v] = a;
        dist_out[v] = d;
    }
}

__global__ void k_val_depth(const int32_t *anc, int32_t *dist, int nv, int root,
                            unsigned long long *err)
{
    unsigned long long e3 = 0;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
        const int a = anc[v];
        if (a == root) continue;
        if (a != NOT_IN_TREE) ++e3;
        dist[v] = INT_MAX;  // outside the tree, or not connected to the root
    }
    if (e3) atomicAdd(err + 3, e3);
}

__global__ void k_val_edges(DGraph out, const int32_t *__restrict__ depth, int directed,
                            unsigned long long *err)
{
    unsigned long long e4 = 0, e5 = 0;
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < out.nv; u += gridDim.x * blockDim.x) {
        const int du = depth[u];
        if (du == INT_MAX) continue;
        for (int j = out.row_ptr[u]; j < out.row_ptr[u + 1]; ++j) {
            const int dv = __ldg(depth + __ldg(out.col + j));
            if (dv == INT_MAX)
                ++e4;
            else if (directed ? dv > du + 1 : (dv - du > 1 || du - dv > 1))
                ++e5;
        }
    }
    if (e4) atomicAdd(err + 4, e4);
    if (e5) atomicAdd(err + 5, e5);
}

static int tree_grid(DevCtx *c) { return c->sm_count * 8; }

int engine_bfs_parents(DevCtx *c, const GraphPairH &gp, int32_t s, int32_t *h_parents,
                       int32_t *h_levels, const fc_opts &o, cudaStream_t st)
{
    int rc = engine_bfs(c, gp, s, h_levels, o, nullptr, st);
    if (rc) return rc;
    // the visit log is free once the traversal is done: it holds the parents
    DGraph in;
    std::memcpy(&in, &gp.rev, sizeof(in));
    k_parents<<<tree_grid(c), TREE_BLOCK, 0, st>>>(in, c->levels, c->log, s);
    FC_CUDA_TRY(cudaGetLastError());
    FC_CUDA_TRY(cudaMemcpyAsync(h_parents, c->log, sizeof(int32_t) * (size_t)gp.fwd.nv,
                                cudaMemcpyDeviceToHost, st));
    FC_CUDA_TRY(cudaStreamSynchronize(st));
    return FC_OK;
}

int engine_stcon_path(DevCtx *c, const GraphPairH &gp, int32_t s, int32_t t, int32_t *h_path,
                      int32_t cap, int32_t *len, const fc_opts &o, cudaStream_t st)
{
    int rc = engine_bfs(c, gp, s, nullptr, o, nullptr, st);
    if (rc) return rc;
    int32_t lt = -1;
    FC_CUDA_TRY(cudaMemcpyAsync(&lt, c->levels + t, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    FC_CUDA_TRY(cudaStreamSynchronize(st));
    if (lt < 0) {
        *len = 0;
        return FC_OK;
    }
    const int n = lt + 1;
    *len = n;
    if (n > cap) {
        set_error("path of %d vertices does not fit in %d", n, cap);
        return FC_ERR_OVERFLOW;
    }
    DGraph in;
    std::memcpy(&in, &gp.rev, sizeof(in));
    k_parents<<<tree_grid(c), TREE_BLOCK, 0, st>>>(in, c->levels, c->log, s);
    FC_CUDA_TRY(cudaGetLastError());
    // the path goes into the level array, no longer needed
    k_walk<<<1, 1, 0, st>>>(c->log, t, c->levels, n);
    FC_CUDA_TRY(cudaGetLastError());
    FC_CUDA_TRY(cudaMemcpyAsync(h_path, c->levels, sizeof(int32_t) * (size_t)n,
                                cudaMemcpyDeviceToHost, st));
    FC_CUDA_TRY(cudaStreamSynchronize(st));
    return FC_OK;
}

int engine_validate_bfs(DevCtx *c, const GraphPairH &gp, int directed, int32_t root,
                        const int32_t *h_parents, int64_t *errors, cudaStream_t st)
{
    const int nv = gp.fwd.nv;
    const size_t n = (size_t)nv;
    int32_t *buf = nullptr;
    unsigned long long *err = nullptr;
    FC_CUDA_TRY(cudaMallocAsync(&buf, sizeof(int32_t) * 5 * n, st));
    cudaError_t e = cudaMallocAsync(&err, sizeof(unsigned long long) * 8, st);
    if (e != cudaSuccess) {
        cudaFreeAsync(buf, st);
        FC_CUDA_TRY(e);
    }
    int32_t *par = buf, *anc0 = buf + n, *dist0 = buf + 2 * n, *anc1 = buf + 3 * n,
            *dist1 = buf + 4 * n;
    DGraph in, out;
    std::memcpy(&in, &gp.rev, sizeof(in));
    std::memcpy(&out, &gp.fwd, sizeof(out));
    const int G = tree_grid(c);
    int rc = FC_OK;
    do {
        cudaError_t ce;
        if ((ce = cudaMemcpyAsync(par, h_parents, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st)) ||
            (ce = cudaMemsetAsync(err, 0, sizeof(unsigned long long) * 8, st))) {
            fc_set_last_cuda_error(ce, "validation set-up", __FILE__, __LINE__);
            rc = FC_ERR_CUDA;
            break;
        }
        k_val_init<<<G, TREE_BLOCK, 0, st>>>(par, nv, root, anc0, dist0, err);
        k_val_parent_edge<<<G, TREE_BLOCK, 0, st>>>(in, par, root, err);
        // ceil(log2(nv)) + 1 rounds take every chain that reaches the root
        // there; an odd number of rounds leaves the result in the second set
        int rounds = 1;
        while ((1ll << rounds) < (long long)nv + 1) ++rounds;
        ++rounds;
        for (int r = 0; r < rounds; ++r) {
            if (r & 1)
                k_val_jump<<<G, TREE_BLOCK, 0, st>>>(anc1, dist1, anc0, dist0, nv, root);
            else
                k_val_jump<<<G, TREE_BLOCK, 0, st>>>(anc0, dist0, anc1, dist1, nv, root);
        }
        int32_t *anc = (rounds & 1) ? anc1 : anc0, *dist = (rounds & 1) ? dist1 : dist0;
        k_val_depth<<<G, TREE_BLOCK, 0, st>>>(anc, dist, nv, root, err);
        k_val_edges<<<G, TREE_BLOCK, 0, st>>>(out, dist, directed, err);
        if ((ce = cudaGetLastError())) {
            fc_set_last_cuda_error(ce, "validation kernels", __FILE__, __LINE__);
            rc = FC_ERR_CUDA;
            break;
        }
        unsigned long long h[8];
        if ((ce = cudaMemcpyAsync(h, err, sizeof(h), cudaMemcpyDeviceToHost, st)) ||
            (ce = cudaStreamSynchronize(st))) {
            fc_set_last_cuda_error(ce, "validation result", __FILE__, __LINE__);
            rc = FC_ERR_CUDA;
            break;
        }
        for (int i = 0; i < 8; ++i) errors[i] = (int64_t)h[i];
    } while (0);
    cudaFreeAsync(buf, st);
    cudaFreeAsync(err, st);
    cudaStreamSynchronize(st);
    return rc;
}

}  // namespace fc
