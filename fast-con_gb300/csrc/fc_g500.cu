// fc_g500.cu -- the Graph500 Kronecker generator on the device, bit-compatible
// with the generator the reference driver uses (make_graph, bernaschi/
// ST_CONN_ONE_ATOMIC/current-st/generator/make_graph.c:35-104, sequential
// build with GRAPHGEN_UNDIRECTED, self-loops and duplicates kept).
//
// make_graph draws M edges of a 2^scale-vertex R-MAT by recursive quadrant
// splitting: a node (a square of the adjacency matrix holding ne edges) draws
// how many edges fall in each quadrant (binomial counts), and its children do
// the same, down to single cells; a node with one edge walks down alone.
// Every node's random stream is the root stream jumped ahead by an amount
// that depends only on the node's position, so all nodes of a level are
// independent: here one kernel launch expands one level, a thread per node.
// The vertex labels are then permuted by random keys (rand_sort_shared,
// generator/permutation_gen.c:156-237): a key per vertex from its own jumped
// stream, vertices grouped by key in key order, each group sorted by vertex
// and shuffled by Fisher-Yates from the group's stream.  The reference also
// shuffles the order of the edge list (scramble_edges_shared); the CSR built
// from the edges does not depend on that order, so it is not done.
//
// The unit is compiled with -fmad=false: the binomial sampler's doubles are
// rounded as the generator rounds them.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "fc_engine.h"
#include "fc_g500.cuh"
#include "fc_ingest.h"
#include "fc_internal.cuh"

namespace fc {
namespace g500 {

struct Node {
    long long fei;  // first edge index
    long long ne;   // edges in the node (>= 2)
    int bs, bt;     // first row / column of the node's square
};

struct GenArgs {
    const Mat5 *table;
    Mrg root;
    Initiator ini;
    long long nverts_total;
    int32_t *src, *dst;
};

// The node at (bs, bt) of side nv, jumped to its own stream.
__device__ inline Mrg node_stream(const GenArgs &g, long long bs, long long bt, long long nv)
{
    return mrg_jump(g.table, g.root, 0, (unsigned long long)((bs + g.nverts_total) / nv),
                    (unsigned long long)((bt + g.nverts_total) / nv));
}

// Finish a node that needs no children list: a single cell (all its edges
// are the same edge) or a single edge walking down alone.
__device__ inline void finish_leaf(const GenArgs &g, long long fei, long long ne, long long nv,
                                   long long bs, long long bt)
{
    if (nv == 1) {
        for (long long i = 0; i < ne; ++i) {
            g.src[fei + i] = (int32_t)bs;
            g.dst[fei + i] = (int32_t)bt;
        }
        return;
    }
    Mrg st = node_stream(g, bs, bt, nv);
    long long s = 0, t = 0;
    one_edge(bs, bt, nv, g.ini, st, &s, &t);
    g.src[fei] = (int32_t)s;
    g.dst[fei] = (int32_t)t;
}

// One level: every node of side nv splits its edges over its four quadrants;
// quadrants with two or more edges go to the next level's list, the others
// are finished here.
__global__ void k_g500_level(GenArgs g, const Node *in, long long n_in, long long nv, Node *out,
                             unsigned long long *n_out, unsigned long long cap)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n_in;
         i += (long long)gridDim.x * blockDim.x) {
        const Node nd = in[i];
        Mrg st = node_stream(g, nd.bs, nd.bt, nv);
        long long cnt[4];
        quadrant_counts(nd.ne, g.ini, st, nd.bs == nd.bt, cnt);
        const long long h = nv / 2;
        long long fei = nd.fei;
        for (int q = 0; q < 4; ++q) {
            if (!cnt[q]) continue;
            const long long bs = nd.bs + h * (q / 2), bt = nd.bt + h * (q % 2);
            if (cnt[q] == 1 || h == 1) {
                finish_leaf(g, fei, cnt[q], h, bs, bt);
            } else {
                const unsigned long long k = atomicAdd(n_out, 1ull);
                if (k < cap) out[k] = Node{fei, cnt[q], (int)bs, (int)bt};
            }
            fei += cnt[q];
        }
    }
}

// Permutation keys: uniform in [0, ht) from each vertex's stream (jump
// 2^128 + v 2^64); counts per key.
__global__ void k_g500_keys(const Mat5 *table, Mrg root, long long n, unsigned long long ht,
                            int32_t *key, int32_t *count)
{
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
         v += (long long)gridDim.x * blockDim.x) {
        Mrg st = mrg_jump(table, root, 1, (unsigned long long)v, 0);
        const int32_t k = (int32_t)mrg_below(st, ht);
        key[v] = k;
        atomicAdd(count + k, 1);
    }
}

__global__ void k_g500_scatter(const int32_t *key, long long n, const long long *start,
                               int32_t *fill, int32_t *perm)
{
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
         v += (long long)gridDim.x * blockDim.x) {
        const int32_t k = key[v];
        perm[start[k] + atomicAdd(fill + k, 1)] = (int32_t)v;
    }
}

// Each key's group: sorted by vertex, then shuffled by Fisher-Yates from the
// key's stream (jump 2^128 + key 2^64 + 100).
__global__ void k_g500_groups(const Mat5 *table, Mrg root, unsigned long long ht,
                              const long long *start, int32_t *perm)
{
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < (long long)ht;
         k += (long long)gridDim.x * blockDim.x) {
        const long long b = start[k], n = start[k + 1] - b;
        if (n <= 1) continue;
        int32_t *a = perm + b;
        for (long long i = 1; i < n; ++i) {  // insertion sort: groups hold a few vertices
            const int32_t x = a[i];
            long long j = i - 1;
            while (j >= 0 && a[j] > x) {
                a[j + 1] = a[j];
                --j;
            }
            a[j + 1] = x;
        }
        Mrg st = mrg_jump(table, root, 1, (unsigned long long)k, 100);
        for (long long i = n - 1; i > 0; --i) {
            const long long j = (long long)mrg_below(st, (unsigned long long)(i + 1));
            if (i != j) {
                const int32_t t = a[i];
                a[i] = a[j];
                a[j] = t;
            }
        }
    }
}

// Relabel both ends; the smaller label first, as the generator stores them.
__global__ void k_g500_label(const int32_t *perm, long long m, int32_t *src, int32_t *dst)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m;
         i += (long long)gridDim.x * blockDim.x) {
        const int32_t a = perm[src[i]], b = perm[dst[i]];
        src[i] = a < b ? a : b;
        dst[i] = a < b ? b : a;
    }
}

const std::vector<Mat5> &jump_tables()
{
    static std::vector<Mat5> t;
    static std::once_flag once;
    std::call_once(once, [] {
        t.resize((size_t)JUMP_BYTES * 256);
        build_jump_tables(t.data());
    });
    return t;
}

}  // namespace g500

static int grid_of(long long n)
{
    return (int)std::max(1LL, std::min(8192LL, (n + 255) / 256));
}

// M edges of the 2^scale-vertex Graph500 graph into new device arrays
// (*d_src, *d_dst, M entries each, caller frees), in the generator's vertex
// labels; self-loops and repeated edges included, as the generator keeps them.
int gen_graph500_device(int scale, long long m, unsigned long long seed1, unsigned long long seed2,
                        const double initiator[4], int32_t **d_src, int32_t **d_dst,
                        cudaStream_t st)
{
    using namespace g500;
    *d_src = *d_dst = nullptr;
    if (scale < 1 || scale > 29 || m < 1) {
        set_error("graph500 generator: scale %d, %lld edges (scale 1..29, edges >= 1)", scale, m);
        return FC_ERR_INVALID;
    }
    const long long n = 1LL << scale;
    Initiator ini;
    double sum = 0;
    for (int i = 0; i < 4; ++i) {
        ini.q[i] = initiator[i];
        if (!(initiator[i] >= 0.) || !(initiator[i] <= 1.)) {
            set_error("graph500 generator: initiator entry %d outside [0, 1]", i);
            return FC_ERR_INVALID;
        }
        sum += initiator[i];
    }
    if (sum < 0.999999 || sum > 1.000001) {
        set_error("graph500 generator: initiator sums to %g, not 1", sum);
        return FC_ERR_INVALID;
    }
    const std::vector<Mat5> &tables = jump_tables();
    Mat5 *d_table = nullptr;
    Node *nodes[2] = {nullptr, nullptr};
    unsigned long long *d_cnt = nullptr;
    int32_t *key = nullptr, *count = nullptr, *perm = nullptr, *fill = nullptr;
    long long *start = nullptr;
    int rc = FC_OK;
    const unsigned long long ht = 2ull * (unsigned long long)n + 128;
    // an internal node holds at least two edges: at most m / 2 per level
    const unsigned long long cap = (unsigned long long)(m / 2 + 1);
    auto done = [&](int r) {
        cudaFree(d_table);
        cudaFree(nodes[0]);
        cudaFree(nodes[1]);
        cudaFree(d_cnt);
        cudaFree(key);
        cudaFree(count);
        cudaFree(perm);
        cudaFree(fill);
        cudaFree(start);
        if (r != FC_OK) {
            cudaFree(*d_src);
            cudaFree(*d_dst);
            *d_src = *d_dst = nullptr;
        }
        return r;
    };
#define G5_TRY(expr)                                                  \
    do {                                                              \
        cudaError_t e_ = (expr);                                      \
        if (e_ != cudaSuccess) {                                      \
            fc_set_last_cuda_error(e_, #expr, __FILE__, __LINE__);    \
            return done(e_ == cudaErrorMemoryAllocation ? FC_ERR_OOM : FC_ERR_CUDA); \
        }                                                             \
    } while (0)
    G5_TRY(cudaMalloc(&d_table, sizeof(Mat5) * tables.size()));
    G5_TRY(cudaMemcpyAsync(d_table, tables.data(), sizeof(Mat5) * tables.size(),
                           cudaMemcpyHostToDevice, st));
    G5_TRY(cudaMalloc(d_src, sizeof(int32_t) * (size_t)m));
    G5_TRY(cudaMalloc(d_dst, sizeof(int32_t) * (size_t)m));
    G5_TRY(cudaMalloc(&nodes[0], sizeof(Node) * (size_t)cap));
    G5_TRY(cudaMalloc(&nodes[1], sizeof(Node) * (size_t)cap));
    G5_TRY(cudaMalloc(&d_cnt, sizeof(unsigned long long)));
    GenArgs g;
    g.table = d_table;
    g.root = mrg_seed(seed1, seed2);
    g.ini = ini;
    g.nverts_total = n;
    g.src = *d_src;
    g.dst = *d_dst;
    long long n_cur = 0;
    if (m == 1) {
        // a single edge walks down from the root alone (on the host: it is
        // one short walk)
        Mrg s0 = mrg_jump(tables.data(), g.root, 0, 1, 1);
        long long a = 0, b = 0;
        one_edge(0, 0, n, ini, s0, &a, &b);
        const int32_t ha = (int32_t)a, hb = (int32_t)b;
        G5_TRY(cudaMemcpyAsync(*d_src, &ha, sizeof(int32_t), cudaMemcpyHostToDevice, st));
        G5_TRY(cudaMemcpyAsync(*d_dst, &hb, sizeof(int32_t), cudaMemcpyHostToDevice, st));
        G5_TRY(cudaStreamSynchronize(st));
    } else {
        // the root: all m edges in the whole matrix
        const Node root{0, m, 0, 0};
        G5_TRY(cudaMemcpyAsync(nodes[0], &root, sizeof(Node), cudaMemcpyHostToDevice, st));
        n_cur = 1;
    }
    long long nv = n;
    int cur = 0;
    while (n_cur > 0) {
        G5_TRY(cudaMemsetAsync(d_cnt, 0, sizeof(unsigned long long), st));
        k_g500_level<<<grid_of(n_cur), 256, 0, st>>>(g, nodes[cur], n_cur, nv, nodes[cur ^ 1],
                                                     d_cnt, cap);
        G5_TRY(cudaGetLastError());
        unsigned long long h_cnt = 0;
        G5_TRY(cudaMemcpyAsync(&h_cnt, d_cnt, sizeof(h_cnt), cudaMemcpyDeviceToHost, st));
        G5_TRY(cudaStreamSynchronize(st));
        if (h_cnt > cap) {
            set_error("graph500 generator: node list overflow (%llu > %llu)", h_cnt, cap);
            return done(FC_ERR_CUDA);
        }
        n_cur = (long long)h_cnt;
        nv /= 2;
        cur ^= 1;
    }
    // the vertex permutation
    G5_TRY(cudaMalloc(&key, sizeof(int32_t) * (size_t)n));
    G5_TRY(cudaMalloc(&count, sizeof(int32_t) * (size_t)ht));
    G5_TRY(cudaMalloc(&fill, sizeof(int32_t) * (size_t)ht));
    G5_TRY(cudaMalloc(&start, sizeof(long long) * ((size_t)ht + 1)));
    G5_TRY(cudaMalloc(&perm, sizeof(int32_t) * (size_t)n));
    G5_TRY(cudaMemsetAsync(count, 0, sizeof(int32_t) * (size_t)ht, st));
    G5_TRY(cudaMemsetAsync(fill, 0, sizeof(int32_t) * (size_t)ht, st));
    k_g500_keys<<<grid_of(n), 256, 0, st>>>(d_table, g.root, n, ht, key, count);
    G5_TRY(cudaGetLastError());
    rc = scan_i32(count, (long long)ht, start, st);
    if (rc) return done(rc);
    k_g500_scatter<<<grid_of(n), 256, 0, st>>>(key, n, start, fill, perm);
    k_g500_groups<<<grid_of((long long)ht), 256, 0, st>>>(d_table, g.root, ht, start, perm);
    k_g500_label<<<grid_of(m), 256, 0, st>>>(perm, m, *d_src, *d_dst);
    G5_TRY(cudaGetLastError());
    G5_TRY(cudaStreamSynchronize(st));
#undef G5_TRY
    return done(FC_OK);
}

}  // namespace fc
