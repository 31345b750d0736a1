// fc_engine.h -- host-side interface of the traversal engines (internal).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <vector>

#include "fastcon.h"

namespace fc {

struct DGraphH {  // host copy of a device CSR
    const int32_t *row_ptr;
    const int32_t *col;
    int32_t nv;
    int32_t pad_;
    int64_t ne;
    const int32_t *remap;  // nullable: caller's vertex id -> id in this CSR (a renumbered copy)
};

// forward CSR (expands the s side) and reverse CSR (expands the t side);
// identical for undirected graphs
struct GraphPairH {
    DGraphH fwd, rev;
};

struct TeamCounters;
struct QueryStat {
    long long inspected;
    long long alg_bytes;
    int steps;
    int bu_steps;
    int visited;
    int escalated;
    long long visited_deg;  // degree sum of the claimed vertices
};

// Per-device context: workspaces grown on demand, events, the batched arena.
struct DevCtx {
    int device = -1;
    int sm_count = 0;
    int coop = 0;
    std::mutex mu;
    // persistent / host-loop workspace (one query at a time)
    uint8_t *status = nullptr;
    int32_t *levels = nullptr;
    int32_t *log = nullptr;
    size_t ws_nv = 0;
    TeamCounters *tc = nullptr;      // device
    int2 *tjobs = nullptr;           // row jobs of team steps (grid / host-loop engines)
    int tjobs_cap = 0;
    TeamCounters *h_tc = nullptr;    // pinned mirror
    void *d_graphs = nullptr;        // GraphPair table
    size_t graphs_cap = 0;
    std::vector<unsigned char> graphs_last;  // the table's last upload (host copy)
    // batched arena
    uint8_t *b_status = nullptr;
    int32_t *b_log = nullptr;
    size_t b_slots = 0, b_status_stride = 0, b_log_stride = 0;
    // pool engine: one slot record and one row-job area per resident CTA
    void *p_slots = nullptr;
    void *p_jobs = nullptr;
    int *p_open = nullptr;           // PoolArgs::open
    int p_grid = 0;
    // learned schedule weights (1,703 floats) and feature box (24 floats),
    // device and host copies
    float *d_mlp = nullptr;
    float h_mlp[1727];
    int mlp_ready = 0;
    int b_log_cap = 0;
    int *b_ctr = nullptr;            // [0] next query, [1] spill count, [2] error
    int *h_bctr = nullptr;           // pinned mirror of b_ctr
    int deferred_engine = -1;        // engine whose error words are in flight to
                                     // h_bctr / h_tc (BATCH_DEFER_CHECK), else -1
    int32_t *b_spill = nullptr;
    size_t b_spill_cap = 0;
    QueryStat *qstat = nullptr;
    size_t qstat_cap = 0;
    int32_t *d_tmp_q = nullptr;      // staging for host-array batches
    size_t tmp_q_cap = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evm = nullptr;
    cudaStream_t stream = nullptr;
    // cached CUDA graph of the last batched launch, keyed by its arguments
    cudaGraphExec_t gexec = nullptr;
    unsigned char gkey[640];
    size_t gkey_len = 0;
    int graph_replays = 0;           // replays of the cached graph (tests)
    int graph_captures = 0;          // captures made
    int *selftest = nullptr;         // barrier + flag of the wait self-test
    // staging of host-array batches (queries in, answers out)
    int32_t *b_stage = nullptr;
    size_t b_stage_cap = 0;
    // plain BFS engine (fc_bfs.cu): visited bitmap, levels in the search's
    // numbering and in the caller's, frontier queues, counters
    unsigned *bfs_bm = nullptr;
    int32_t *bfs_lev = nullptr;
    int32_t *bfs_out = nullptr;
    int2 *bfs_q = nullptr;           // frontier queues (row ranges)
    size_t bfs_nv = 0;
    long long bfs_pcap = 0;
    void *bfs_ctr = nullptr;
    void *h_bfs_ctr = nullptr;
};

// Device staging for a host-array batch of n queries: 5n ints, kept between
// calls so that repeated batches of the same size reuse a captured graph.
int32_t *batch_staging(DevCtx *c, size_t n, int *rc);

DevCtx *get_ctx(int *err);

int engine_bfs(DevCtx *c, const GraphPairH &gp, int32_t s, int32_t *h_levels,
               const fc_opts &o, fc_stats *st, cudaStream_t stream);

// Plain (top-down, level-synchronous) BFS on the visited-bitmap engine of
// fc_bfs.cu; L (nullable) is the graph's degree-ordered copy.
struct BfsLayout;
int bfs_layout_build(const GraphPairH &gp, BfsLayout **out, cudaStream_t st, int only_if_skewed);
void bfs_layout_free(BfsLayout *L);
// The renumbered CSR of a layout as a graph a batch can run on (remap = the
// caller's id -> renumbered id map).
void bfs_layout_graph(const BfsLayout *L, DGraphH *out);
int engine_bfs_plain(DevCtx *c, const GraphPairH &gp, const BfsLayout *L, int32_t s,
                     int32_t *h_levels, const fc_opts &o, fc_stats *st, cudaStream_t stream);
int engine_bfs_trace(DevCtx *c, int32_t *nlevels, int64_t *level_ns, int64_t *frontier,
                     int64_t *entries, int32_t cap);

int engine_stcon(DevCtx *c, const GraphPairH &gp, int32_t s, int32_t t, int32_t *conn,
                 int32_t *hops, const fc_opts &o, fc_stats *st, cudaStream_t stream);

// Training-data hooks of the batched engine (all device pointers, nullable).
struct BatchExtras {
    const unsigned char *script = nullptr;  // nq * script_len action bytes
    int script_len = 0;
    int32_t *trace = nullptr;               // trace_cap records of 24 ints
    int trace_cap = 0;
    int32_t *trace_count = nullptr;
    long long *inspected = nullptr;         // per query
};

// check: BATCH_NO_CHECK returns once the launches are queued; BATCH_CHECK
// waits for them and reads the device-side error words; BATCH_DEFER_CHECK
// queues the copies of those words to pinned host memory and returns, and the
// caller calls engine_finish_checks after its own synchronisation of the
// stream (one wait for the results and the checks together).  Statistics
// (st != nullptr) always wait.
constexpr int BATCH_NO_CHECK = 0, BATCH_CHECK = 1, BATCH_DEFER_CHECK = 2;
// Page-locked host arrays of a host-array batch on the batched engine: the
// engine copies s, t (and gi) into its device arguments before the kernels
// and the answers (and, with BATCH_DEFER_CHECK, the error words) back after
// them, all inside the batch's CUDA graph when one is used.
struct BatchHostIO {
    const int32_t *s, *t, *gi;  // gi nullable
    int32_t *conn, *hops;
};
int engine_stcon_batch(DevCtx *c, const GraphPairH *gps, int ngraphs, const int32_t *d_gi,
                       const int32_t *d_s, const int32_t *d_t, int32_t nq, int32_t *d_conn,
                       int32_t *d_hops, const fc_opts &o, fc_stats *st, cudaStream_t stream,
                       int check, const BatchExtras *ex = nullptr,
                       const BatchHostIO *hio = nullptr);
// The error words a BATCH_DEFER_CHECK call queued, read after the stream was
// synchronised: FC_OK, or FC_ERR_TIMEOUT with the workspaces reset.
int engine_finish_checks(DevCtx *c);

// BFS tree, shortest path, predecessor-map validation (fc_tree.cu).
int engine_bfs_parents(DevCtx *c, const GraphPairH &gp, int32_t s, int32_t *h_parents,
                       int32_t *h_levels, const fc_opts &o, cudaStream_t st);
int engine_stcon_path(DevCtx *c, const GraphPairH &gp, int32_t s, int32_t t, int32_t *h_path,
                      int32_t cap, int32_t *len, const fc_opts &o, cudaStream_t st);
int engine_validate_bfs(DevCtx *c, const GraphPairH &gp, int directed, int32_t root,
                        const int32_t *h_parents, int64_t *errors, cudaStream_t st);

// s~t connectivity by multi-seed region growth (fc_multiseed.cu)
int engine_stcon_multiseed(DevCtx *c, const GraphPairH &gp, int32_t s, int32_t t, int32_t nseeds,
                           unsigned long long seed, int32_t *connected, fc_stats *st,
                           cudaStream_t stream);

// Grow the single-query workspaces (status, levels, log, team jobs) to nv.
int ensure_workspace(DevCtx *c, size_t nv);

// Bounded-wait self-test: one CTA waits at a two-CTA barrier until the wait
// expires; returns FC_ERR_TIMEOUT when it did.
int engine_selftest_wait(DevCtx *c, int timeout_ms, double *elapsed_ms, cudaStream_t stream);

// The scan / compaction / search primitives on caller data (fc_selftest.cu).
int engine_selftest_primitives(DevCtx *c, int which, const int32_t *h_in, int n, int32_t *h_out,
                               int32_t *h_aux, cudaStream_t st);

void set_error(const char *fmt, ...);

}  // namespace fc
