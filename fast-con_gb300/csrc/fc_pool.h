// fc_pool.h -- host interface of the work-sharing engine (internal).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fc_engine.h"

namespace fc {

struct GraphPair;
struct PoolSlot;
struct RowJob;

struct PoolArgs {
    const GraphPair *graphs;
    const int32_t *graph_idx;
    const int32_t *qs;
    const int32_t *qt;
    const int32_t *list;      // optional subset of query indices
    const int *list_count;    // device count of list entries (nullable)
    int nlist;                // count when list_count is NULL
    int mode, sched, force_variant;
    int private_variant;      // variant for steps the owner runs alone (-1: the schedule's)
    int exclusive;            // 1: CTA 0 owns every query in turn, arrays span the graph
    PoolSlot *slots;          // one per CTA
    int *open;                // one per CTA: 1 while its owner has a step published
                              // (a hint: pollers read only these slots' tile words)
    RowJob *jobs;             // POOL_JOBS per CTA
    uint8_t *status_base;
    size_t status_stride;
    int32_t *levels;          // BFS mode (exclusive only)
    int32_t *log_base;
    size_t log_stride;
    int log_cap;
    long long private_edges;  // steps reading more entries than this are shared
    int tile_e;               // top-down tiles aim at this many adjacency entries
    int split_e;              // rows longer than this become row jobs of this length
    int *ctr;                 // [0] next query [1] finished [2] spill count [3] error [4] invalid
    int32_t *spill;
    int32_t *out_conn;
    int32_t *out_hops;
    QueryStat *qstat;
    // learned schedule and its training data
    const float *mlp;                 // MLP weights (nullable: the heuristic decides)
    const unsigned char *script;      // per query script_len action bytes (nullable)
    int script_len;
    int32_t *trace;                   // TRACE_WORDS ints per step record (nullable)
    int trace_cap;
    int *trace_count;
    long long *out_inspected;         // per-query adjacency entries read (nullable)
};

// One trace record per executed step (ints; features are float bit patterns):
// [0] query [1] step [2] side [3] direction [4] variant [5] met in this step
// [6,7] entries read by the step (lo, hi) [8,9] owner-measured ns (lo, hi)
// [10] vertices claimed [11] frontier vertices [12..23] the 12 features
constexpr int TRACE_WORDS = 24;

size_t pool_slot_bytes();
size_t pool_job_bytes();  // per slot
int pool_block(int requested);                             // 128 or 256
int pool_grid(int sm_count, int ctas_per_sm, int block);   // co-resident CTAs
int pool_max_grid(int sm_count);                           // over both block sizes
int pool_launch(const PoolArgs &a, int grid, int block, cudaStream_t st);

}  // namespace fc
