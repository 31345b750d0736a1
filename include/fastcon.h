/*
 * fastcon.h -- C ABI of the GB300-native ST-CON / BFS library (libfastcon.so).
 *
 * Plain C: opaque handles, int32/int64 arrays, int status codes; no C++ or
 * torch types cross this boundary and nothing aborts the process.  A graph
 * handle owns all device memory it uses; calls on one handle must be
 * serialised by the caller (one handle per host thread, or a lock).
 *
 * Each entry point names the reference interface it replaces (paths relative
 * to the reference project root; S/ = bernaschi/ST_CONN_ONE_ATOMIC/current-st/
 * st-conn/, K/ = BFS-4K/).
 *
 * Answer semantics (all integer, bit-exact against the reference CPU path
 * Graph::bfs, K/src/host/graph.cpp:83-97):
 *   levels[v]  = hop distance from s, -1 where the reference stores INF
 *   connected  = (levels[t] != -1), hops = levels[t] (-1 when not connected)
 */
#ifndef FASTCON_H
#define FASTCON_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define FC_OK              0
#define FC_ERR_INVALID     1  /* bad argument: null pointer, vertex out of range, bad CSR */
#define FC_ERR_CUDA        2  /* a CUDA call failed (fc_last_error_message has details)   */
#define FC_ERR_OOM         3  /* device or host allocation failed                         */
#define FC_ERR_IO          4  /* file cannot be opened / read                             */
#define FC_ERR_FORMAT      5  /* file contents cannot be parsed                           */
#define FC_ERR_TIMEOUT     6  /* a bounded device-side wait expired (kernel returned)     */
#define FC_ERR_OVERFLOW    7  /* graph exceeds the int32 CSR limits                        */
#define FC_ERR_NO_DEVICE   8  /* no CUDA device                                            */
#define FC_ERR_UNSUPPORTED 9  /* option combination not supported                          */

/* ---- ingest flags (fc_graph_from_edges*) -------------------------------- */
#define FC_INGEST_DIRECTED   1  /* keep (u,v) only; default adds (v,u) for every edge   */
#define FC_INGEST_KEEP_LOOPS 2  /* keep self-loops; default drops them                  */
#define FC_INGEST_KEEP_DUPS  4  /* keep repeated edges; default keeps one copy          */

/* ---- scheduling policies ----------------------------------------------- */
#define FC_SCHED_PLAIN     0  /* alternate s-side and t-side, top-down only            */
#define FC_SCHED_HEURISTIC 1  /* side with the smaller frontier-edge sum first;
                                 bottom-up when the frontier's edges exceed the
                                 unexplored edges / 14 (fixed thresholds)               */
#define FC_SCHED_LEARNED   2  /* MLP chooses the side (heads for direction and
                                 variant are trained, not applied); the heuristic
                                 until weights are loaded                              */

/* ---- execution engines ------------------------------------------------- */
#define FC_ENGINE_AUTO       0
#define FC_ENGINE_HOSTLOOP   1  /* one kernel launch per level, host reads counters   */
#define FC_ENGINE_PERSISTENT 2  /* one cooperative launch, grid barrier per level     */
#define FC_ENGINE_BATCHED    3  /* many queries per launch, one CTA per query         */

typedef struct fc_graph fc_graph;

typedef struct fc_opts {
    int32_t sched;        /* FC_SCHED_*                                     */
    int32_t engine;       /* FC_ENGINE_*                                    */
    int32_t block;        /* threads per CTA: 128, 256 or 512 (0 = tuned)   */
    int32_t ctas_per_sm;  /* resident CTAs per SM: batched (0 = 3); plain BFS
                             engine 2, 3 or 4 (0 = 4)                       */
    int32_t use_graph;    /* batched: capture the launch in a CUDA graph    */
    int32_t max_slots;    /* batched: cap on concurrent queries (0 = all)   */
    void   *stream;       /* cudaStream_t, NULL = the library's own stream  */
    int32_t cta_work_k;   /* work-sharing engine: a step reading more than
                             cta_work_k * 1024 adjacency entries is cut into
                             tiles that every CTA may take (0 = 8;
                             < 0 = share every step)                        */
    int32_t variant;      /* top-down expansion variant: 0 = chosen by the
                             schedule, 1 = CTA/warp/scan hybrid, 2 = warp-
                             centric, 3 = one lane per row                  */
    int32_t tile_entries; /* work-sharing engine: a shared top-down tile aims
                             at this many adjacency entries (0 = 16384 for
                             batches, 65536 for one query on the grid)      */
    int32_t job_entries;  /* work-sharing engine: rows longer than this are
                             cut into jobs of this length (0 = 2048 for
                             batches, 8192 for one query on the grid)       */
    int32_t private_variant; /* work-sharing engine: expansion variant of the
                             steps an owner CTA runs alone (same codes as
                             `variant`; 0 = the schedule's choice)          */
    int32_t vertex_order; /* numbering the search runs on, FC_ORDER_*: full
                             BFS (fc_bfs_levels*) and s-t batches of
                             undirected graphs, except on the host-loop
                             engine; single s-t queries use the copy only
                             with FC_ORDER_DEGREE.  Ids in and levels out
                             are always the caller's.                      */
    int32_t slot_log_cap; /* batches: at most this many entries in each
                             query slot's visit log (0 = as large as the
                             arena's memory budget allows, normally one per
                             vertex).  A query whose claims could outgrow it
                             is finished by the whole grid afterwards;
                             smaller logs trade memory for such passes.    */
    int32_t reserved[1];
} fc_opts;

/* ---- vertex numbering of the searches ------------------------------------ */
/* The degree-ordered copy (vertices renumbered by descending degree class,
 * each row listing its highest-degree neighbours first) is built by the first
 * search that uses it and kept by the graph handle: as much device memory
 * again as the CSR, plus an id map.  It packs the hubs' visited state into a
 * few cache sectors per query slot, and searches that stop at the first hit
 * (the meeting of two sides, a bottom-up parent) stop sooner; a batch of
 * 1,024 s-t queries on R-MAT scale 24 runs about 40% faster on it. */
#define FC_ORDER_AUTO   0  /* degree-ordered copy when the graph has hubs
                              (a vertex of degree >= 256), else as given      */
#define FC_ORDER_GIVEN  1  /* search the caller's numbering                   */
#define FC_ORDER_DEGREE 2  /* always search a degree-ordered copy             */

typedef struct fc_stats {
    int64_t edges_inspected;  /* adjacency entries read by expansion steps   */
    int64_t visited;          /* vertices claimed                            */
    int32_t steps;            /* expansion steps (levels of either side)     */
    int32_t bottom_up_steps;
    double  gpu_ms;           /* device time of the call (CUDA events)       */
    int64_t alg_bytes;        /* algorithmic HBM bytes of all steps: 4-byte
                                 status words, 8 per row range, 4 per column
                                 and queue entry (top-down 12|F| + 8E_F + 8|N|,
                                 E_F the entries the step read: a meeting step
                                 that stops early counts only what it read;
                                 bottom-up 12 per scanned vertex + 8 per
                                 neighbour checked + 8|N|)                    */
    int32_t escalated;        /* batched: queries finished by the grid engine */
    int32_t launches;         /* kernels launched by the call                 */
    double  kernel_ms[2];     /* batched: [0] CTA-per-query kernel,
                                 [1] grid kernel for escalated queries       */
    int64_t kernel_alg_bytes[2]; /* alg_bytes of the queries each kernel
                                    finished (same split as kernel_ms)       */
    int32_t graph;            /* batched with use_graph: 1 = replayed the
                                 cached CUDA graph, 2 = captured a new one,
                                 0 = direct launches                          */
    int32_t pad_;
    int64_t visited_adjacency; /* adjacency entries of the claimed vertices
                                  (their degree sum); half of it is the
                                  reference's TEPS numerator count_visited_edges
                                  (S/adj_func.c:334-357) on a symmetric graph  */
} fc_stats;

void fc_opts_init(fc_opts *o);

/* ---- graphs ------------------------------------------------------------ */

/* Load an edge-list file and build the CSR on the device.  Replaces
 * load_graph (S/load_graph.c:20-104; SNAP "# Nodes: N Edges: M" header, raw
 * ids) followed by run_make_struct (S/make_struct.c:39), and
 * readGraph::readGraphHeader + readSTD (K/Util/readGraph.h:18-20; SNAP,
 * MatrixMarket, DIMACS9, DIMACS10 detected from the first token).
 * force_dir: -1 = as the file says (undirected when unspecified, as the
 * bernaschi driver forces), 0 = directed, 1 = undirected.  relabel != 0
 * renumbers SNAP ids by first appearance (BFS-4K), 0 keeps raw ids. */
int fc_graph_load_edgelist(const char *path, int force_dir, int relabel, fc_graph **g);

/* The host half of fc_graph_load_edgelist: parse an edge-list file with
 * nthreads host threads (<= 0: all) into 0-based int32 pairs, in file order.
 * Replaces the single-threaded readers load_graph (S/load_graph.c:20-104)
 * and readSTD (K/Util/readGraphSTD.cpp).  *n = number of pairs, *nv =
 * vertex count, *file_directed = -1 unknown, 0 undirected, 1 directed.
 * When cap < *n nothing is copied and FC_ERR_OVERFLOW is returned with *n
 * set (call again with larger arrays); src/dst may be NULL when cap == 0. */
int fc_parse_edgelist(const char *path, int relabel, int nthreads, int32_t *src, int32_t *dst,
                      int64_t cap, int64_t *n, int32_t *nv, int32_t *file_directed);

/* Adopt a finished CSR from host memory (copied into 128-byte-aligned device
 * arrays).  Replaces Graph::ToCSR's output handed to
 * cudaGraph::cudaGraph(Graph&) (K/include/device/cudaGraph.cuh:14-35).
 * row_ptr must be non-decreasing with row_ptr[0] = 0, row_ptr[nv] = ne, and
 * every col entry in [0, nv).  directed = 0 promises the CSR is symmetric. */
int fc_graph_from_csr(const int32_t *row_ptr, int32_t nv, const int32_t *col, int64_t ne,
                      int directed, fc_graph **g);

/* Build the CSR on the device from a host COO edge list.  Replaces
 * make_g_undirect + make_own_csr_nomulti (S/make_struct.c:304-359,
 * 553-738): symmetrise, drop self-loops, sort, deduplicate (see FC_INGEST_*). */
int fc_graph_from_edges(const int32_t *src, const int32_t *dst, int64_t n, int32_t nv,
                        int flags, fc_graph **g);

/* Same, with the edge list already in device memory (left untouched). */
int fc_graph_from_device_edges(const int32_t *d_src, const int32_t *d_dst, int64_t n,
                               int32_t nv, int flags, fc_graph **g);

/* Seeded synthetic graphs generated and ingested on the device (no host
 * copy of the edge list).  The generators follow fastcon/graphs.py bit for
 * bit.  The R-MAT generator stands in for the reference's Graph500 driver
 * path make_graph -> run_make_struct (S/main.c:358-371): nedges samples
 * with initiator (a, b, c, 1-a-b-c), vertex ids permuted by a seeded
 * bijection when perm_seed >= 0. */
int fc_graph_generate_rmat(int32_t scale, int64_t nedges, double a, double b, double c,
                           uint64_t seed, int64_t perm_seed, fc_graph **g);
/* The Graph500 Kronecker graph the reference driver generates, made on the
 * device: the edges of make_graph(scale, nedges, seed1, seed2, initiator)
 * (bernaschi/ST_CONN_ONE_ATOMIC/current-st/generator/make_graph.c:35-104,
 * called at S/main.c:370), bit for bit, followed by run_make_struct
 * (symmetrise, drop self-loops, deduplicate).  initiator (nullable) = the
 * four quadrant probabilities a, b, c, d (default .57, .19, .19, .05).
 * 1 <= scale <= 29. */
int fc_graph_generate_graph500(int32_t scale, int64_t nedges, uint64_t seed1, uint64_t seed2,
                               const double *initiator, fc_graph **g);
/* The same generator's raw edge list (host arrays of nedges entries): both
 * ends in the generator's vertex labels, the smaller first, self-loops and
 * repeated edges kept as make_graph keeps them; in the generator's own order
 * before its final shuffle of the list (scramble_edges_shared), which this
 * does not apply. */
int fc_graph_generate_graph500_edges(int32_t scale, int64_t nedges, uint64_t seed1,
                                     uint64_t seed2, const double *initiator, int32_t *src,
                                     int32_t *dst);

/* w x h 4-neighbour grid, each edge dropped with probability p_del, plus
 * `shortcuts` uniformly random extra edges. */
int fc_graph_generate_grid(int32_t w, int32_t h, double p_del, uint64_t del_seed,
                           int64_t shortcuts, uint64_t sc_seed, fc_graph **g);

int fc_graph_info(const fc_graph *g, int32_t *nv, int64_t *ne, int32_t *directed);
/* Copy the device CSR back (row_ptr: nv+1 entries, col: ne entries). */
int fc_graph_get_csr(const fc_graph *g, int32_t *row_ptr, int32_t *col);
void fc_graph_free(fc_graph *g);

/* ---- queries ------------------------------------------------------------ */

/* Full BFS level array from s (host output, nv entries, -1 = unreachable).
 * Replaces cudaGraph::Reset + cudaBFS4K (K/src/device/BFS_WorkEfficient.cu:
 * 81-133) whose result is left in devDistance, and Graph::BfsInit + bfs on
 * the host (K/src/host/graph.cpp:70-97).  With FC_ENGINE_AUTO and
 * FC_SCHED_PLAIN the search runs on the plain BFS engine: top-down levels
 * in one cooperative launch, visited bits in a bitmap, and (opts.vertex_order)
 * on a degree-ordered copy of the graph that the first such call builds and
 * the graph handle keeps (as much device memory again as the CSR). */
int fc_bfs_levels(fc_graph *g, int32_t s, int32_t *levels);
int fc_bfs_levels_ex(fc_graph *g, int32_t s, int32_t *levels, const fc_opts *opts,
                     fc_stats *stats);

/* Per-level record of the last plain-BFS-engine search on the current device
 * (the reference times its levels under DBG_TIME, START_TIMER / STOP_TIMER in
 * S/include/header.h): *nlevels = levels expanded; for the first min(cap,
 * 256) levels l (nullable arrays): level_ns[l] = device time of level l's
 * expansion, frontier[l] = vertices at distance l, entries[l] = adjacency
 * entries read expanding them. */
int fc_bfs_trace(int32_t *nlevels, int64_t *level_ns, int64_t *frontier, int64_t *entries,
                 int32_t cap);

/* One s-t connectivity query: connected flag and exact hop distance (-1 when
 * not connected).  Replaces make_stcon (S/include/make_stcon.h:11-17,
 * S/make_stcon.c:730-1497), which returns only DEPTH = ceil(d/2), and the
 * double-source BFS of BFS_4K_DS (BFS_4K_DS/src/device/BFS_WorkEfficient.cu:
 * 110-162), which returns only found / not found. */
int fc_stcon(fc_graph *g, int32_t s, int32_t t, int32_t *connected, int32_t *hops);
int fc_stcon_ex(fc_graph *g, int32_t s, int32_t t, int32_t *connected, int32_t *hops,
                const fc_opts *opts, fc_stats *stats);

/* Compatibility shim for make_stcon's return value: depth = ceil(hops / 2)
 * (simultaneous two-sided rounds), -1 when not connected, 0 when s == t. */
int fc_stcon_depth(fc_graph *g, int32_t s, int32_t t, int32_t *depth);

/* Many queries, possibly over several graphs, in one call (host arrays).
 * graph_idx[i] selects gs[graph_idx[i]] (graph_idx may be NULL: all on
 * gs[0]).  Replaces the per-query loop of run_make_stcon
 * (S/make_stcon.c:416-576) and the one-CTA-per-source launch of
 * BFS_4K_BLOCK (BFS_4K_BLOCK/src/device/BFS_WorkEfficient.cu:64-206). */
int fc_stcon_batch(fc_graph *const *gs, int32_t ngraphs, const int32_t *graph_idx,
                   const int32_t *s, const int32_t *t, int32_t nq, int32_t *connected,
                   int32_t *hops, const fc_opts *opts, fc_stats *stats);

/* Same with every array in device memory (inputs resident in HBM); the
 * call is asynchronous on the chosen stream unless stats is non-NULL. */
int fc_stcon_batch_device(fc_graph *const *gs, int32_t ngraphs, const int32_t *d_graph_idx,
                          const int32_t *d_s, const int32_t *d_t, int32_t nq,
                          int32_t *d_connected, int32_t *d_hops, const fc_opts *opts,
                          fc_stats *stats);

/* ---- learned schedule (no counterpart in the reference) ------------------ */

/* Install the MLP weights of FC_SCHED_LEARNED for the current device: n =
 * 1,703 floats, W1[32][12] b1[32] W2[32][32] b2[32] W3[7][32] b3[7], or
 * 1,727 = those followed by the training feature box lo[12], hi[12] (steps
 * whose features fall outside it are left to the heuristic).  Logits 0-1
 * pick the side, 2-3 top-down / bottom-up, 4-6 the expansion variant.  Only
 * the side head is applied, with a logit margin above ln 3 and while the
 * other side's step reads at most twice the heuristic's; direction and
 * variant stay the heuristic's.  The network
 * reads 12 features per step (frontier sizes and adjacency sums of both
 * sides scaled by the graph size, unexplored fraction, last side, frontier
 * degree mix, radii).  fc_sched_get_weights copies n (1,703 or 1,727). */
int fc_sched_set_weights(const float *w, int32_t n);
int fc_sched_get_weights(float *w, int32_t n);

/* Training kernels.  X: n x 12 features, Y: n x 3 labels (side, direction,
 * variant; -1 = no label), SW (nullable): n x 3 per-head sample weights.
 * fc_mlp_loss_grad: mean weighted softmax cross-entropy and its gradient at
 * weights w (for gradient checks).  fc_mlp_train: `epochs` passes of
 * mini-batch Adam over the samples in the given order; w_inout holds the
 * initial weights and receives the trained ones; loss_curve (nullable,
 * `epochs` floats) gets each epoch's mean loss. */
int fc_mlp_loss_grad(const float *X, const int32_t *Y, const float *SW, int32_t n, const float *w,
                     float *grad, float *loss);
int fc_mlp_train(const float *X, const int32_t *Y, const float *SW, int32_t n, int32_t epochs,
                 int32_t batch, float lr, float *w_inout, float *loss_curve);

/* Batched s-t queries with training-data hooks (device arrays, synchronous).
 * d_script (nullable): script_len action bytes per query forcing its first
 * steps (bit 0 side, bit 1 bottom-up, bits 2-3 variant + 1; 0xFF = let the
 * schedule decide); after the script the schedule of `opts` continues.
 * d_trace (nullable): one record of 24 ints per executed step (query, step,
 * side, direction, variant, met, entries read lo/hi, ns lo/hi, vertices
 * claimed, frontier size, 12 float features as bit patterns), at most
 * trace_cap records, *d_trace_count = records produced.  d_inspected
 * (nullable): adjacency entries read per query. */
int fc_stcon_batch_scripted(fc_graph *g, const int32_t *d_s, const int32_t *d_t, int32_t nq,
                            const uint8_t *d_script, int32_t script_len, const fc_opts *opts,
                            int32_t *d_hops, int64_t *d_inspected, int32_t *d_trace,
                            int32_t trace_cap, int32_t *d_trace_count);

/* Batch of s-t queries that allocates nothing (no counterpart in the
 * reference).  For callers that cannot allocate device memory while they
 * query -- e.g. a service that reserved all device memory for its own pool
 * and forbids allocator calls afterwards, or a plug-in inside a framework
 * that owns the device memory.  The caller passes the graph as device CSR
 * arrays (d_rrow_ptr / d_rcol: reverse CSR of a directed graph, or NULL for
 * a symmetric one) and device arrays for queries and results.  sched is
 * FC_SCHED_PLAIN or FC_SCHED_HEURISTIC; FC_SCHED_LEARNED is accepted and runs
 * as FC_SCHED_HEURISTIC (the network's weights live in allocated memory);
 * other values give FC_ERR_INVALID.  Working memory is a fixed 20 MiB device
 * array inside the library (held on every GPU that loads the library's
 * device code, until exit), so graphs are limited to 1,048,576 vertices
 * (larger: FC_ERR_INVALID).  Calls share that array: calls whose kernels
 * overlap on the GPU race and must be serialised.  The first call on a
 * device (and the first after that device's context was re-created) sets up:
 * it loads the library's device code if the CUDA runtime loads it lazily
 * (CUDA_MODULE_LOADING=LAZY, the default), which is when the array is placed
 * in device memory, and looks up the array's address.  That first call may
 * therefore allocate: make it before reserving device memory and before any
 * stream capture, or set CUDA_MODULE_LOADING=EAGER.  Asynchronous on
 * `stream` (a cudaStream_t); out-of-range query ids give connected = 0,
 * hops = -2. */
int fc_stcon_batch_noalloc(const int32_t *d_row_ptr, const int32_t *d_col, int32_t nv, int64_t ne,
                           const int32_t *d_rrow_ptr, const int32_t *d_rcol, const int32_t *d_s,
                           const int32_t *d_t, int32_t nq, int32_t *d_connected, int32_t *d_hops,
                           int32_t sched, void *stream);

/* Autotuner for repeated batches: runs the caller's sample batch (device
 * arrays, as fc_stcon_batch_device) under each candidate setting of
 * ctas_per_sm {2,3,4} x cta_work_k {2,4,8} x tile_entries {4096,8192,16384},
 * `reps` timed runs each after a warm-up (1 <= reps <= 100), and writes the
 * fastest into *inout (engine = FC_ENGINE_BATCHED; the schedule and the other
 * fields are kept).  *best_ms (nullable) = its median kernel time.  No
 * counterpart in the reference, whose launch shapes are compile-time
 * constants (K/config.h, S/make_stcon.c:29-46). */
int fc_autotune_batch(fc_graph *const *gs, int32_t ngraphs, const int32_t *d_graph_idx,
                      const int32_t *d_s, const int32_t *d_t, int32_t nq, int32_t reps,
                      fc_opts *inout, double *best_ms);

/* ---- after the traversal: trees, paths, validation -------------------------- */
/* BFS tree from s: parents[v] = the smallest-id in-neighbour of v one level
 * closer to s, parents[s] = s, -1 where unreachable (host array, nv).  The
 * reference's predecessor array h_pred (S/make_stcon.c:1189-1455) holds the
 * vertex that claimed v first; this rule makes the tree deterministic.
 * levels (nullable, host, nv) receives the BFS levels as fc_bfs_levels. */
int fc_bfs_parents(fc_graph *g, int32_t s, int32_t *parents, int32_t *levels);

/* One shortest s -> t path: path[0] = s, ..., path[*len - 1] = t, each
 * vertex's predecessor chosen as in fc_bfs_parents.  *len = hops + 1, or 0
 * when t is unreachable; FC_ERR_OVERFLOW (with *len set) when cap is too
 * small.  The reference reconstructs paths from the two colours' predecessor
 * arrays only to validate them (validate_stcon_bfs, S/make_stcon.c:1578-1641). */
int fc_stcon_path(fc_graph *g, int32_t s, int32_t t, int32_t *path, int32_t cap, int32_t *len);

/* Validation of a predecessor map (host array, nv) on the GPU, restating the
 * Graph500 rules of validate_bfs_result (S/reference_functions.c:99-434) for
 * one GPU.  errors[8]: [0] the root is not its own parent, [1] a non-root
 * vertex is its own parent or a parent is out of range, [2] no edge from a
 * parent to its vertex, [3] a parent chain does not reach the root, [4] an
 * edge leaves the tree, [5] an edge's endpoint depths differ by more than one
 * (directed graphs: the head deeper than the tail + 1), [6] vertices in the
 * tree (a count), [7] 0.  Returns FC_OK whatever the counts. */
int fc_validate_bfs(fc_graph *g, int32_t root, const int32_t *parents, int64_t *errors);

/* Is t reachable from s (undirected graphs), by growing BFS regions from
 * nseeds seeds at once -- s, t and nseeds - 2 vertices drawn by a hash of
 * `seed` -- and joining regions in a device union-find whenever an edge
 * links two of them (the BFS_4K_MULTI fork, KM/src/device/
 * BFS_WorkEfficient.cu:9-233 with the closure of BFS_WE_AdjMatrixAnalysis.cu:
 * 4-35).  Exact: yes as soon as s's and t's regions are joined, no when the
 * growth stops first.  No distance.  2 <= nseeds <= 4096; directed graphs:
 * FC_ERR_UNSUPPORTED.  stats (nullable): steps = levels grown. */
int fc_stcon_multiseed(fc_graph *g, int32_t s, int32_t t, int32_t nseeds, uint64_t seed,
                       int32_t *connected, fc_stats *stats);

/* ---- failure detection ---------------------------------------------------- */
/* Self-test of the bounded device-side waits every traversal kernel uses (no
 * counterpart in the reference, whose grid barrier GlobalSync,
 * BFS-4K/src/device/Util/GlobalSync.cu:12, spins without bound).  Launches one CTA into a grid barrier sized for two CTAs:
 * nothing else arrives, so the wait expires after timeout_ms (1..2000) and
 * the kernel returns with FC_ERR_TIMEOUT recorded.  Returns FC_ERR_TIMEOUT
 * when the wait expired as designed (the device stays usable), FC_OK never,
 * another code on failure; *elapsed_ms (nullable) gets the kernel's time. */
int fc_selftest_wait(int32_t timeout_ms, double *elapsed_ms);

/* Self-test of the scan, compaction and search primitives the expansion steps
 * use, on caller data (host arrays; no counterpart in the reference, which
 * takes these from Thrust and CUB: S/mythrustlib.cu:25-34,175-185, checked by
 * check_queue_off, S/test/gputestfunc.cu:225-258).
 *   which 0: out[i] = inclusive warp scan of in within each group of 32;
 *   which 1: out[i] = inclusive block scan within each group of 256,
 *            aux[g] = group g's total;
 *   which 2: in = row lengths, 256 rows to a tile; for every entry of each
 *            tile's rows laid end to end, out = the row (0..255) the
 *            load-balanced search finds (out holds sum(in) entries);
 *   which 3: in = values >= 0 to append (-1 = none), one CTA offering eight
 *            per thread and round; out = the log the per-warp claim buffers
 *            write, aux[0] = its length (each offered value exactly once). */
int fc_selftest_primitives(int32_t which, const int32_t *in, int32_t n, int32_t *out,
                           int32_t *aux);

/* ---- misc ---------------------------------------------------------------- */
const char *fc_strerror(int code);
const char *fc_last_error_message(void);  /* thread-local detail of the last error */
int fc_device_info(int32_t *sm_count, int64_t *total_mem, int32_t *cc_major,
                   int32_t *cc_minor);
int fc_version(void);  /* major*10000 + minor*100 + patch */

#ifdef __cplusplus
}
#endif
#endif /* FASTCON_H */
