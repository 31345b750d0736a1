/*
 * fc_oracle.h -- CPU oracle for the ST-CON / BFS hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code.  It is used by tests/, by __graft_entry__.smoke() and by
 * bench.py's CPU-baseline leg, always as the checker, never as the thing that
 * is measured or shipped.
 *
 * Every function is a plain-C restatement of a reference routine; the
 * citation next to each declaration names the reference file:line it follows
 * (paths relative to the reference project root):
 *   K/ = BFS-4K/,  S/ = bernaschi/ST_CONN_ONE_ATOMIC/current-st/st-conn/
 *
 * Parity pins: the restatement is checked against (1) the reference's own
 * Graph::bfs compiled from its sources into oracle/_ref/ (see Makefile), and
 * (2) the 100-row known-answer ST-CON run S/data/st_stats_20200418_140644
 * (DEPTH = ceil(d/2) on the Graph500 R-MAT scale-16 graph), both committed as
 * fixtures under tests/golden/.
 */
#ifndef FC_ORACLE_H
#define FC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Flags for oracle_build_csr (same meaning as the product's FC_INGEST_*). */
#define ORACLE_SYMMETRIZE 1   /* add (v,u) for every (u,v)                  */
#define ORACLE_DROP_LOOPS 2   /* remove (u,u)                               */
#define ORACLE_DEDUPE     4   /* keep one copy of each (u,v); rows sorted   */

/* Level-synchronous queue BFS from src.  Restates Graph::BfsInit +
 * Graph::bfs (K/src/host/graph.cpp:70-97).  levels[v] = hop count, or -1
 * where the reference stores INF (K/config.h:50).  queue is scratch of nv
 * ints.  Returns the number of visited vertices; *edges_inspected (if not
 * NULL) receives the sum of the visited vertices' degrees
 * (Graph::visitedEdges, K/src/host/graph.cpp:104-112). */
int32_t oracle_bfs_levels(int32_t nv, const int32_t *row_ptr, const int32_t *col,
                          int32_t src, int32_t *levels, int32_t *queue,
                          int64_t *edges_inspected);

/* ST-CON answer the reference's CPU path yields: one full BFS rooted at s,
 * connected = Distance[t] != INF, hops = Distance[t] (-1 if not connected).
 * Queries are independent and run on nthreads POSIX threads, each with its
 * own BFS buffers.  edges_inspected (nullable) gets one count per query. */
int oracle_stcon_batch(int32_t nv, const int32_t *row_ptr, const int32_t *col,
                       int32_t nq, const int32_t *s, const int32_t *t,
                       int32_t *connected, int32_t *hops,
                       int64_t *edges_inspected, int nthreads);

/* Stronger CPU baseline (not the reference's path): bidirectional BFS that
 * alternates the side with the smaller frontier-edge sum and stops at the
 * first meeting level.  Same answers as oracle_stcon_batch. */
int oracle_stcon_bidir_batch(int32_t nv, const int32_t *row_ptr, const int32_t *col,
                             int32_t nq, const int32_t *s, const int32_t *t,
                             int32_t *connected, int32_t *hops,
                             int64_t *edges_inspected, int nthreads);

/* Canonical CSR from a COO edge list.  Restates the ingest semantics of
 * make_g_undirect (S/make_struct.c:304-359, k_add_vu
 * S/cudakernel/gstruct_kernel.cu:187-204: symmetrise, self-loops dropped)
 * and make_own_csr_nomulti (S/make_struct.c:553-738: sort by (u,v), drop
 * duplicates, offsets per vertex).  Edges with an endpoint outside [0,nv)
 * make the call fail (returns -1).  col must hold up to 2*n entries.
 * Returns the number of directed entries written. */
int64_t oracle_build_csr(int32_t nv, int64_t n, const int32_t *src, const int32_t *dst,
                         int flags, int32_t *row_ptr, int32_t *col);

/* Same as oracle_build_csr with the per-row sort spread over nthreads. */
int64_t oracle_build_csr_mt(int32_t nv, int64_t n, const int32_t *src, const int32_t *dst,
                            int flags, int32_t *row_ptr, int32_t *col, int nthreads);

/* R-MAT edge samples from the counter-based hash of fastcon/graphs.py
 * (input generation for the CPU baseline; identical to the GPU generator):
 * level k of edge i draws x = hash(seed, k+1, i) >> 32 and picks the quadrant
 * by integer thresholds a, a+b, a+b+c scaled by 2^32; ids are then permuted
 * by the seeded bijection when perm_seed >= 0. */
void oracle_gen_rmat(int scale, int64_t nedges, double a, double b, double c, uint64_t seed,
                     int64_t perm_seed, int32_t *src, int32_t *dst, int nthreads);

/* Graph500 TEPS numerator: for every visited vertex v (levels[v] != -1)
 * count the neighbours u <= v.  Restates count_visited_edges
 * (S/adj_func.c:334-357). */
int64_t oracle_count_visited_edges(int32_t nv, const int32_t *row_ptr, const int32_t *col,
                                   const int32_t *levels);

/* Edge-list file reader.  Formats, detected from the first token as
 * readGraphHeader does (K/Util/readGraphHeader.cpp:14-45):
 *   '#'               SNAP; header "# Nodes: N Edges: M" (S/load_graph.c:45-55)
 *   '%%MatrixMarket'  MatrixMarket coordinate, 1-based (K/Util/readGraphSTD.cpp:57-75)
 *   'c' / 'p'         DIMACS9 "a u v w" arcs, 1-based (K/Util/readGraphSTD.cpp:78-99)
 *   '%' or a number   DIMACS10/METIS adjacency lines, 1-based (K/Util/readGraphSTD.cpp:101-125)
 * SNAP ids are kept raw (the bernaschi loader) unless relabel != 0, in which
 * case they are renumbered by first appearance (NodeMap::insertNode,
 * K/Util/readUtil.cpp:3-11; readGraphSnap K/Util/readGraphSTD.cpp:128-145).
 * Call once with src = dst = NULL to get *nv, *n and *file_directed
 * (1 directed, 0 undirected, -1 undefined); then again with arrays of *n
 * entries.  Returns 0, or -1 on an unreadable / malformed file. */
int oracle_read_edgelist(const char *path, int relabel, int32_t *nv, int64_t *n,
                         int *file_directed, int32_t *src, int32_t *dst);

#ifdef __cplusplus
}
#endif
#endif
