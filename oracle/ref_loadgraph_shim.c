/*
 * ref_loadgraph_shim.c -- C entry point around the reference's own SNAP
 * edge-list reader load_graph (bernaschi/ST_CONN_ONE_ATOMIC/current-st/
 * st-conn/load_graph.c:20-104), compiled with that unmodified file by
 * oracle/Makefile into oracle/_ref/libref_loadgraph.so.  Test
 * infrastructure only: it pins the oracle's and the product's raw-id SNAP
 * reading to the reference.
 *
 * load_graph reads the share of the file body that belongs to MPI rank
 * `rank` of `size`; one rank of one reads all of it.  callmalloc is the
 * reference's checked malloc (cputils.c, which needs CUDA and MPI, so it is
 * supplied here).
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

int rank = 0, size = 1, lgsize = 0;

void *callmalloc(size_t nbytes, const char *funcname)
{
    (void)funcname;
    return malloc(nbytes ? nbytes : 1);
}

void load_graph(char *fname_graph, int64_t *nedges_ptr, int64_t **result_ptr, int64_t *gnverts);

/* *edges = 2 * *nedges int64 (u, v pairs in file order, raw ids), to be
 * released with ref_free; *nverts = the header's node count. */
int ref_load_graph(const char *path, int64_t *nedges, int64_t **edges, int64_t *nverts)
{
    load_graph((char *)path, nedges, edges, nverts);
    return 0;
}

void ref_free(void *p) { free(p); }
