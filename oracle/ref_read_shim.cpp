/*
 * ref_read_shim.cpp -- C entry point around the reference's own edge-list
 * readers readGraph::readGraphHeader + readGraph::readSTD
 * (BFS-4K/Util/readGraphHeader.cpp:14-61, BFS-4K/Util/readGraphSTD.cpp:14-145,
 * first-appearance renumbering NodeMap::insertNode BFS-4K/Util/readUtil.cpp:3-11)
 * and the COO -> CSR step Graph::ToCSR (BFS-4K/src/host/graph.cpp:19-42),
 * compiled with those unmodified files by oracle/Makefile into
 * oracle/_ref/libref_read.so.  Test infrastructure only: it pins the
 * oracle's and the product's readers to the reference.
 *
 * The readers report progress on std::cout; it is muted for the call.
 */
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <sstream>

#include "readGraph.h"

/* user_dir: 0 directed, 1 undirected, 2 as the file says (UNDEFINED).
 * Outputs (malloc'd, release with ref_read_free): coo = 2 * *coo_n ints (the
 * COO list in the order the reader stored it), row_ptr = *V + 1 ints and
 * col = row_ptr[*V] ints (the CSR Graph::ToCSR built from it).  *dir = the
 * direction the header resolved (0 directed, 1 undirected). */
extern "C" int ref_read_graph(const char *path, int user_dir, int *V, int *E, int *dir,
                              int *coo_n, int **coo, int **row_ptr, int **col)
{
    std::stringstream sink;
    std::streambuf *old = std::cout.rdbuf(sink.rdbuf());
    int v = 0, e = 0, nof_lines = 0;
    GDirection d = (GDirection)user_dir;
    readGraph::readGraphHeader(path, v, e, nof_lines, d);
    Graph g(v, e, d);
    readGraph::readSTD(path, g, nof_lines);
    std::cout.rdbuf(old);
    *V = v;
    *E = e;
    *dir = (int)g.Direction;
    *coo_n = g.COOSize;
    *coo = (int *)std::malloc(sizeof(int) * 2 * (size_t)(g.COOSize + 1));
    for (int i = 0; i < g.COOSize; ++i) {
        (*coo)[2 * i] = g.COO_Edges[i].x;
        (*coo)[2 * i + 1] = g.COO_Edges[i].y;
    }
    const int ne = g.OutNodes[v];
    *row_ptr = (int *)std::malloc(sizeof(int) * (size_t)(v + 1));
    std::memcpy(*row_ptr, g.OutNodes, sizeof(int) * (size_t)(v + 1));
    *col = (int *)std::malloc(sizeof(int) * (size_t)(ne + 1));
    std::memcpy(*col, g.OutEdges, sizeof(int) * (size_t)ne);
    delete[] g.OutNodes;
    delete[] g.OutEdges;
    delete[] g.OutDegree;
    delete[] g.COO_Edges;
    return 0;
}

extern "C" void ref_read_free(void *p) { std::free(p); }
