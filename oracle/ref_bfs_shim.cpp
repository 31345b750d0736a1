/*
 * ref_bfs_shim.cpp -- C entry point around the reference's own CPU BFS
 * (class Graph, BFS-4K/src/host/graph.cpp:70-97), compiled together with
 * the reference's unmodified source files by oracle/Makefile into
 * oracle/_ref/libref_bfs.so.  Test infrastructure only: it pins the oracle
 * restatement (fc_oracle.c) and can serve as the timed CPU baseline.
 *
 * The graph is handed over as a finished CSR: the Graph members OutNodes /
 * OutEdges are filled directly, so the reference's COO reader and ToCSR (which
 * keeps duplicate edges) are bypassed.  Distance values are returned raw:
 * unreachable vertices hold the reference's INF (65535, BFS-4K/config.h:50).
 */
#include <cstring>
#include "graph.h"

extern "C" int ref_bfs_many(int V, int E, const int *row_ptr, const int *col,
                            int nsrc, const int *src, int *dist /* nsrc*V */,
                            int *visited /* nsrc, nullable */)
{
    Graph g(V, E, UNDIRECTED);
    std::memcpy(g.OutNodes, row_ptr, sizeof(int) * (size_t)(V + 1));
    std::memcpy(g.OutEdges, col, sizeof(int) * (size_t)E);
    for (int i = 0; i < nsrc; ++i) {
        g.BfsInit(src[i], dist + (size_t)i * (size_t)V);
        g.bfs();
        if (visited) visited[i] = g.visitedNodes();
    }
    delete[] g.OutNodes;
    delete[] g.OutEdges;
    delete[] g.OutDegree;
    delete[] g.COO_Edges;
    return 0;
}

extern "C" int ref_inf(void) { return (int)INF; }
