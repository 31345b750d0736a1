/*
 * bfs4k_wrapper.cpp -- the BFS-4K drop-in of the integration notes, built
 * against the reference's own host header (BFS-4K/include/host/graph.h): a
 * class with the method names of cudaGraph (BFS-4K/include/device/
 * cudaGraph.cuh:14-35) whose cudaBFS4K() runs on libfastcon.so, driven the way
 * BFS-4K/bfs4K.cpp:26-54 drives the original, and compared with the
 * reference's own CPU BFS (Graph::BfsInit + Graph::bfs, BFS-4K/src/host/
 * graph.cpp:70-97) on the same Graph.
 *
 *   bfs4k_wrapper <edge list file readable by readGraph::readSTD> [sources...]
 *
 * Prints "ok <sources> <vertices>" and exits 0 when every level matches.
 */
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "fastcon.h"
#include "graph.h"
#include "readGraph.h"

class cudaGraph {
    fc_graph *g_ = nullptr;
    int source_ = 0;

public:
    std::vector<int> hostDistance;  // INF (65535) where unreachable
    explicit cudaGraph(Graph &graph)
    {
        int rc = fc_graph_from_csr(graph.OutNodes, graph.V, graph.OutEdges, graph.OutNodes[graph.V],
                                   graph.Direction == DIRECTED, &g_);
        if (rc != FC_OK) {
            std::fprintf(stderr, "fc_graph_from_csr: %s\n", fc_last_error_message());
            std::exit(1);
        }
        hostDistance.resize(graph.V);
    }
    ~cudaGraph() { fc_graph_free(g_); }
    void Reset(const int Sources[], int /*nof_sources*/) { source_ = Sources[0]; }
    void cudaBFS4K()
    {
        if (fc_bfs_levels(g_, source_, hostDistance.data()) != FC_OK) {
            std::fprintf(stderr, "fc_bfs_levels: %s\n", fc_last_error_message());
            std::exit(1);
        }
        for (int &d : hostDistance)
            if (d < 0) d = INF;
    }
};

int main(int argc, char **argv)
{
    if (argc < 2) return 2;
    int V, E, nof_lines;
    GDirection dir = UNDEFINED;
    readGraph::readGraphHeader(argv[1], V, E, nof_lines, dir);
    Graph graph(V, E, dir);
    readGraph::readSTD(argv[1], graph, nof_lines);
    cudaGraph dev(graph);
    std::vector<int> want(V);
    int nsrc = 0;
    for (int i = 2; i < argc || (argc == 2 && i == 2); ++i) {
        const int src = argc > 2 ? std::atoi(argv[i]) : 0;
        dev.Reset(&src, 1);
        dev.cudaBFS4K();
        graph.BfsInit(src, want.data());
        graph.bfs();
        for (int v = 0; v < V; ++v)
            if (dev.hostDistance[v] != want[v]) {
                std::printf("mismatch source %d vertex %d: %d vs %d\n", src, v,
                            dev.hostDistance[v], want[v]);
                return 1;
            }
        ++nsrc;
    }
    std::printf("ok %d %d\n", nsrc, V);
    return 0;
}
