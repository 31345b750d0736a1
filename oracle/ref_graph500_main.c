/*
 * ref_graph500_main.c -- writes the edge list produced by the reference's
 * vendored Graph500 generator (bernaschi/.../generator, sequential build,
 * make_graph() at make_graph.c:35-104) to a binary file of int64 pairs.
 * Used only to regenerate the known-answer fixture: the call below is the
 * same one the reference driver makes for a generated graph
 * (st-conn/main.c:358-371): make_graph(SCALE, edgefactor * 2^SCALE, seed1,
 * seed2, {.57,.19,.19,.05}).
 *
 * usage: graph500_gen SCALE EDGEFACTOR SEED1 SEED2 OUT.bin
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include "make_graph.h"

int main(int argc, char **argv)
{
    if (argc != 6) {
        fprintf(stderr, "usage: %s SCALE EDGEFACTOR SEED1 SEED2 OUT.bin\n", argv[0]);
        return 2;
    }
    int scale = atoi(argv[1]);
    double ef = atof(argv[2]);
    uint64_t s1 = strtoull(argv[3], NULL, 10), s2 = strtoull(argv[4], NULL, 10);
    double initiator[4] = {.57, .19, .19, .05};
    int64_t nedges = 0, *edges = NULL;
    make_graph(scale, (int64_t)(ef * pow(2., scale)), s1, s2, initiator, &nedges, &edges);
    FILE *f = fopen(argv[5], "wb");
    if (!f) return 1;
    fwrite(edges, sizeof(int64_t), (size_t)(2 * nedges), f);
    fclose(f);
    free(edges);
    printf("%lld\n", (long long)nedges);
    return 0;
}
