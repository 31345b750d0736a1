/*
 * stcon_driver.c -- a C caller of libfastcon.so written the way the
 * bernaschi ST-CON driver would call it after the swap that the integration
 * notes describe: load_graph + run_make_struct (S/main.c:378,438) become
 * fc_graph_load_edgelist, the per-query make_stcon (S/make_stcon.c:446)
 * becomes fc_stcon_depth / fc_stcon, the query loop of run_make_stcon
 * (S/make_stcon.c:416-576) becomes one fc_stcon_batch, and a BFS level array
 * comes from fc_bfs_levels.
 *
 *   stcon_driver <snap edge list> <pairs file: one "s t" per line>
 *
 * Prints one line per pair "q <i> <depth> <connected> <hops>", one per pair
 * of the batch "b <i> <connected> <hops>", and "levels <source> <reached>
 * <sum of levels>" for a BFS from the first pair's s.  Exit status 0 when
 * every call returned FC_OK.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "fastcon.h"

static int fail(const char *what, int rc)
{
    fprintf(stderr, "%s: %s (%s)\n", what, fc_strerror(rc), fc_last_error_message());
    return 1;
}

int main(int argc, char **argv)
{
    if (argc != 3) {
        fprintf(stderr, "usage: %s <edge list> <pairs>\n", argv[0]);
        return 2;
    }
    fc_graph *g = NULL;
    int rc = fc_graph_load_edgelist(argv[1], /*force_dir=*/1, /*relabel=*/0, &g);
    if (rc != FC_OK) return fail("fc_graph_load_edgelist", rc);

    FILE *f = fopen(argv[2], "r");
    if (!f) return 2;
    int32_t cap = 1024, nq = 0;
    int32_t *s = malloc(sizeof(int32_t) * cap), *t = malloc(sizeof(int32_t) * cap);
    long a, b;
    while (fscanf(f, "%ld %ld", &a, &b) == 2) {
        if (nq == cap) {
            cap *= 2;
            s = realloc(s, sizeof(int32_t) * cap);
            t = realloc(t, sizeof(int32_t) * cap);
        }
        s[nq] = (int32_t)a;
        t[nq] = (int32_t)b;
        ++nq;
    }
    fclose(f);

    for (int32_t i = 0; i < nq; ++i) {
        int32_t depth, connected, hops;
        if ((rc = fc_stcon_depth(g, s[i], t[i], &depth)) != FC_OK) return fail("fc_stcon_depth", rc);
        if ((rc = fc_stcon(g, s[i], t[i], &connected, &hops)) != FC_OK) return fail("fc_stcon", rc);
        printf("q %d %d %d %d\n", i, depth, connected, hops);
    }
    int32_t *conn = malloc(sizeof(int32_t) * (nq ? nq : 1));
    int32_t *hop = malloc(sizeof(int32_t) * (nq ? nq : 1));
    rc = fc_stcon_batch(&g, 1, NULL, s, t, nq, conn, hop, NULL, NULL);
    if (rc != FC_OK) return fail("fc_stcon_batch", rc);
    for (int32_t i = 0; i < nq; ++i) printf("b %d %d %d\n", i, conn[i], hop[i]);

    int32_t nv;
    int64_t ne;
    int32_t directed;
    if ((rc = fc_graph_info(g, &nv, &ne, &directed)) != FC_OK) return fail("fc_graph_info", rc);
    int32_t *lev = malloc(sizeof(int32_t) * (size_t)nv);
    if (nq > 0) {
        if ((rc = fc_bfs_levels(g, s[0], lev)) != FC_OK) return fail("fc_bfs_levels", rc);
        long long reached = 0, sum = 0;
        for (int32_t v = 0; v < nv; ++v)
            if (lev[v] >= 0) {
                ++reached;
                sum += lev[v];
            }
        printf("levels %d %lld %lld\n", s[0], reached, sum);
    }
    free(lev);
    free(conn);
    free(hop);
    free(s);
    free(t);
    fc_graph_free(g);
    return 0;
}
