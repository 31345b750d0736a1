// fc_parse.h -- multi-threaded edge-list file parser (host side of ingest).
#pragma once

#include <stdint.h>

#include <vector>

namespace fc {

struct Parsed {
    std::vector<int32_t> src, dst;
    long long nv = 0;
    int file_directed = -1;  // -1 unknown, 0 undirected, 1 directed
};

// Parse the file at `path` (SNAP, MatrixMarket, DIMACS9 or DIMACS10/METIS,
// detected from the first line).  relabel = 1 renumbers SNAP ids by first
// appearance.  nthreads <= 0 uses every hardware thread.  Returns FC_OK or an
// FC_ERR_* code with the message set.
int parse_edgelist_file(const char *path, int relabel, int nthreads, Parsed &P);

}  // namespace fc
