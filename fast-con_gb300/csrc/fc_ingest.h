// fc_ingest.h -- device CSR construction and graph generators (internal).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fc {

// Build a canonical CSR from a device COO list (src[i] == -1 marks "no
// edge").  On success *out_row_ptr / *out_col are new device allocations
// owned by the caller.
int ingest_device_edges(const int32_t *d_src, const int32_t *d_dst, long long n, int nv, int flags,
                        int32_t **out_row_ptr, int32_t **out_col, long long *out_ne,
                        cudaStream_t st);

int gen_rmat_device(int scale, long long nedges, double a, double b, double c,
                    unsigned long long seed, long long perm_seed, int32_t *d_src, int32_t *d_dst,
                    cudaStream_t st);

// Sort every row of a CSR with int64 offsets off[0..nv] ascending, in place
// (ne entries in col).  Waits for the stream.
int sort_rows_i32(const long long *off, int nv, long long ne, int32_t *col, cudaStream_t st);

// Exclusive scan of n int32 values into out[0..n), out[n] = total (int64).
int scan_i32(const int32_t *in, long long n, long long *out, cudaStream_t st);

// M edges of the Graph500 generator (fc_g500.cu) into new device arrays.
int gen_graph500_device(int scale, long long m, unsigned long long seed1, unsigned long long seed2,
                        const double initiator[4], int32_t **d_src, int32_t **d_dst,
                        cudaStream_t st);

long long grid_edge_slots(int w, int h, long long shortcuts);

int gen_grid_device(int w, int h, double p_del, unsigned long long del_seed, long long shortcuts,
                    unsigned long long sc_seed, int32_t *d_src, int32_t *d_dst, cudaStream_t st);

}  // namespace fc
