/*
 * mpi.h -- minimal stand-in so that the reference's single-rank edge-list
 * reader (load_graph, bernaschi/.../st-conn/load_graph.c:20-104) compiles
 * without an MPI installation.  Test infrastructure only (oracle/_ref).  The
 * reader calls nothing from MPI but MPI_Abort on an unopenable file, which
 * here ends the process the same way.
 */
#ifndef FC_REF_STUB_MPI_H
#define FC_REF_STUB_MPI_H
#include <stdlib.h>
typedef int MPI_Comm;
#define MPI_COMM_WORLD 0
#define MPI_LONG_LONG 0
#define MPI_INT 0
static inline int MPI_Abort(MPI_Comm comm, int code)
{
    (void)comm;
    exit(code);
}
#endif
