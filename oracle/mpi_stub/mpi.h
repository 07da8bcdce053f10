/* Single-rank stand-in for <mpi.h>, used only to compile the reference engine
 * as the CPU oracle (TEST INFRASTRUCTURE, never linked into the product).
 *
 * The engine (src/16SCD_Mg_Cl_K_COPY_fast.cpp) calls MPI_Init/Comm_rank/
 * Comm_size/Allreduce/Reduce/Finalize (lines 6219-6221, 2572, 6284, 6404).
 * With one rank every collective is a copy of the send buffer. */
#ifndef TIS_MPI_STUB_H
#define TIS_MPI_STUB_H
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 8
#define MPI_INT 4
#define MPI_LONG 8
#define MPI_SUM 0
#define MPI_MAX 1

static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op o, MPI_Comm c)
{ (void)o; (void)c; memmove(r, s, (size_t)n * (size_t)t); return 0; }
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op o, int root, MPI_Comm c)
{ (void)o; (void)root; (void)c; memmove(r, s, (size_t)n * (size_t)t); return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
#endif
