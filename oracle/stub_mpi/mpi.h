/* Single-rank stand-in for <mpi.h>, used only to compile the reference's own
 * sources into the test harness (oracle/_ref).  Size 1, rank 0; a reduction
 * over one rank is a copy, a broadcast from rank 0 is a no-op.  This mirrors
 * what the reference's MPI calls compute with one process. */
#pragma once
#include <string.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 8
#define MPI_INT 4
#define MPI_SUM 1
static inline int MPI_Init(int* a, char*** b) { (void)a; (void)b; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int* n) { (void)c; *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int* r) { (void)c; *r = 0; return 0; }
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op o, MPI_Comm c) {
  (void)o; (void)c; if (s != r) memcpy(r, s, (size_t)n * (size_t)t); return 0; }
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op o, int root, MPI_Comm c) {
  (void)o; (void)root; (void)c; if (s != r) memcpy(r, s, (size_t)n * (size_t)t); return 0; }
static inline int MPI_Bcast(void* b, int n, MPI_Datatype t, int root, MPI_Comm c) {
  (void)b; (void)n; (void)t; (void)root; (void)c; return 0; }
