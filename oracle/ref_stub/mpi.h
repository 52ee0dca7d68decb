/* Single-rank stand-in for <mpi.h>, used only to compile the reference's
 * 3D/2D MPI drivers into the reference oracle (oracle/_ref).  With one rank
 * and periodic boundaries the reference never calls Sendrecv; Allreduce is a
 * copy.  TEST INFRASTRUCTURE ONLY. */
#ifndef ORACLE_MPI_STUB_H
#define ORACLE_MPI_STUB_H
#include <stdio.h>
#include <string.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_PROC_NULL (-1)
#define MPI_DOUBLE 8
#define MPI_INT 4
#define MPI_MAX 1
#define MPI_SUM 2
#define MPI_MIN 3
static inline int MPI_Init(int *a, char ***b) { (void)a; (void)b; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Abort(MPI_Comm c, int e) { (void)c; (void)e; return 0; }
static inline int MPI_Bcast(void *b, int n, MPI_Datatype t, int r, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)r; (void)c; return 0; }
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op o, MPI_Comm c)
{ (void)o; (void)c; memcpy(r, s, (size_t)n * (size_t)t); return 0; }
static inline int MPI_Sendrecv(const void *sb, int sn, MPI_Datatype st, int d, int stag, void *rb,
                               int rn, MPI_Datatype rt, int s, int rtag, MPI_Comm c, MPI_Status *x)
{ (void)sb; (void)sn; (void)st; (void)d; (void)stag; (void)rb; (void)rn; (void)rt; (void)s;
  (void)rtag; (void)c; (void)x; return 0; }
static inline double MPI_Wtime(void) { return 0.0; }
#endif
