/*
 * Single-rank stand-in for the MPI subset the SW2 sources call (test
 * infrastructure: used only to build the reference as a CPU oracle).
 *
 * Semantics are those of an MPI job with exactly one rank: reductions and
 * broadcasts copy the send buffer to the receive buffer, rank is 0, size is 1.
 * Point-to-point calls are never reached with one rank in SW2 (the halo code
 * takes its single-map branch, sppde/sppde_hupdate.c:356-358); if one is
 * reached anyway it aborts so that a wrong build cannot pass silently.
 */
#ifndef SW2_ORACLE_MPI_STUB_H
#define SW2_ORACLE_MPI_STUB_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3
#define MPI_IN_PLACE ((void *)1)

static inline size_t sw2stub_size(MPI_Datatype t) { return t == MPI_INT ? sizeof(int) : sizeof(double); }

static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Initialized(int *flag) { *flag = 1; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Abort(MPI_Comm c, int code) { (void)c; exit(code ? code : 1); }
static inline double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
  (void)op; (void)c;
  if (s != MPI_IN_PLACE) memmove(r, s, (size_t)n * sw2stub_size(t));
  return 0;
}
static inline int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c) {
  (void)b; (void)n; (void)t; (void)root; (void)c; return 0;
}
static inline int sw2stub_p2p(const char *what) {
  fprintf(stderr, "mpi stub: %s reached with a single rank\n", what);
  abort();
}
static inline int MPI_Sendrecv(const void *sb, int sn, MPI_Datatype st, int dst, int stag, void *rb, int rn,
                               MPI_Datatype rt, int src, int rtag, MPI_Comm c, MPI_Status *status) {
  (void)sb; (void)sn; (void)st; (void)dst; (void)stag; (void)rb; (void)rn; (void)rt; (void)src; (void)rtag; (void)c; (void)status;
  return sw2stub_p2p("MPI_Sendrecv");
}
static inline int MPI_Ssend(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c) {
  (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; return sw2stub_p2p("MPI_Ssend");
}
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status *st) {
  (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st; return sw2stub_p2p("MPI_Recv");
}

#endif
