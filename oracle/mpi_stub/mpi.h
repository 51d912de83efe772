/*
 * Single-rank stand-in for <mpi.h>, used only to compile the unmodified girih
 * reference sources (src/driver.c, src/utils.c, the src/kernels sources, ...) into the
 * CPU oracle and CPU baseline binary.  It is test infrastructure: nothing in the
 * GPU library includes it.
 *
 * Semantics are those of an MPI job with exactly one rank:
 *   - a Cartesian neighbour is the rank itself along a periodic dimension and
 *     MPI_PROC_NULL otherwise; messages to itself are delivered (mpi_stub.c),
 *     which the diamond stepper's periodic y exchanges need
 *     (src/mpi_utils.c:66-80, src/kernels/diamond_ts.c:128-290);
 *   - reductions copy the send buffer (src/utils.c:844-860);
 *   - broadcasts and barriers do nothing;
 *   - MPI_Wtime is a monotonic wall clock (src/performance.c:74-78).
 */
#ifndef GIRIH_SINGLE_RANK_MPI_H
#define GIRIH_SINGLE_RANK_MPI_H

#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef int MPI_Errhandler;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 1
#define MPI_PROC_NULL (-2)
#define MPI_ANY_TAG (-1)
#define MPI_ANY_SOURCE (-1)
#define MPI_MAX_ERROR_STRING 256
#define MPI_THREAD_MULTIPLE 3
#define MPI_ORDER_C 56
#define MPI_ORDER_FORTRAN 57
#define MPI_ERRORS_RETURN 0
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)

/* basic datatypes encode their byte size so that reductions can copy */
#define MPI_INT 4
#define MPI_FLOAT 1004
#define MPI_DOUBLE 1008
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

static inline int girih_stub_type_size(MPI_Datatype t) {
  return (t == MPI_INT) ? 4 : (t == MPI_FLOAT) ? 4 : (t == MPI_DOUBLE) ? 8 : 0;
}

static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Init_thread(int *argc, char ***argv, int req, int *prov) {
  (void)argc; (void)argv; *prov = req; return 0;
}
static inline int MPI_Query_thread(int *prov) { *prov = MPI_THREAD_MULTIPLE; return 0; }
static inline int MPI_Is_thread_main(int *flag) { *flag = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Error_string(int e, char *s, int *len) { (void)e; s[0] = 0; *len = 0; return 0; }
static inline int MPI_Errhandler_set(MPI_Comm c, MPI_Errhandler h) { (void)c; (void)h; return 0; }

static inline double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static inline int MPI_Cart_coords(MPI_Comm c, int rank, int nd, int *coords) {
  (void)c; (void)rank; for (int i = 0; i < nd; i++) coords[i] = 0; return 0;
}

/* Cartesian topology, datatypes and point-to-point messages: oracle/mpi_stub/mpi_stub.c
 * (a rank's messages to itself along periodic dimensions; see there) */
int MPI_Cart_create(MPI_Comm old, int nd, const int *dims, const int *periods, int reorder, MPI_Comm *out);
int MPI_Cart_shift(MPI_Comm c, int dir, int disp, int *src, int *dst);
int MPI_Type_create_subarray(int nd, const int *sizes, const int *subsizes, const int *starts, int order,
                             MPI_Datatype old, MPI_Datatype *out);
int MPI_Type_contiguous(int n, MPI_Datatype old, MPI_Datatype *out);
int MPI_Type_commit(MPI_Datatype *t);
int MPI_Type_free(MPI_Datatype *t);
int MPI_Isend(const void *b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c, MPI_Request *r);
int MPI_Irecv(void *b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Request *r);
int MPI_Send(const void *b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c);
int MPI_Recv(void *b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status *s);
int MPI_Wait(MPI_Request *r, MPI_Status *s);
int MPI_Waitall(int n, MPI_Request *r, MPI_Status *s);
int MPI_Test(MPI_Request *r, int *flag, MPI_Status *s);

static inline int MPI_Reduce(const void *sb, void *rb, int n, MPI_Datatype t, MPI_Op op, int root,
                             MPI_Comm c) {
  (void)op; (void)root; (void)c;
  if (sb != rb) memcpy(rb, sb, (size_t)n * (size_t)girih_stub_type_size(t));
  return 0;
}
static inline int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c) {
  (void)b; (void)n; (void)t; (void)root; (void)c; return 0;
}

#endif
