/*
 * Single-rank MPI runtime behind oracle/mpi_stub/mpi.h -- test and baseline
 * infrastructure only (linked into the reference builds under oracle/_ref/).
 *
 * With one rank the only messages are a rank's messages to itself.  The
 * reference makes the y direction of its Cartesian topology periodic for the
 * diamond (MWD) time stepper (src/mpi_utils.c:66-80), so on one rank the
 * diamond halo exchanges (src/kernels/diamond_ts.c:128-290) send strided halo
 * regions, described by subarray datatypes (src/mpi_utils.c:257-319), from the
 * grid to itself.  This file carries those messages: Cartesian neighbours are
 * the rank itself along periodic dimensions and MPI_PROC_NULL otherwise;
 * datatypes are the basic ones, contiguous runs and 3-d subarrays; a send packs
 * its data when it is posted; a receive takes the earliest pending message
 * from the same communicator whose tag it accepts, and a message the earliest
 * matching pending receive (MPI's non-overtaking order for one source).
 * Waits block (the reference posts sends and receives from several OpenMP
 * threads) and give up with an error after a bounded time.
 */
#include "mpi.h"

#include <pthread.h>
#include <sched.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

enum { MAX_TYPES = 1024, MAX_REQS = 4096, KIND_SUBARRAY = 1, KIND_CONTIG = 2 };

typedef struct {
  int used, kind, elem;
  int nd, order, sizes[3], subsizes[3], starts[3];
  int count; /* contiguous: elements */
} stub_type;

typedef struct {
  int used, done, is_send;
  int waited; /* a send whose handle was completed while its message was still queued */
  MPI_Comm comm;
  int tag;
  /* send: the packed message; receive: where to unpack */
  char *msg;
  size_t bytes;
  void *buf;
  int count;
  MPI_Datatype type;
  long seq; /* posting order */
} stub_req;

static pthread_mutex_t g_lock = PTHREAD_MUTEX_INITIALIZER;
static stub_type g_types[MAX_TYPES];
static stub_req g_reqs[MAX_REQS];
static long g_seq;
static int g_periods[3];

#define TYPE_BASE 10000

static int basic_size(MPI_Datatype t) { return girih_stub_type_size(t); }

static stub_type *derived(MPI_Datatype t) {
  if (t < TYPE_BASE || t >= TYPE_BASE + MAX_TYPES) return NULL;
  stub_type *d = &g_types[t - TYPE_BASE];
  return d->used ? d : NULL;
}

static size_t type_bytes(MPI_Datatype t) {
  const stub_type *d = derived(t);
  if (!d) return (size_t)basic_size(t);
  if (d->kind == KIND_CONTIG) return (size_t)d->count * d->elem;
  size_t n = (size_t)d->elem;
  for (int i = 0; i < d->nd; i++) n *= (size_t)d->subsizes[i];
  return n;
}

/* Visit the contiguous runs of `count` items of type t in buf, in type order. */
static void copy_runs(const stub_type *d, char *base, char *flat, int to_flat) {
  /* dims in fastest-first order */
  int sz[3] = {1, 1, 1}, sub[3] = {1, 1, 1}, st[3] = {0, 0, 0};
  for (int i = 0; i < d->nd; i++) {
    const int k = d->order == MPI_ORDER_FORTRAN ? i : d->nd - 1 - i;
    sz[i] = d->sizes[k];
    sub[i] = d->subsizes[k];
    st[i] = d->starts[k];
  }
  const size_t run = (size_t)sub[0] * d->elem;
  size_t off = 0;
  for (int c = 0; c < sub[2]; c++)
    for (int b = 0; b < sub[1]; b++) {
      const size_t at = (((size_t)(st[2] + c) * sz[1] + (size_t)(st[1] + b)) * sz[0] + (size_t)st[0]) * d->elem;
      if (to_flat) memcpy(flat + off, base + at, run);
      else memcpy(base + at, flat + off, run);
      off += run;
    }
}

static void pack(const void *buf, int count, MPI_Datatype t, char *out) {
  const stub_type *d = derived(t);
  if (!d || d->kind == KIND_CONTIG) {
    memcpy(out, buf, (size_t)count * type_bytes(t));
    return;
  }
  const size_t one = type_bytes(t);
  for (int i = 0; i < count; i++) copy_runs(d, (char *)buf, out + i * one, 1);
}

static void unpack(void *buf, int count, MPI_Datatype t, const char *in) {
  const stub_type *d = derived(t);
  if (!d || d->kind == KIND_CONTIG) {
    memcpy(buf, in, (size_t)count * type_bytes(t));
    return;
  }
  const size_t one = type_bytes(t);
  for (int i = 0; i < count; i++) copy_runs(d, (char *)buf, (char *)in + i * one, 0);
}

static int new_req(void) {
  for (int i = 0; i < MAX_REQS; i++)
    if (!g_reqs[i].used) {
      memset(&g_reqs[i], 0, sizeof(g_reqs[i]));
      g_reqs[i].used = 1;
      g_reqs[i].seq = g_seq++;
      return i + 1;
    }
  fprintf(stderr, "single-rank MPI stub: out of request slots\n");
  abort();
}

static int tag_ok(int want, int have) { return want == MPI_ANY_TAG || want == have; }

/* deliver a packed message into a posted receive; the lock is held */
static void deliver(stub_req *send, stub_req *recv) {
  const size_t cap = (size_t)recv->count * type_bytes(recv->type);
  if (send->bytes > cap) {
    fprintf(stderr, "single-rank MPI stub: message of %zu bytes into a %zu-byte receive\n", send->bytes, cap);
    abort();
  }
  unpack(recv->buf, recv->count, recv->type, send->msg);
  free(send->msg);
  send->msg = NULL;
  send->done = recv->done = 1;
  if (send->waited) send->used = 0;
}

int MPI_Cart_create(MPI_Comm old, int nd, const int *dims, const int *periods, int reorder, MPI_Comm *out) {
  (void)old;
  (void)dims;
  (void)reorder;
  pthread_mutex_lock(&g_lock);
  for (int i = 0; i < nd && i < 3; i++) g_periods[i] = periods ? periods[i] : 0;
  pthread_mutex_unlock(&g_lock);
  *out = MPI_COMM_WORLD;
  return 0;
}

int MPI_Cart_shift(MPI_Comm c, int dir, int disp, int *src, int *dst) {
  (void)c;
  (void)disp;
  const int self = dir >= 0 && dir < 3 && g_periods[dir];
  *src = self ? 0 : MPI_PROC_NULL;
  *dst = self ? 0 : MPI_PROC_NULL;
  return 0;
}

int MPI_Type_create_subarray(int nd, const int *sizes, const int *subsizes, const int *starts, int order,
                             MPI_Datatype old, MPI_Datatype *out) {
  if (nd < 1 || nd > 3 || derived(old)) return 1;
  pthread_mutex_lock(&g_lock);
  for (int i = 0; i < MAX_TYPES; i++)
    if (!g_types[i].used) {
      stub_type *d = &g_types[i];
      memset(d, 0, sizeof(*d));
      d->used = 1;
      d->kind = KIND_SUBARRAY;
      d->elem = basic_size(old);
      d->nd = nd;
      d->order = order;
      for (int k = 0; k < 3; k++) {
        d->sizes[k] = k < nd ? sizes[k] : 1;
        d->subsizes[k] = k < nd ? subsizes[k] : 1;
        d->starts[k] = k < nd ? starts[k] : 0;
      }
      *out = TYPE_BASE + i;
      pthread_mutex_unlock(&g_lock);
      return 0;
    }
  pthread_mutex_unlock(&g_lock);
  return 1;
}

int MPI_Type_contiguous(int n, MPI_Datatype old, MPI_Datatype *out) {
  if (derived(old)) return 1;
  pthread_mutex_lock(&g_lock);
  for (int i = 0; i < MAX_TYPES; i++)
    if (!g_types[i].used) {
      stub_type *d = &g_types[i];
      memset(d, 0, sizeof(*d));
      d->used = 1;
      d->kind = KIND_CONTIG;
      d->elem = basic_size(old);
      d->count = n;
      *out = TYPE_BASE + i;
      pthread_mutex_unlock(&g_lock);
      return 0;
    }
  pthread_mutex_unlock(&g_lock);
  return 1;
}

int MPI_Type_commit(MPI_Datatype *t) {
  (void)t;
  return 0;
}

int MPI_Type_free(MPI_Datatype *t) {
  pthread_mutex_lock(&g_lock);
  stub_type *d = derived(*t);
  if (d) d->used = 0;
  pthread_mutex_unlock(&g_lock);
  return 0;
}

int MPI_Isend(const void *b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c, MPI_Request *r) {
  pthread_mutex_lock(&g_lock);
  const int id = new_req();
  stub_req *s = &g_reqs[id - 1];
  s->is_send = 1;
  s->comm = c;
  s->tag = tag;
  if (dst == MPI_PROC_NULL) {
    s->done = 1;
  } else {
    s->bytes = (size_t)n * type_bytes(t);
    s->msg = (char *)malloc(s->bytes ? s->bytes : 1);
    if (!s->msg) abort();
    pack(b, n, t, s->msg);
    /* the earliest pending receive that accepts it */
    stub_req *best = NULL;
    for (int i = 0; i < MAX_REQS; i++) {
      stub_req *q = &g_reqs[i];
      if (q->used && !q->is_send && !q->done && q->comm == c && tag_ok(q->tag, tag) && (!best || q->seq < best->seq))
        best = q;
    }
    if (best) deliver(s, best);
  }
  *r = id;
  pthread_mutex_unlock(&g_lock);
  return 0;
}

int MPI_Irecv(void *b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Request *r) {
  pthread_mutex_lock(&g_lock);
  const int id = new_req();
  stub_req *q = &g_reqs[id - 1];
  q->comm = c;
  q->tag = tag;
  q->buf = b;
  q->count = n;
  q->type = t;
  if (src == MPI_PROC_NULL) {
    q->done = 1;
  } else {
    /* the earliest pending message it accepts */
    stub_req *best = NULL;
    for (int i = 0; i < MAX_REQS; i++) {
      stub_req *s = &g_reqs[i];
      if (s->used && s->is_send && s->msg && s->comm == c && tag_ok(tag, s->tag) && (!best || s->seq < best->seq))
        best = s;
    }
    if (best) deliver(best, q);
  }
  *r = id;
  pthread_mutex_unlock(&g_lock);
  return 0;
}

/* Complete request r if it can be; the lock is held.  A send completes once
 * its data are packed (its buffer may be reused); its slot lives on while the
 * message waits for a receive. */
static int try_complete(MPI_Request *r) {
  if (*r < 1 || *r > MAX_REQS) return 1;
  stub_req *q = &g_reqs[*r - 1];
  if (!q->used) return 1;
  if (q->is_send) {
    if (q->msg) q->waited = 1;
    else q->used = 0;
  } else if (q->done) {
    q->used = 0;
  } else {
    return 0;
  }
  *r = 0;
  return 1;
}

int MPI_Test(MPI_Request *r, int *flag, MPI_Status *st) {
  (void)st;
  pthread_mutex_lock(&g_lock);
  *flag = try_complete(r);
  pthread_mutex_unlock(&g_lock);
  return 0;
}

int MPI_Wait(MPI_Request *r, MPI_Status *st) {
  (void)st;
  /* a receive completes when a thread posts its message: wait for it, boundedly
   * (about a minute) */
  for (long spins = 0;; spins++) {
    pthread_mutex_lock(&g_lock);
    const int done = try_complete(r);
    pthread_mutex_unlock(&g_lock);
    if (done) return 0;
    if (spins > 40000000L) {
      fprintf(stderr, "single-rank MPI stub: a receive was never matched\n");
      abort();
    }
    sched_yield();
  }
}

int MPI_Waitall(int n, MPI_Request *r, MPI_Status *st) {
  for (int i = 0; i < n; i++) MPI_Wait(&r[i], st ? &st[i] : NULL);
  return 0;
}

int MPI_Send(const void *b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c) {
  MPI_Request r;
  MPI_Isend(b, n, t, dst, tag, c, &r);
  return MPI_Wait(&r, NULL);
}

int MPI_Recv(void *b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status *s) {
  MPI_Request r;
  MPI_Irecv(b, n, t, src, tag, c, &r);
  return MPI_Wait(&r, s);
}
