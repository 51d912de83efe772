/*
 * C caller of libgirih_gpu -- test program.
 *
 * Does what the reference-side GPU stepper (girih_gb300/host/gpu_ts.c) does,
 * from plain C and without the reference tree: builds arrays with the
 * reference initialisation (CPU oracle restatement), creates a context, uploads,
 * runs nt steps, downloads, and checks U1/U2 bit for bit against the oracle's
 * serial operators (the exact FP64 plain mode).  Exit code 0 = all operators
 * identical.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "girih_gpu.h"
#include "girih_oracle.h"

static int check(int op, int nx, int ny, int nz, int nt) {
  int r, to, nc, arr;
  if (go_op_info(op, &r, &to, &nc, &arr)) return 1;
  int pnx = nx + 2 * r;
  if (pnx % 8) pnx += 8 - pnx % 8; /* the reference's padding, src/utils.c:367-372 */
  size_t n = (size_t)pnx * (ny + 2 * r) * (nz + 2 * r);
  double *U1 = calloc(n, 8), *U2 = calloc(n, 8), *U3 = to == 2 ? calloc(n, 8) : NULL;
  double *coef = calloc(arr ? n * nc : 11, 8);
  double *G1 = calloc(n, 8), *G2 = calloc(n, 8);
  go_fill_ref(op, nx, ny, nz, pnx, U1, U2, U3, coef);

  girih_gpu_desc d;
  memset(&d, 0, sizeof(d));
  d.target_kernel = op;
  d.stencil_shape[0] = nx; d.stencil_shape[1] = ny; d.stencil_shape[2] = nz;
  d.ldomain_shape[0] = pnx; d.ldomain_shape[1] = ny + 2 * r; d.ldomain_shape[2] = nz + 2 * r;
  d.host_real_size = 8;
  d.precision = GIRIH_FP64;
  d.schedule = GIRIH_SCHED_PLAIN;
  d.exact = 1;
  girih_gpu_ctx *c = NULL;
  int e = girih_gpu_create(&c, &d);
  if (!e) e = girih_gpu_upload(c, U1, U2, U3, coef);
  float ms = 0;
  if (!e) e = girih_gpu_run(c, nt, &ms);
  if (!e) e = girih_gpu_download(c, G1, G2);
  if (e) {
    fprintf(stderr, "op %d: %s (%s)\n", op, girih_gpu_strerror(e), girih_gpu_last_error());
    return 1;
  }
  girih_gpu_destroy(c);
  go_run(op, nx, ny, nz, pnx, nt, U1, U2, U3, coef, 1);
  int bad = memcmp(U1, G1, n * 8) != 0 || memcmp(U2, G2, n * 8) != 0;
  printf("op %d %dx%dx%d nt %d: %s (%.3f ms)\n", op, nx, ny, nz, nt, bad ? "DIFFERENT" : "bit-identical", ms);
  free(U1); free(U2); free(U3); free(coef); free(G1); free(G2);
  return bad;
}

int main(void) {
  int fails = 0;
  const int ops[] = {0, 1, 2, 3, 4, 5};
  for (int i = 0; i < 6; i++) fails += check(ops[i], 23, 17, 13, 6);
  return fails ? 1 : 0;
}
