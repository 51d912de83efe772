/*
 * TEST INFRASTRUCTURE ONLY: a stand-in for libgirih_gpu.so backed by the CPU
 * oracle, so that the reference-side drop-in (girih_gb300/host/gpu_ts.c and
 * gpu_driver.c) can be exercised end to end on a machine without a GPU.  It
 * implements the entry points the drop-in calls with the declarations of
 * include/girih_gpu.h; the time loop is the oracle's go_run / go_run_source,
 * which reproduce the reference bit for bit.  Never shipped: the product
 * library is girih_gb300/libgirih_gpu.so.
 */
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "girih_gpu.h"
#include "girih_oracle.h"

struct girih_gpu_ctx {
  girih_gpu_desc d;
  int r, to, nc, arr;
  size_t n;  /* elements of one array (ldomain) */
  double *U1, *U2, *U3, *coef;
  size_t ncoef;
  int pt[3];
  double *src;
  int src_n;
  int uploaded;
};

int girih_gpu_create(girih_gpu_ctx **out, const girih_gpu_desc *d) {
  if (!out || !d) return GIRIH_GPU_EINVAL;
  girih_gpu_ctx *c = (girih_gpu_ctx *)calloc(1, sizeof(*c));
  if (!c) return GIRIH_GPU_ENOMEM;
  c->d = *d;
  if (go_op_info(d->target_kernel, &c->r, &c->to, &c->nc, &c->arr) || d->host_real_size != 8) {
    free(c);
    return GIRIH_GPU_EUNSUPPORTED;
  }
  c->n = (size_t)d->ldomain_shape[0] * d->ldomain_shape[1] * d->ldomain_shape[2];
  c->ncoef = c->arr ? (size_t)c->nc * c->n : 11;
  c->U1 = (double *)calloc(c->n, 8);
  c->U2 = (double *)calloc(c->n, 8);
  c->U3 = (double *)calloc(c->n, 8);
  c->coef = (double *)calloc(c->ncoef, 8);
  if (!c->U1 || !c->U2 || !c->U3 || !c->coef) {
    girih_gpu_destroy(c);
    return GIRIH_GPU_ENOMEM;
  }
  *out = c;
  return GIRIH_GPU_OK;
}

void girih_gpu_destroy(girih_gpu_ctx *c) {
  if (!c) return;
  free(c->U1);
  free(c->U2);
  free(c->U3);
  free(c->coef);
  free(c->src);
  free(c);
}

int girih_gpu_upload(girih_gpu_ctx *c, const void *U1, const void *U2, const void *U3, const void *coef) {
  if (!c || !U1 || !U2 || !coef) return GIRIH_GPU_EINVAL;
  memcpy(c->U1, U1, c->n * 8);
  memcpy(c->U2, U2, c->n * 8);
  if (c->to == 2 && U3) memcpy(c->U3, U3, c->n * 8);
  memcpy(c->coef, coef, (c->arr ? c->ncoef : (size_t)c->nc) * 8);  /* nc scalars for constant operators */
  c->uploaded = 1;
  return GIRIH_GPU_OK;
}

int girih_gpu_set_source(girih_gpu_ctx *c, const int pt[3], const double *source, int n) {
  if (!c || n < 0) return GIRIH_GPU_EINVAL;
  free(c->src);
  c->src = NULL;
  c->src_n = 0;
  if (!source || n == 0) return GIRIH_GPU_OK;
  c->src = (double *)malloc(sizeof(double) * (size_t)n);
  if (!c->src) return GIRIH_GPU_ENOMEM;
  memcpy(c->src, source, sizeof(double) * (size_t)n);
  memcpy(c->pt, pt, sizeof(c->pt));
  c->src_n = n;
  return GIRIH_GPU_OK;
}

int girih_gpu_run(girih_gpu_ctx *c, int nt, float *ms_out) {
  if (!c || !c->uploaded) return GIRIH_GPU_ESTATE;
  struct timespec a, b;
  clock_gettime(CLOCK_MONOTONIC, &a);
  const int nx = c->d.stencil_shape[0], ny = c->d.stencil_shape[1], nz = c->d.stencil_shape[2];
  const int pnx = c->d.ldomain_shape[0];
  int e = c->src_n ? go_run_source(c->d.target_kernel, nx, ny, nz, pnx, nt, c->U1, c->U2, c->U3, c->coef, c->pt,
                                   c->src, c->src_n, 1)
                   : go_run(c->d.target_kernel, nx, ny, nz, pnx, nt, c->U1, c->U2, c->U3, c->coef, 1);
  clock_gettime(CLOCK_MONOTONIC, &b);
  if (ms_out) *ms_out = (float)(1e3 * (b.tv_sec - a.tv_sec) + 1e-6 * (b.tv_nsec - a.tv_nsec));
  return e ? GIRIH_GPU_EINVAL : GIRIH_GPU_OK;
}

int girih_gpu_download(girih_gpu_ctx *c, void *U1, void *U2) {
  if (!c || !c->uploaded) return GIRIH_GPU_ESTATE;
  if (U1) memcpy(U1, c->U1, c->n * 8);
  if (U2) memcpy(U2, c->U2, c->n * 8);
  return GIRIH_GPU_OK;
}

int girih_gpu_info(girih_gpu_ctx *c, girih_gpu_info_t *info) {
  if (!c || !info) return GIRIH_GPU_EINVAL;
  memset(info, 0, sizeof(*info));
  info->precision = c->d.precision;
  info->schedule = c->d.schedule;
  info->fusion_depth = c->d.fusion_depth > 0 ? c->d.fusion_depth : 1;
  info->bytes_per_lup = 8.0 * (2 + (c->to == 2 ? 2 : 0) + (c->arr ? c->nc : 0));  /* FP64, one step per pass */
  strcpy(info->kernel_name, "oracle stand-in");
  return GIRIH_GPU_OK;
}

/* The tuner only chooses among schedules that give the same steps; the
 * stand-in has one, so tuning leaves everything as it is. */
int girih_gpu_autotune(girih_gpu_ctx *c, int trial_steps, girih_gpu_info_t *chosen) {
  (void)trial_steps;
  if (!c) return GIRIH_GPU_EINVAL;
  if (!c->uploaded) return GIRIH_GPU_ESTATE;
  return chosen ? girih_gpu_info(c, chosen) : GIRIH_GPU_OK;
}

const char *girih_gpu_strerror(int err) { return err ? "error (oracle stand-in)" : "ok"; }
const char *girih_gpu_last_error(void) { return ""; }
