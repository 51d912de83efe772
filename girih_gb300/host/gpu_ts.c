/*
 * GPU time stepper for the girih driver: the entry
 *     {"GPU (libgirih_gpu)", gpu_ts}
 * of the time-stepper table (reference: struct time_stepper,
 * src/data_structures.h:412-415; table src/wrappers.h:28-36).  It has the
 * signature of every reference stepper, void (*)(Parameters *), and is called
 * the same way: by the performance harness inside its MPI_Wtime bracket
 * (src/performance.c:74-78) and by the verifier (src/verification.c:37), which
 * then compares p->U1 with the serial reference operators.
 *
 * Each call advances p->U1/p->U2 by nt steps exactly like
 * naive_nonblocking_ts (src/kernels/nb_naive_ts.c:187-203): the host arrays are
 * copied to the GPU, the time loop runs there, and U1 (state nt-1) and U2
 * (state nt) are copied back.  The reference CLI has no precision or schedule
 * options, so they come from the environment:
 *   GIRIH_GPU_PRECISION = fp64 (default) | fp32 | mixed | fp64df (FP64 fields, fused
 *                         passes in double-float arithmetic)
 *   GIRIH_GPU_SCHEDULE  = plain (default) | fused | auto
 *   GIRIH_GPU_EXACT     = 1 (default for fp64 plain: the serial reference's rounding,
 *                         so --verify 1 passes its bit-exact check) | 0
 *   GIRIH_GPU_DEVICE    = CUDA device ordinal (default 0)
 *   GIRIH_GPU_AUTOTUNE  = 1: time the tile shapes and fusion depths on this grid
 *                         (girih_gpu_autotune, the counterpart of the MWD
 *                         auto-tuner, src/kernels/diamond_utils.c:691-847) when
 *                         the stepper first sees a grid; the state is restored,
 *                         but that first call's time includes the tuning
 * The MWD option --t-dim (diamond time unroll, default -1 = tune) sets the
 * fusion depth of the fused schedule to t_dim + 1 time steps per pass (clamped
 * to the deepest pass provided for the operator and precision).
 * Errors are reported through the reference's RAISE_ERROR.
 *
 * gpu_ts_report() prints the run's rates in the key format of the reference's
 * scripts/parse.py (get_summary: "RANK0 MStencil/s  MIN/AVG/MAX"), which the
 * reference's own report no longer emits (it prints GStencil/s,
 * src/utils.c:872-875), so the existing plotting scripts ingest GPU runs.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "data_structures.h"
#include "girih_gpu.h"

static girih_gpu_ctx *g_ctx = NULL;
static girih_gpu_desc g_desc;
static const char *const precisions[] = {"fp64", "fp32", "mixed", "fp64df"};  /* GIRIH_FP64 .. GIRIH_FP64_DF */
static const char *const schedules[] = {"plain", "fused", "auto"};

/* per-call wall time (the span the reference's MPI_Wtime bracket measures,
 * src/performance.c:74-78) and device time, over all calls */
static struct {
  int calls;
  double wall_min, wall_max, wall_sum, dev_min;
} g_stats;

static double wall_now(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static int env_choice(const char *name, const char *const *names, int n, int def) {
  const char *v = getenv(name);
  if (!v || !*v) return def;
  for (int i = 0; i < n; i++)
    if (strcmp(v, names[i]) == 0) return i;
  fprintf(stderr, "ERROR: %s=%s is not one of the accepted values\n", name, v);
  exit(1);
}

static void gpu_ts_release(void) {
  if (g_ctx) girih_gpu_destroy(g_ctx);
  g_ctx = NULL;
}

static void gpu_ts_fail(Parameters *p, const char *what, int err) {
  if (p->mpi_rank == 0)
    fprintf(stderr, "ERROR: %s: %s (%s)\n", what, girih_gpu_strerror(err), girih_gpu_last_error());
  gpu_ts_release();
  RAISE_ERROR("GPU time stepper failed");
}

void gpu_ts(Parameters *p) {
  const double t0 = wall_now();
  if (p->mpi_size != 1) RAISE_ERROR("the GPU time stepper runs one grid per process: use a single rank");
  /* the regular operators: the star ones and the 27-point box (kernel 7); the
   * solar kernel (SOLAR type) is not provided */
  if (p->stencil.type != REGULAR || (p->stencil.shape != STAR && p->stencil.shape != BOX))
    RAISE_ERROR("the GPU time stepper provides the star and box operators only");

  girih_gpu_desc d;
  memset(&d, 0, sizeof(d));
  d.target_kernel = p->target_kernel;
  for (int i = 0; i < 3; i++) {
    d.stencil_shape[i] = p->lstencil_shape[i];
    d.ldomain_shape[i] = p->ldomain_shape[i];
  }
  d.host_real_size = (int)sizeof(real_t);
  d.precision = env_choice("GIRIH_GPU_PRECISION", precisions, 4, GIRIH_FP64);
  d.schedule = env_choice("GIRIH_GPU_SCHEDULE", schedules, 3, GIRIH_SCHED_PLAIN);
  const char *ex = getenv("GIRIH_GPU_EXACT");
  d.exact = ex ? atoi(ex) != 0 : (d.precision == GIRIH_FP64 && d.schedule == GIRIH_SCHED_PLAIN);
  const char *dev = getenv("GIRIH_GPU_DEVICE");
  d.device = dev ? atoi(dev) : 0;
  if (p->t_dim >= 0) d.fusion_depth = p->t_dim + 1;
  const char *tune = getenv("GIRIH_GPU_AUTOTUNE");
  const int autotune = tune && atoi(tune) != 0;

  if (g_ctx && memcmp(&d, &g_desc, sizeof(d)) != 0) gpu_ts_release();
  int e, fresh = 0;
  if (!g_ctx) {
    if ((e = girih_gpu_create(&g_ctx, &d))) {
      g_ctx = NULL;
      gpu_ts_fail(p, "girih_gpu_create", e);
    }
    g_desc = d;
    fresh = 1;
    atexit(gpu_ts_release);
  }
  if ((e = girih_gpu_upload(g_ctx, p->U1, p->U2, p->U3, p->coef))) gpu_ts_fail(p, "girih_gpu_upload", e);
  if (fresh && autotune) {
    girih_gpu_info_t tuned;
    if ((e = girih_gpu_autotune(g_ctx, 0, &tuned))) gpu_ts_fail(p, "girih_gpu_autotune", e);
    if (p->verbose && p->mpi_rank == 0)
      printf("GPU stepper autotune: %s schedule, depth %d, tile %d x %d\n",
             tuned.schedule == GIRIH_SCHED_PLAIN ? "plain" : "fused", tuned.fusion_depth, tuned.block_x,
             tuned.block_y);
  }
  /* the reference's source-point update (nb_naive_ts.c:190,196), when switched on */
  if (p->source_point_enabled == 1 && p->has_source == 1 && p->source && p->nt > 0) {
    double *src = (double *)malloc(sizeof(double) * (size_t)p->nt);
    if (!src) RAISE_ERROR("host allocation failed");
    for (int i = 0; i < p->nt; i++) src[i] = (double)p->source[i];
    e = girih_gpu_set_source(g_ctx, p->lsource_pt, src, p->nt);
    free(src);
    if (e) gpu_ts_fail(p, "girih_gpu_set_source", e);
  } else if ((e = girih_gpu_set_source(g_ctx, NULL, NULL, 0))) {
    gpu_ts_fail(p, "girih_gpu_set_source", e);
  }
  float ms = 0.f;
  if ((e = girih_gpu_run(g_ctx, p->nt, &ms))) gpu_ts_fail(p, "girih_gpu_run", e);
  if ((e = girih_gpu_download(g_ctx, p->U1, p->U2))) gpu_ts_fail(p, "girih_gpu_download", e);

  /* the device time of the loop is the stepper's compute time
   * (the reference accumulates it the same way, nb_naive_ts.c:205-206) */
  p->prof.compute += ms * 1e-3;
  const double wall = wall_now() - t0;
  if (g_stats.calls == 0 || wall < g_stats.wall_min) g_stats.wall_min = wall;
  if (g_stats.calls == 0 || wall > g_stats.wall_max) g_stats.wall_max = wall;
  if (g_stats.calls == 0 || ms * 1e-3 < g_stats.dev_min) g_stats.dev_min = ms * 1e-3;
  g_stats.wall_sum += wall;
  g_stats.calls++;
  if (p->verbose && p->mpi_rank == 0) {
    girih_gpu_info_t info;
    girih_gpu_info(g_ctx, &info);
    int steps = 2 * ((p->nt + 1) / 2);
    printf("GPU stepper: %s %s depth %d, %d launches, device time %.3f ms, %.3f GLUP/s (device only)\n",
           precisions[info.precision], schedules[info.schedule], info.fusion_depth, info.launches_last_run, ms,
           ms > 0 ? (double)p->ln_stencils * steps / (ms * 1e6) : 0.0);
  }
}

/* Rates of the calls so far in scripts/parse.py's keys (MStencil/s per time
 * step: ln_stencils * nt / time, the reference's GStencil/s x 1000), plus the
 * device-only rate of the fastest call, then one machine-readable line (prefix
 * "GPU stepper JSON: ") with the form the library ran, its compulsory bytes
 * per lattice update and the algorithmic HBM rate they imply. */
void gpu_ts_report(const Parameters *p) {
  if (p->mpi_rank != 0 || g_stats.calls == 0) return;
  const double per_step = (double)p->ln_stencils * p->nt / 1e6;
  printf("RANK0 MStencil/s  MIN: %f\n", per_step / g_stats.wall_max);
  printf("RANK0 MStencil/s  AVG: %f\n", per_step / (g_stats.wall_sum / g_stats.calls));
  printf("RANK0 MStencil/s  MAX: %f\n", per_step / g_stats.wall_min);
  if (g_stats.dev_min > 0) printf("GPU device MStencil/s MAX: %f\n", per_step / g_stats.dev_min);
  girih_gpu_info_t info;
  if (!g_ctx || girih_gpu_info(g_ctx, &info) != 0) return;
  const double glups_wall = per_step / g_stats.wall_min / 1e3;
  const double glups_dev = g_stats.dev_min > 0 ? per_step / g_stats.dev_min / 1e3 : 0.0;
  const int prec = info.precision >= 0 && info.precision <= GIRIH_FP64_DF ? info.precision : 0;
  const int sched = info.schedule >= 0 && info.schedule <= GIRIH_SCHED_AUTO ? info.schedule : 0;
  printf("GPU stepper JSON: {\"stepper\": \"GPU (libgirih_gpu)\", \"target_kernel\": %d, "
         "\"grid\": [%d, %d, %d], \"nt\": %d, \"calls\": %d, \"precision\": \"%s\", \"schedule\": \"%s\", "
         "\"fusion_depth\": %d, \"tile\": [%d, %d], \"kernel\": \"%s\", \"bytes_per_lup\": %.1f, "
         "\"glups_wall_max\": %.6g, \"glups_device_max\": %.6g, \"algorithmic_gbs_device\": %.6g}\n",
         p->target_kernel, p->lstencil_shape[0], p->lstencil_shape[1], p->lstencil_shape[2], p->nt, g_stats.calls,
         precisions[prec], schedules[sched], info.fusion_depth, info.block_x, info.block_y, info.kernel_name,
         info.bytes_per_lup, glups_wall, glups_dev, glups_dev * info.bytes_per_lup);
}
