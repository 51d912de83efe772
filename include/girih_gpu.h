/*
 * libgirih_gpu -- GB300 (sm_103a) star-stencil time stepper behind a C ABI.
 *
 * This is the device boundary of the girih stencil hot path.  The reference
 * plugs time steppers into a table of `void (*)(Parameters *)`
 * (src/data_structures.h:412-415, table src/wrappers.h:28-36) and calls them
 * from the performance harness (src/performance.c:75) and the verifier
 * (src/verification.c:37).  A GPU stepper added to that table calls the entry
 * points below; girih_gb300/host/gpu_ts.c is that stepper.
 *
 * Conventions
 *   - every call returns 0 on success or a GIRIH_GPU_E* code; nothing aborts
 *     (the reference's RAISE_ERROR, src/data_structures.h:417-432, exits);
 *     girih_gpu_strerror() names a code, girih_gpu_last_error() gives detail;
 *   - host arrays stay owned by the caller, in the reference layout: x-fastest
 *     (src/kernels/stencils.h:29-32), shape ldomain_shape (interior + 2r halo,
 *     x padded, src/utils.c:367-374), element size host_real_size (real_t);
 *   - the library owns all device memory and copies in and out;
 *   - one context = one grid on one device with one stream; contexts are not
 *     thread-safe, distinct contexts may be used from distinct threads.
 *
 * Operator ids are the reference's --target-kernel ids
 * (src/kernels/stencils.c:260-271) plus GIRIH_OP_STAR7_LEAPFROG:
 *   0  star r=4, time order 2, constant coef (iso_ref, stencils.c:27-41)
 *   1  star r=1, time order 1, constant coef (iso_ref_2space_1time, :73-78)
 *   2  star r=1, variable coef, 2 arrays     (iso_ref_2space_1time_var, :94-99)
 *   3  star r=1, variable axis-symmetric, 4  (..._var_axsym, :121-126)
 *   4  star r=4, variable axis-symmetric, 13 (iso_ref_8space_1time_var_axsym, :148-162)
 *   5  star r=1, variable no-symmetry, 7     (..._var_nosym, :193-201)
 *   7  box 27-point, constant coef, 4 scalars (box_ref_2space_1time, :227-242; plain schedule)
 *   8  star r=1, time order 2, constant coef (radius-1 analogue of 0; no reference id)
 */
#ifndef GIRIH_GPU_H
#define GIRIH_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GIRIH_GPU_ABI_VERSION 1

enum {
  GIRIH_GPU_OK = 0,
  GIRIH_GPU_EINVAL = 1,       /* bad argument or inconsistent shapes */
  GIRIH_GPU_EUNSUPPORTED = 2, /* operator / precision / schedule combination not provided */
  GIRIH_GPU_ECUDA = 3,        /* a CUDA runtime call failed */
  GIRIH_GPU_ENOMEM = 4,       /* device allocation failed */
  GIRIH_GPU_ESTATE = 5,       /* call out of order (e.g. run before upload) */
  GIRIH_GPU_ETIMEOUT = 6,     /* a bounded device-side wait gave up */
  GIRIH_GPU_ENODEV = 7,       /* no usable CUDA device */
  GIRIH_GPU_ERANGE = 8,       /* a value left the range the selected precision can carry */
  GIRIH_GPU_EBOUNDS = 9,      /* bounds-checked build (libgirih_gpu_check.so): a kernel index left
                                 its array or shared-memory block; the access was skipped */
  GIRIH_GPU_ECOVERAGE = 10    /* bounds-checked build: a point was written other than once per step
                                 (or a halo / padding point was written) */
};

enum { GIRIH_OP_STAR7_LEAPFROG = 8 };

enum {
  GIRIH_FP64 = 0,  /* FP64 fields and coefficients, FP64 arithmetic */
  GIRIH_FP32 = 1,  /* FP32 fields and coefficients, FP32 arithmetic */
  GIRIH_MIXED = 2,  /* FP32 fields; variable coefficients in BF16 with a per-array
                      FP32 scale; FP32 accumulation; compensated leapfrog update */
  GIRIH_FP64_DF = 3 /* FP64 fields in HBM; the fused schedule computes in double-float
                      (pairs of FP32, ~48-bit significand; GB300 runs FP32 at 64x its FP64
                      rate); run() returns GIRIH_GPU_ERANGE if a value leaves the FP32
                      exponent range.  The plain schedule is the FP64 kernel. */
};

enum {
  GIRIH_SCHED_PLAIN = 0, /* one time step per kernel launch */
  GIRIH_SCHED_FUSED = 1, /* several time steps per HBM pass (temporal blocking) */
  GIRIH_SCHED_AUTO = 2   /* fused where provided and profitable, else plain */
};

typedef struct {
  int target_kernel;     /* operator id, see above */
  int stencil_shape[3];  /* interior nx, ny, nz (Parameters.lstencil_shape) */
  int ldomain_shape[3];  /* host array shape (Parameters.ldomain_shape) */
  int host_real_size;    /* sizeof(real_t) of the host arrays: 8 or 4 */
  int precision;         /* GIRIH_FP64 / GIRIH_FP32 / GIRIH_MIXED */
  int schedule;          /* GIRIH_SCHED_* */
  int fusion_depth;      /* time steps per pass for the fused schedule; 0 = autotune */
  int block_x, block_y;  /* fused output tile; 0 = autotune */
  int exact;             /* FP64 plain only: 1 = same rounding as the serial reference
                            (no fused multiply-add, reference evaluation order) */
  int device;            /* CUDA device ordinal */
} girih_gpu_desc;

typedef struct {
  int precision, schedule;     /* what run() executes */
  int fusion_depth;            /* time steps per launch (1 for plain) */
  int block_x, block_y;        /* output tile of the fused kernel (0 for plain) */
  int launches_last_run;       /* kernel launches issued by the last run() */
  int steps_last_run;          /* time steps advanced by the last run() */
  double bytes_per_lup;        /* compulsory HBM bytes per lattice update, one step per pass */
  double device_bytes;         /* device memory held by the context */
  char kernel_name[64];        /* dominant kernel of run() */
} girih_gpu_info_t;

typedef struct girih_gpu_ctx girih_gpu_ctx;

/* Context lifetime.  create() validates the descriptor and allocates device
 * memory; nothing is copied yet.  Replaces the reference's per-run
 * arrays_allocate (src/utils.c:153-218) on the device side. */
int girih_gpu_create(girih_gpu_ctx **out, const girih_gpu_desc *d);
void girih_gpu_destroy(girih_gpu_ctx *c);

/* Copy the caller's arrays (reference layout) to the device.  U3 (roc2) is
 * required for time-order-2 operators and ignored otherwise; coef holds r+1
 * scalars for constant operators and n arrays of ldomain size otherwise
 * (COEF macro, src/kernels/stencils.h:32). */
int girih_gpu_upload(girih_gpu_ctx *c, const void *U1, const void *U2, const void *U3,
                     const void *coef);

/* Advance the grid like the reference's steppers: for it in 0..nt step 2
 * { U1 <- op(U2); U2 <- op(U1) } (src/kernels/nb_naive_ts.c:187-203), so odd nt
 * runs nt+1 steps.  Continues from the current device state.  *ms_out (may be
 * NULL) receives the device time of the whole loop from CUDA events on the
 * context's stream; the loop is replayed from a captured CUDA graph. */
int girih_gpu_run(girih_gpu_ctx *c, int nt, float *ms_out);

/* Copy the current U1 (state after steps-1 updates) and U2 (after all steps)
 * back into the caller's arrays (halo included, padding untouched); either
 * pointer may be NULL. */
int girih_gpu_download(girih_gpu_ctx *c, void *U1, void *U2);

/* FP64 device reduction of the current U1 against a reference U1 given in the
 * host layout: out = {max|a-b|, max|b|, sum (a-b)^2, sum b^2} over the
 * interior.  max-norm relative error = out[0]/out[1]. */
int girih_gpu_error_norms(girih_gpu_ctx *c, const void *ref_U1, double out[4]);

/* The same norms between the U1 of two contexts on the same device and grid
 * (a = test, b = reference), without leaving the device. */
int girih_gpu_compare(girih_gpu_ctx *a, girih_gpu_ctx *b, double out[4]);

/* Seeded synthetic initialisation on the device, bit-identical to the CPU
 * oracle's go_fill_seeded(): ranges = {f_lo, f_hi, roc2_lo, roc2_hi, c_lo,
 * c_hi}; const_coefs gives the r+1 scalars of a constant operator.  With
 * GIRIH_SEED_F32_EXACT in flags every value is first rounded to FP32, so FP32
 * and FP64 contexts start from identical data. */
enum { GIRIH_SEED_F32_EXACT = 1 };
int girih_gpu_fill_seeded(girih_gpu_ctx *c, uint64_t seed, const double ranges[6],
                          const double *const_coefs, int flags);

/* Copy the device roc2 array (time-order-2 operators, Parameters.U3) back into
 * the caller's array in the reference layout. */
int girih_gpu_download_roc2(girih_gpu_ctx *c, void *U3);

/* Source-point injection, the reference's per-sweep point update
 * (src/kernels/nb_naive_ts.c:190,196: U(lsource_pt) += source[it]): in every
 * later girih_gpu_run, after sweep s (counted from 0 within the run) the array
 * just updated gets source[s] added at the array point pt = {i, j, k} (indices
 * with the halo, as the reference's lsource_pt, src/utils.c:310).  Sweeps
 * s >= n add nothing; n = 0 or source = NULL switches the update off.  pt must
 * be an interior point (GIRIH_GPU_EINVAL otherwise).  The n values are copied.
 * Every schedule and precision applies it; the value is added in the compute
 * precision after the sweep's own rounding, as the reference does. */
int girih_gpu_set_source(girih_gpu_ctx *c, const int pt[3], const double *source, int n);

int girih_gpu_info(girih_gpu_ctx *c, girih_gpu_info_t *info);

/* Autotuner (replaces the reference's CPU tile auto-tuning, auto_tune_params in
 * src/kernels/diamond_utils.c:691-847): times, on this context's own grid, each
 * candidate the schedule allows -- the plain kernel (GIRIH_SCHED_AUTO only) and
 * every fused tile shape and fusion depth -- over trial_steps steps (0 = a
 * default), keeps the fastest and restores the grid state.  Choices are cached
 * per operator, precision and size class (log2 of the point count), and later
 * contexts created with fusion_depth = 0 and no tile pick them up.  *chosen
 * (may be NULL) receives the result.  After an error return the grid state is
 * unspecified (upload again). */
int girih_gpu_autotune(girih_gpu_ctx *c, int trial_steps, girih_gpu_info_t *chosen);

/* Time-fused stepping without any device allocation.  This entry point has no
 * counterpart in the reference.  It is for callers that cannot call cudaMalloc:
 * a host application that owns the device's memory through its own pool (an
 * allocation behind its back escapes its accounting or fails under its cap), or
 * a code path that must not take the device synchronisation cudaMalloc/cudaFree
 * can cause.  The caller passes its own device arrays U1, U2 (in/out) and U3
 * (roc2, time-order-2 operators) in the reference layout (ldomain_shape,
 * element type FP64 for GIRIH_FP64, FP32 otherwise) and the r+1 constant
 * coefficients; operators 0, 1 and 8; U1 and U2 must carry equal halos; an
 * explicit tile (block_x, block_y) must not name a TMA-staged variant, whose
 * tensor maps only a context keeps (GIRIH_GPU_EUNSUPPORTED).  The
 * call advances nt steps like girih_gpu_run() (U1 = state steps-1, U2 = state
 * steps; halos and x padding of the caller's arrays keep their values) and
 * waits for its work on `stream` (a cudaStream_t, NULL = default stream) to
 * finish before it returns.  The two spare state arrays of the fused schedule
 * live in a static device array of GIRIH_NOALLOC_SCRATCH_BYTES that every GPU
 * loading this library holds until the process exits: grids whose two state
 * arrays do not fit are rejected with GIRIH_GPU_EINVAL.  All calls share that
 * array and it keeps the last call's contents (each call re-initialises what
 * it reads), so calls that overlap on the GPU race: serialise them.  The first
 * call in a device context (and the first after a cudaDeviceReset()) does a
 * one-time set-up, looking up the array's device address; make that first
 * call before any stream capture begins. */
#define GIRIH_NOALLOC_SCRATCH_BYTES (64u << 20)
int girih_gpu_fused_run_noalloc(const girih_gpu_desc *d, void *U1, void *U2, const void *U3,
                                const double *coefs, int nt, void *stream);

/* Batched time stepping (no counterpart in the reference, which advances one
 * grid per process): n independent grids of any sizes, operators 0, 1 and 8,
 * one precision and one device, advanced together by one persistent kernel
 * launch per fused pass that pulls (grid, tile, z chunk) work items from an
 * atomic counter, largest first; the whole time loop is a captured CUDA graph.
 * Each grid is an ordinary context: girih_gpu_batch_grid() returns it for
 * upload / fill_seeded / download / norms. */
typedef struct girih_gpu_batch girih_gpu_batch;
int girih_gpu_batch_create(girih_gpu_batch **out, int n, const girih_gpu_desc *descs);
void girih_gpu_batch_destroy(girih_gpu_batch *b);
girih_gpu_ctx *girih_gpu_batch_grid(girih_gpu_batch *b, int g);
/* Fusion depth per (operator, size class), timed on one grid of each class;
 * grid states are restored. */
int girih_gpu_batch_autotune(girih_gpu_batch *b, int trial_steps);
/* Advance every grid like girih_gpu_run(); *ms_out = device time of the loop. */
int girih_gpu_batch_run(girih_gpu_batch *b, int nt, float *ms_out);
/* The same steps with each grid's own single-grid kernels, one grid after the
 * other (the comparison baseline), also graph-replayed. */
int girih_gpu_batch_run_looped(girih_gpu_batch *b, int nt, float *ms_out);
int girih_gpu_batch_info(girih_gpu_batch *b, int *launches_last_run, int *items_last_run, int *depths);

const char *girih_gpu_strerror(int err);
const char *girih_gpu_last_error(void); /* detail of the calling thread's last error */
int girih_gpu_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif
