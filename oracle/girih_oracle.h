/*
 * girih CPU oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the girih reference's serial star-stencil operators,
 * its deterministic initialisation and its ping-pong time loop.  It exists to
 * check the GPU library (tests, the smoke check and the CPU baseline leg of the
 * benchmark); the GPU product path never links or calls it.
 *
 * Parity is pinned: the restatement is compared bit-for-bit against golden
 * vectors produced by the unmodified reference code (compiled from its own
 * sources by oracle/Makefile, outputs under oracle/_ref/), see
 * tests/golden/make_golden.py.
 *
 * Layout (reference src/kernels/stencils.h:29-32, src/utils.c:367-374): arrays
 * are x-fastest with shape (pnx, ny+2r, nz+2r) where pnx >= nx+2r is the padded
 * x pitch (the reference's ldomain_shape[0]).  Interior points are
 * [r, nx+r) x [r, ny+r) x [r, nz+r).  Variable-coefficient array m lives at
 * coef + m * pnx*(ny+2r)*(nz+2r) (COEF macro, stencils.h:32).
 */
#ifndef GIRIH_ORACLE_H
#define GIRIH_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Operator ids: 0..5 and 7 are the reference's --target-kernel ids
 * (src/kernels/stencils.c:260-271); 8 is the 7-point, time-order-2 (leapfrog)
 * constant-coefficient operator that has no reference id. */
enum {
  GO_OP_STAR25_CONST_LEAPFROG = 0, /* iso_ref, stencils.c:27-41 */
  GO_OP_STAR7_CONST = 1,           /* iso_ref_2space_1time, stencils.c:73-78 */
  GO_OP_STAR7_VAR = 2,             /* iso_ref_2space_1time_var, stencils.c:94-99 */
  GO_OP_STAR7_VAR_AXSYM = 3,       /* iso_ref_2space_1time_var_axsym, stencils.c:121-126 */
  GO_OP_STAR25_VAR_AXSYM = 4,      /* iso_ref_8space_1time_var_axsym, stencils.c:148-162 */
  GO_OP_STAR7_VAR_NOSYM = 5,       /* iso_ref_2space_1time_var_nosym, stencils.c:193-201 */
  GO_OP_BOX27_CONST = 7,           /* box_ref_2space_1time, stencils.c:227-242 */
  GO_OP_STAR7_CONST_LEAPFROG = 8   /* new: radius-1 analogue of operator 0 */
};

/* Returns 0 and fills radius, time order, number of coefficients (scalars for
 * constant operators, arrays for variable ones) and whether the coefficients
 * are arrays; returns -1 for an unknown or unsupported id. */
int go_op_info(int op, int *radius, int *time_order, int *n_coef, int *coef_is_array);

/* The reference's default coefficient list (src/utils.c:116-119). */
void go_default_coefs(double out[11]);

/* Reference initialisation for one rank (src/utils.c:605-697 domain_data_fill_std,
 * src/utils.c:436-496 init_coeff): ramp interior, +BOUNDARY_SRC_VAL on the two
 * x-boundary planes of U1/U2, roc2 = ramp, coefficients replicated from the
 * default list.  U3 may be NULL for time-order-1 operators; coef must hold
 * r+1 scalars (constant) or n_coef arrays (variable). */
void go_fill_ref(int op, int nx, int ny, int nz, int pnx,
                 double *U1, double *U2, double *U3, double *coef);

/* Counter-based seeded value: SplitMix64 of (seed, stream, idx) mapped to
 * [lo, hi).  Shared bit-for-bit with the GPU library's seeded initialiser. */
double go_seeded_value(uint64_t seed, uint32_t stream, uint64_t idx, double lo, double hi);

/* Seeded initialisation.  Every point of the (nx+2r)(ny+2r)(nz+2r) domain,
 * halo included, gets a value indexed by its unpadded linear index; padding
 * columns are zero.  U1 and U2 get identical field values (stream 0), U3 gets
 * roc2 values (stream 1, [r_lo, r_hi)), variable coefficient array m gets
 * stream 2+m in [c_lo, c_hi).  Constant-coefficient scalars are not touched.
 * round_f32 != 0 rounds every value to the nearest FP32 number (kept as double),
 * so FP32 and FP64 runs can start from identical data.  nthreads > 1 fills
 * with OpenMP; the values do not depend on it. */
void go_fill_seeded(int op, int nx, int ny, int nz, int pnx, uint64_t seed,
                    double f_lo, double f_hi, double r_lo, double r_hi,
                    double c_lo, double c_hi,
                    double *U1, double *U2, double *U3, double *coef, int round_f32, int nthreads);

/* One sweep u <- op(v) over the interior, in the reference's evaluation order
 * (src/verification.c:315-479, 786-819).  Halo and padding are never written.
 * nthreads > 1 parallelises over z with OpenMP; results do not depend on it. */
int go_step(int op, int nx, int ny, int nz, int pnx, const double *coef,
            double *u, const double *v, const double *roc2, int nthreads);

/* The reference time loop (src/verification.c:281-284,
 * src/kernels/nb_naive_ts.c:187-203): for it in 0..nt step 2 { U1 <- op(U2);
 * U2 <- op(U1) }.  Odd nt therefore runs nt+1 sweeps; afterwards U1 holds the
 * state after (sweeps-1) updates and U2 the state after all of them. */
int go_run(int op, int nx, int ny, int nz, int pnx, int nt,
           double *U1, double *U2, const double *U3, const double *coef, int nthreads);

/* go_run with source-point injection (src/kernels/nb_naive_ts.c:190,196):
 * after sweep `it` (0-based within this run) the array just updated gets
 * source[it] added at the point pt = {i, j, k} (array indices, halo included,
 * like the reference's lsource_pt, src/utils.c:310); sweeps it >= nsrc add
 * nothing.  pt must be an interior point.  Returns -3 for a point outside the
 * interior. */
int go_run_source(int op, int nx, int ny, int nz, int pnx, int nt, double *U1, double *U2,
                  const double *U3, const double *coef, const int pt[3], const double *source,
                  int nsrc, int nthreads);

/* Error norms over the interior: out = {max|a-b|, max|b|, sum (a-b)^2, sum b^2}. */
void go_norms(const double *a, const double *b, int nx, int ny, int nz, int pnx, int r,
              double out[4]);

#ifdef __cplusplus
}
#endif
#endif
