/*
 * Golden-vector harness -- TEST INFRASTRUCTURE ONLY.
 *
 * Links the unmodified girih reference objects (compiled from the reference's
 * own sources by oracle/Makefile) and runs the reference's own time stepper on
 * the reference's own data structures, then writes the resulting U1 and U2
 * arrays (full padded local domain, real_t = double) to a file.  The output is
 * the known answer the CPU oracle restatement is pinned against.
 *
 * Usage:
 *   ref_golden <kernel> <nx> <ny> <nz> <nt> <ts> <init> <out.bin>
 *              [seed f_lo f_hi r_lo r_hi c_lo c_hi [c0 c1 c2 c3 c4]]
 *   init = "ref"    : the reference's own initialisation (utils.c:436-497, 605-697)
 *   init = "seeded" : fields / roc2 / coefficient arrays overwritten with the
 *                     oracle's seeded values after the reference's allocation;
 *                     optional c0..c4 replace the constant coefficients.
 * With GIRIH_REF_SOURCE=1 in the environment the reference's source-point
 * update runs (src/kernels/nb_naive_ts.c:190,196): the point is the
 * reference's centred source (src/utils.c:247-251, 302-315) and the values are
 * the reference's source[i] = i (src/performance.c:53-54).  The reference's
 * init() switches the update off (src/utils.c:336); the harness switches it
 * back on after init.
 * Prints "ldomain <nnx> <nny> <nnz> nt <nt> source <i> <j> <k>" on stdout.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "data_structures.h" /* reference: src/data_structures.h */
#include "girih_oracle.h"

/* Reference entry points (src/utils.c, src/mpi_utils.c, src/kernels/ *_ts.c). */
extern void param_default(Parameters *);
extern void mpi_topology_init(Parameters *);
extern void init(Parameters *);
extern void mpi_halo_init(Parameters *);
extern void mpi_halo_finalize(Parameters *);
extern void arrays_allocate(Parameters *);
extern void arrays_free(Parameters *);
extern void init_coeff(Parameters *);
extern void domain_data_fill(Parameters *);
extern void set_centered_source(Parameters *);
extern void naive_nonblocking_ts(Parameters *);
extern void halo_first_ts(Parameters *);
extern void dynamic_intra_diamond_ts(Parameters *);

/* The stepper table the reference's driver defines in src/wrappers.h:28-36;
 * this harness does not link driver.c, so it provides the same table. */
struct time_stepper TSList[] = {
    {"Spatial Blocking", naive_nonblocking_ts},
    {"Halo-first", halo_first_ts},
    {"Diamond", dynamic_intra_diamond_ts},
    {0, 0},
};

int main(int argc, char **argv) {
  if (argc < 9) {
    fprintf(stderr, "usage: %s kernel nx ny nz nt ts ref|seeded out.bin [...]\n", argv[0]);
    return 2;
  }
  Parameters p;
  memset(&p, 0, sizeof(p));
  p.mpi_rank = 0;
  p.mpi_size = 1;
  param_default(&p);
  p.target_kernel = atoi(argv[1]);
  p.stencil_shape[0] = atoi(argv[2]);
  p.stencil_shape[1] = atoi(argv[3]);
  p.stencil_shape[2] = atoi(argv[4]);
  p.nt = atoi(argv[5]);
  p.target_ts = atoi(argv[6]);
  const char *mode = argv[7];
  const char *out = argv[8];
  p.verbose = 0;
  p.n_tests = 1;
  p.num_threads = 2;
  p.stencil_ctx.thread_group_size = 2;
  p.orig_thread_group_size = 2;

  set_centered_source(&p);
  mpi_topology_init(&p);
  init(&p);
  mpi_halo_init(&p);
  arrays_allocate(&p);
  init_coeff(&p);
  domain_data_fill(&p);

  if (strcmp(mode, "seeded") == 0) {
    if (argc < 16) {
      fprintf(stderr, "seeded mode needs seed f_lo f_hi r_lo r_hi c_lo c_hi\n");
      return 2;
    }
    unsigned long long seed = strtoull(argv[9], 0, 10);
    double v[6];
    for (int i = 0; i < 6; i++) v[i] = atof(argv[10 + i]);
    int op = p.target_kernel, r, to, nc, arr;
    if (go_op_info(op, &r, &to, &nc, &arr)) return 3;
    go_fill_seeded(op, p.stencil_shape[0], p.stencil_shape[1], p.stencil_shape[2],
                   p.ldomain_shape[0], seed, v[0], v[1], v[2], v[3], v[4], v[5], p.U1, p.U2,
                   p.U3, p.coef, 0, 1);
    if (!arr)
      for (int i = 0; i < nc && 16 + i < argc; i++) p.coef[i] = atof(argv[16 + i]);
  } else if (strcmp(mode, "ref") != 0) {
    fprintf(stderr, "unknown init mode %s\n", mode);
    return 2;
  }

  const char *src_env = getenv("GIRIH_REF_SOURCE");
  const int with_source = src_env && atoi(src_env) == 1;
  if (with_source) {
    p.source_point_enabled = 1;
    /* nt + 1 values: the stepper reads source[nt] after the extra sweep of an odd nt */
    p.source = (real_t *)malloc(sizeof(real_t) * (size_t)(p.nt + 1));
    if (!p.source) return 5;
    for (int i = 0; i <= p.nt; i++) p.source[i] = i < p.nt ? (real_t)i : 0;
  }

  TSList[p.target_ts].func(&p);

  FILE *f = fopen(out, "wb");
  if (!f) return 4;
  fwrite(p.U1, sizeof(real_t), p.ln_domain, f);
  fwrite(p.U2, sizeof(real_t), p.ln_domain, f);
  fclose(f);
  printf("ldomain %d %d %d nt %d source %d %d %d\n", p.ldomain_shape[0], p.ldomain_shape[1],
         p.ldomain_shape[2], p.nt, with_source ? p.lsource_pt[0] : -1, with_source ? p.lsource_pt[1] : -1,
         with_source ? p.lsource_pt[2] : -1);
  arrays_free(&p);
  mpi_halo_finalize(&p);
  return 0;
}
