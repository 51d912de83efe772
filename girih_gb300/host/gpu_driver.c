/*
 * mwd_kernel driver with the GPU time stepper in its stepper table.
 *
 * Same program flow as the reference driver (src/driver.c:21-82): MPI start,
 * parameter defaults and CLI (--nx/--ny/--nz/--nt/--target-kernel/--target-ts/
 * --verify/...), topology, initialisation, then verification or the
 * performance test.  The only difference is the table below, which the
 * reference defines in src/wrappers.h:28-36: entry 3 is the GPU stepper, so
 * `--target-ts 3` runs the hot path on the GPU and `--list` shows it; after a
 * GPU performance run the rates are also printed in scripts/parse.py's keys.
 */
#include <stdio.h>

#include "data_structures.h"

extern void naive_nonblocking_ts(Parameters *p);
extern void halo_first_ts(Parameters *p);
extern void dynamic_intra_diamond_ts(Parameters *p);
extern void gpu_ts(Parameters *p);
extern void gpu_ts_report(const Parameters *p);

extern void param_default(Parameters *);
extern void parse_args(int argc, char **argv, Parameters *);
extern void mpi_topology_init(Parameters *);
extern void init(Parameters *);
extern void verify(Parameters *);
extern void performance_test(Parameters *p);

struct time_stepper TSList[] = {
    /* 0 */ {"Spatial Blocking", naive_nonblocking_ts},
    /* 1 */ {"Halo-first", halo_first_ts},
    /* 2 */ {"Diamond", dynamic_intra_diamond_ts},
    /* 3 */ {"GPU (libgirih_gpu)", gpu_ts},
    {0, 0},
};

int main(int argc, char **argv) {
  int provided, rank, size;
  MPI_Init_thread(&argc, &argv, MPI_THREAD_MULTIPLE, &provided);
  MPI_Comm_rank(MPI_COMM_WORLD, &rank);
  MPI_Comm_size(MPI_COMM_WORLD, &size);

  Parameters p;
  p.mpi_rank = rank;
  p.mpi_size = size;
  param_default(&p);
  parse_args(argc, argv, &p);

  if (p.t.shape[0] * p.t.shape[1] * p.t.shape[2] != p.mpi_size) {
    if (p.mpi_rank == 0)
      fprintf(stderr, "ERROR: requested MPI topology shape does not match the available processes count\n");
    MPI_Finalize();
    return 1;
  }
  mpi_topology_init(&p);
  init(&p);
  if (p.verify != 0) {
    verify(&p);
  } else {
    performance_test(&p);
    if (TSList[p.target_ts].func == gpu_ts) gpu_ts_report(&p);  /* scripts/parse.py keys */
  }
  MPI_Finalize();
  return 0;
}
