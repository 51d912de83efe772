// Internal declarations shared by the translation units of libgirih_gpu.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/girih_gpu.h"

namespace girih {

// Device-side geometry of one grid.  Reference index (i, j, k), with the halo
// at 0..r-1, maps to  k*plane + j*px + ox + i.  The x offset ox puts the first
// interior column i = r on a 128-byte boundary; the pitch px is a multiple of
// 128 bytes, so every warp-wide row access of the interior is aligned.
struct Geom {
  int op, r, to, nc, var;     // operator id, radius, time order, #coef, variable?
  int nx, ny, nz;             // interior
  int nnx, nny, nnz;          // interior + 2r (unpadded reference extent)
  int hpx;                    // host x pitch (ldomain_shape[0])
  int ox, px;                 // device x offset and pitch, in elements
  int64_t plane;              // px * nny
  int64_t elems;              // plane * nnz
  __host__ __device__ int64_t at(int i, int j, int k) const {
    return (int64_t)k * plane + (int64_t)j * px + ox + i;
  }
};

Geom make_geom(int op, int nx, int ny, int nz, int hpx, int tsz);
int op_info(int op, int *r, int *to, int *nc, int *var);

// Arguments of every single-grid stencil kernel.  Pointers are device-layout
// arrays; coefficient arrays are `nc` consecutive arrays of geom.elems.
template <class T> struct StepArgs {
  Geom g;
  T *u;               // output (for time order 2 also the old value)
  const T *v;         // input state
  const T *roc2;      // time order 2 only
  const void *coef;   // variable coefficients (T or bf16)
  const float *scale; // bf16 per-array scales (mixed precision)
  T cc[5];            // constant coefficients
  const double *src;  // source point: value of this sweep at src[0] (null: no update)
  int64_t src_off;    // device element offset of the source point
  unsigned *flag;     // checked build: error word (bounds violations)
  unsigned *cov;      // checked build: write counters of u
};

// Plain (one step per launch) kernels: plain.cu
template <class T>
cudaError_t launch_plain(const StepArgs<T> &a, bool exact, bool bf16coef, cudaStream_t s);
const char *plain_kernel_name(int op);

// Utility kernels: util.cu
template <class Tin, class Tout>
cudaError_t launch_to_device_layout(const Geom &g, const Tin *src, Tout *dst, cudaStream_t s);
template <class Tin, class Tout>
cudaError_t launch_to_host_layout(const Geom &g, const Tin *src, Tout *dst, cudaStream_t s);
template <class Tin>
cudaError_t launch_maxabs(const Geom &g, const Tin *src_hostlayout, unsigned long long *acc,
                          cudaStream_t s);
template <class Tin>
cudaError_t launch_quantize_bf16(const Geom &g, const Tin *src_hostlayout, __nv_bfloat16 *dst,
                                 const float *scale, cudaStream_t s);
// b is either in host layout (bh, geometry g) or in another device layout (bd, geometry gb)
template <class Ta, class Tb>
cudaError_t launch_norms(const Geom &g, const Ta *a, const Tb *bh, const Geom &gb, const Tb *bd,
                         double *acc, cudaStream_t s);
template <class T>
cudaError_t launch_seeded(const Geom &g, uint64_t seed, uint32_t stream, double lo, double hi,
                          int round_f32, T *dst_devlayout, double *dst_hostlayout, cudaStream_t s);
// FP64 fields <-> double-float pairs (8 bytes per point, same layout).  The
// split writes every element of `in` (halos included) to each non-null output
// and sets bit 0 of *flag for values outside the FP32 exponent range; the join
// writes the interior points of `out` only.
cudaError_t launch_df_split(const Geom &g, const double *in, void *out0, void *out1, void *out2, unsigned *flag,
                            cudaStream_t s);
cudaError_t launch_df_join(const Geom &g, const void *in, double *out, cudaStream_t s);
cudaError_t launch_halo_equal(const Geom &g, const void *a, const void *b, int tsz,
                              unsigned int *flag, cudaStream_t s);
// Checked build: every interior point of a buffer must have been written
// `expect` times and no other point at all (else kFlagCoverage in *flag); the
// counters are cleared for the next run.
cudaError_t launch_coverage_check(const Geom &g, unsigned *cov, unsigned expect, unsigned *flag, cudaStream_t s);

// Per-thread error detail.
void set_error(const std::string &msg);

}  // namespace girih
