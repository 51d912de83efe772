// Time-fused (temporally blocked) stencil passes: interface.
#pragma once
#include "internal.cuh"

namespace girih {

// Thread-block shapes of the fused kernel.  A CTA covers an input region of
// columns (tile + halo of depth*R on every side); each thread owns VX x columns
// and CY rows of it and streams the whole z range.  Variants 2 and 3 are
// variants 0 and 1 with the input planes staged into shared memory by TMA
// (FP32 storage; variant 2 switches to x quads at radius-1 depth 4 and
// radius-4 depth 1, variant 3 to a 64 x 64 region with x quads at radius-1
// depth <= 2).  The double-float form numbers its own shapes: 0-4 (see
// variant_shape in fused.cu) and the TMA-staged 5 and 6 below.
enum FusedVariant { FV_64x32_512 = 0, FV_32x64_1024 = 1, FV_64x32_512_TMA = 2, FV_32x64_1024_TMA = 3, FV_COUNT = 7 };

// TMA ring depths: NB planes of the input (and old) state in flight (two for
// deep passes and large regions, whose rings would not fit shared memory
// otherwise), NR planes of roc2 (level l reads roc2 (l-1)*(R+1) planes after
// level 1 did).
__host__ __device__ constexpr int fused_tma_nb(int r, int tt, int area) {
  return (r == 4 || tt >= 4 || area > 2048) ? 2 : 4;
}
__host__ __device__ constexpr int fused_tma_nr(int r, int tt, int nb) {
  int need = (tt - 1) * (r + 1) + nb, p = 1;
  while (p < need) p *= 2;
  return p;
}

// Double-float TMA passes (radius 1, constant coefficients; fused_df_tma.cu):
// one column and two adjacent rows per thread, region df_tma_cols x 32 rows
// (variant 5: 32 columns, variant 6: 64), depth <= 2.  Their rings: the input
// state holds planes s-2 .. s+1 (level 1 reads its x/y neighbours there), in
// 4 slots when the z queues are 4 planes long (time order 2) and 6 when they
// are 3 (so that one unrolled z period, lcm(queue, ring, 2), stays short); the
// old state 2 slots; roc2 2*depth slots (level l reads roc2 of plane s - l*D,
// loaded with the input plane s - (l-1)*D).
__host__ __device__ constexpr int df_tma_cols(int variant) { return variant == 5 ? 32 : 64; }
__host__ __device__ constexpr int df_tma_rows(int) { return 32; }
__host__ __device__ constexpr int df_tma_nb(int to) { return to == 2 ? 4 : 6; }
__host__ __device__ constexpr int df_tma_nr(int tt) { return 2 * tt; }
__host__ __device__ constexpr size_t df_tma_smem(int to, int tt, int cols, int rows) {
  return ((size_t)2 * (tt - 1) * cols * rows * 8 + 127) / 128 * 128 +
         (size_t)(df_tma_nb(to) + (to == 2 ? 2 + df_tma_nr(tt) : 0)) * cols * rows * 8 + (size_t)df_tma_nb(to) * 8;
}

// TMA-staged one-step passes of operator 0 (radius 4; fused_df_tma4.cu),
// variant 5 of the double-float, FP32 and mixed forms: output tile 32 x 32
// (one column and two adjacent rows per thread), TMA boxes of the tile plus
// the radius-4 halo (40 x 40) for the input state, of the tile alone for the
// old state and roc2 (read at the point only); the input state ring holds the
// 2R + 1 planes an update reads and the one in flight, the old state and roc2
// rings 2 slots each.  `esize`: bytes per element (8 double-float, 4 FP32).
__host__ __device__ constexpr int tma4_tile() { return 32; }
__host__ __device__ constexpr int tma4_box() { return 40; }
__host__ __device__ constexpr int tma4_nb() { return 10; }
__host__ __device__ constexpr size_t tma4_smem(int esize) {
  return ((size_t)tma4_nb() * tma4_box() * tma4_box() + (size_t)4 * tma4_tile() * tma4_tile()) * esize +
         (size_t)tma4_nb() * 8;
}

struct FusedConfig {
  int depth = 0;    // time steps per pass (0 = not available)
  int variant = 0;  // FusedVariant
  int bx = 0, by = 0;  // output tile of one CTA
  int box_w = 0, box_h = 0;  // TMA box (region) of the variant, 0 without TMA
  int box2_w = 0, box2_h = 0;  // box of the old state and roc2 where it differs (0: box_w x box_h)
};

struct FusedLaunch {
  const void *prev, *cur;  // states t-1 and t (device layout)
  void *out_prev, *out_cur;  // receive states t+steps-1 and t+steps
  const void *roc2;
  int steps;               // <= config depth
  int write_prev;          // time order 1: write state t+steps-1 (last pass only)
  double cc[5];
  unsigned *range_flag;    // bit 1: a TMA copy did not complete within the wait bound
                           // (bit 0, a value outside the FP32 range, is set by the double-float split)
  const void *tma_cur, *tma_prev, *tma_roc2;  // host CUtensorMap objects (TMA variants)
  int tma_box_w, tma_box_h;                   // the box the maps were encoded with
  int tma_box2_w, tma_box2_h;                 // the old state's and roc2's box
  const void *coef;        // variable coefficients (device layout arrays)
  const float *cscale;     // per-array scales of BF16 coefficients (mixed form)
  const double *src;       // source values per step (null: no source point)
  int src_off;             // device element offset of the source point
  int src_t0, src_n;       // step index of this pass's first level; number of values
  unsigned *cov_prev, *cov_cur;  // checked build: write counters of out_prev / out_cur
};

bool fused_supported(const Geom &g, int precision);
int fused_max_depth(const Geom &g, int precision);
FusedConfig make_fused_config(const Geom &g, int precision, int depth, int variant);
FusedConfig choose_fused_config(const Geom &g, int precision, int depth, int bx, int by);
cudaError_t launch_fused(const Geom &g, int tsz, int precision, const FusedConfig &cfg,
                         const FusedLaunch &L, cudaStream_t s);
const char *fused_kernel_name(int op, int precision, const FusedConfig &cfg);

// double-float TMA passes of operators 1 and 8 (fused_df_tma.cu)
template <int OP>
cudaError_t launch_fused_df_tma(const Geom &g, const FusedConfig &cfg, const FusedLaunch &L, cudaStream_t s);
// TMA-staged one-step passes of operator 0 (fused_df_tma4.cu): double-float,
// and FP32 storage with FP32 (COMP = false) or compensated (mixed) arithmetic
cudaError_t launch_fused_df_tma4(const Geom &g, const FusedConfig &cfg, const FusedLaunch &L, cudaStream_t s);
template <bool COMP>
cudaError_t launch_fused_f32_tma4(const Geom &g, const FusedConfig &cfg, const FusedLaunch &L, cudaStream_t s);

// per-(op, type) launchers defined in the fused_*.cu instantiation files
template <int OP, class T, bool COMP>
cudaError_t launch_fused_op(const Geom &g, const FusedConfig &cfg, const FusedLaunch &L, cudaStream_t s);
#define GIRIH_FUSED_SPEC(OP, T, COMP)                                                       \
  template <>                                                                               \
  cudaError_t launch_fused_op<OP, T, COMP>(const Geom &, const FusedConfig &, const FusedLaunch &, \
                                           cudaStream_t);
GIRIH_FUSED_SPEC(1, double, false)
GIRIH_FUSED_SPEC(1, float, false)
GIRIH_FUSED_SPEC(7, double, false)
GIRIH_FUSED_SPEC(7, float, false)
GIRIH_FUSED_SPEC(8, double, false)
GIRIH_FUSED_SPEC(8, float, false)
GIRIH_FUSED_SPEC(8, float, true)
GIRIH_FUSED_SPEC(0, double, false)
GIRIH_FUSED_SPEC(0, float, false)
GIRIH_FUSED_SPEC(0, float, true)
GIRIH_FUSED_SPEC(2, float, false)
GIRIH_FUSED_SPEC(2, float, true)
GIRIH_FUSED_SPEC(3, float, false)
GIRIH_FUSED_SPEC(3, float, true)
GIRIH_FUSED_SPEC(4, float, false)
GIRIH_FUSED_SPEC(4, float, true)
GIRIH_FUSED_SPEC(5, float, false)
GIRIH_FUSED_SPEC(5, float, true)
struct Df64;
GIRIH_FUSED_SPEC(1, Df64, false)
GIRIH_FUSED_SPEC(8, Df64, false)
GIRIH_FUSED_SPEC(0, Df64, false)
GIRIH_FUSED_SPEC(7, Df64, false)
#undef GIRIH_FUSED_SPEC

}  // namespace girih
