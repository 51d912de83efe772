// Time-fused (temporally blocked) stencil passes: interface.
#pragma once
#include "internal.cuh"

namespace girih {

// Thread-block shapes of the fused kernel.  A CTA covers an input region of
// NTX x (NTY*CY) columns (tile + halo of depth*R on every side); each thread
// owns one x column and CY rows of it and streams the whole z range.
enum FusedVariant { FV_64x32_512 = 0, FV_32x64_1024 = 1, FV_COUNT = 2 };

struct FusedConfig {
  int depth = 0;    // time steps per pass (0 = not available)
  int variant = 0;  // FusedVariant
  int bx = 0, by = 0;  // output tile of one CTA
};

struct FusedLaunch {
  const void *prev, *cur;  // states t-1 and t (device layout)
  void *out_prev, *out_cur;  // receive states t+steps-1 and t+steps
  const void *roc2;
  int steps;               // <= config depth
  int write_prev;          // time order 1: write state t+steps-1 (last pass only)
  double cc[5];
  unsigned *range_flag;    // double-float compute: set if a value leaves the FP32 exponent range
};

bool fused_supported(const Geom &g, int precision);
int fused_max_depth(const Geom &g, int precision);
FusedConfig make_fused_config(const Geom &g, int precision, int depth, int variant);
FusedConfig choose_fused_config(const Geom &g, int precision, int depth, int bx, int by);
cudaError_t launch_fused(const Geom &g, int tsz, int precision, const FusedConfig &cfg,
                         const FusedLaunch &L, cudaStream_t s);
const char *fused_kernel_name();

// per-(op, type) launchers defined in the fused_*.cu instantiation files
template <int OP, class T, bool COMP>
cudaError_t launch_fused_op(const Geom &g, const FusedConfig &cfg, const FusedLaunch &L, cudaStream_t s);
#define GIRIH_FUSED_SPEC(OP, T, COMP)                                                       \
  template <>                                                                               \
  cudaError_t launch_fused_op<OP, T, COMP>(const Geom &, const FusedConfig &, const FusedLaunch &, \
                                           cudaStream_t);
GIRIH_FUSED_SPEC(1, double, false)
GIRIH_FUSED_SPEC(1, float, false)
GIRIH_FUSED_SPEC(8, double, false)
GIRIH_FUSED_SPEC(8, float, false)
GIRIH_FUSED_SPEC(8, float, true)
GIRIH_FUSED_SPEC(0, double, false)
GIRIH_FUSED_SPEC(0, float, false)
GIRIH_FUSED_SPEC(0, float, true)
struct Df64;
GIRIH_FUSED_SPEC(1, Df64, false)
GIRIH_FUSED_SPEC(8, Df64, false)
GIRIH_FUSED_SPEC(0, Df64, false)
#undef GIRIH_FUSED_SPEC

}  // namespace girih
