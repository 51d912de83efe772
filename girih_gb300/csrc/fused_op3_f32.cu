// Instantiation of the time-fused kernel for operator 3 (variable coefficients), FP32 fields, FP32 coefficients.
#include "fused_impl.cuh"

namespace girih {
template <>
cudaError_t launch_fused_op<3, float, false>(const Geom &g, const FusedConfig &cfg, const FusedLaunch &L,
                                          cudaStream_t s) {
  return launch_fused_op_impl<3, float, false>(g, cfg, L, s);
}
}  // namespace girih
