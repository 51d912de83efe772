// Instantiation of the time-fused kernel for operator 1: FP64 storage, double-float compute.
#include "fused_impl.cuh"

namespace girih {
template <>
cudaError_t launch_fused_op<1, Df64, false>(const Geom &g, const FusedConfig &cfg, const FusedLaunch &L,
                                         cudaStream_t s) {
  return launch_fused_op_impl<1, Df64, false>(g, cfg, L, s);
}
}  // namespace girih
