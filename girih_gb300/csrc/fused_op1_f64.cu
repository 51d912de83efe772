// Instantiation of the time-fused kernel for operator 1, double.
#include "fused_impl.cuh"

namespace girih {
template <>
cudaError_t launch_fused_op<1, double, false>(const Geom &g, const FusedConfig &cfg, const FusedLaunch &L,
                                          cudaStream_t s) {
  return launch_fused_op_impl<1, double, false>(g, cfg, L, s);
}
}  // namespace girih
