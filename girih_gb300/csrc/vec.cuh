// Vector moves of a thread's x group and the preloaded variable coefficients
// of a group, shared by the plain and the fused kernels.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

namespace girih {

// One aligned vector move of N bytes (4, 8 or 16).
template <int N> struct VecBits;
template <> struct VecBits<4> { using type = unsigned; };
template <> struct VecBits<8> { using type = uint2; };
template <> struct VecBits<16> { using type = uint4; };

template <class X, int VX> union VecU {
  typename VecBits<(int)sizeof(X) * VX>::type v;
  X e[VX];
  __device__ __forceinline__ VecU() {}
};

// Variable coefficients of one column of a thread's x group, preloaded for the
// whole group (the accessor of apply_op; the element index is not needed).
template <class T, int NC, int VX, int V> struct CoefGroup {
  const T (&cf)[NC][VX];
  __device__ __forceinline__ T operator()(int m, int64_t) const { return cf[m][V]; }
};

// Load the nc coefficients of VX consecutive columns starting at element e:
// one vector load per array (FP32: 4*VX bytes; BF16: 2*VX bytes, scaled).
template <class T, bool BF16, int NC, int VX>
__device__ __forceinline__ void load_coef_group(const void *coef, int64_t stride, const float *scale, int64_t e,
                                                T (&cf)[NC][VX]) {
#pragma unroll
  for (int m = 0; m < NC; m++) {
    if constexpr (BF16) {
      const __nv_bfloat16 *p = static_cast<const __nv_bfloat16 *>(coef) + m * stride + e;
      const float sc = __ldg(scale + m);
      if constexpr (VX == 1) {
        cf[m][0] = __bfloat162float(p[0]) * sc;
      } else {
        union {
          typename VecBits<2 * VX>::type v;
          __nv_bfloat16 h[VX];
        } u;
        u.v = __ldg(reinterpret_cast<const decltype(u.v) *>(p));
#pragma unroll
        for (int k = 0; k < VX; k++) cf[m][k] = __bfloat162float(u.h[k]) * sc;
      }
    } else {
      VecU<T, VX> u;
      u.v = __ldg(reinterpret_cast<const decltype(u.v) *>(static_cast<const T *>(coef) + m * stride + e));
#pragma unroll
      for (int k = 0; k < VX; k++) cf[m][k] = u.e[k];
    }
  }
}

}  // namespace girih
