// Star-stencil operator bodies for the device, one per reference operator id.
//
// Every body restates the reference's serial operator (src/verification.c:315-479)
// in the same association order.  Arithmetic goes through an `A` policy:
//   ExactArith  -- every product and sum rounded on its own (__dmul_rn /
//                  __dadd_rn), so FP64 results equal the serial reference bit
//                  for bit;
//   FastArith   -- plain operators; nvcc contracts products into adds (FMA),
//                  which changes the last bits (max-norm relative error ~1e-15
//                  per step, well inside the 1e-12 parity bound).
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

namespace girih {

struct ExactArith {
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
  // 2v - u as the reference writes it: v + v, then the subtraction
  static __device__ __forceinline__ double twice_minus(double v, double u) { return __dsub_rn(__dadd_rn(v, v), u); }
  static __device__ __forceinline__ float twice_minus(float v, float u) { return __fsub_rn(__fadd_rn(v, v), u); }
};

struct FastArith {
  template <class T> static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
  template <class T> static __device__ __forceinline__ T add(T a, T b) { return a + b; }
  template <class T> static __device__ __forceinline__ T sub(T a, T b) { return a - b; }
  // FP64: 2v - u in one FMA.  2v is exact, so fma(2, v, -u) is (v + v) - u
  // rounded once, bit for bit, wherever 2v does not overflow: one FP64
  // operation of the ten in a leapfrog update, on the pipe that bounds the FP64
  // forms.  FP32 keeps the two operations (the FP32 sweeps are bound by memory,
  // and the FMA form measured 9 % slower in the x-quad sweep).
  static __device__ __forceinline__ double twice_minus(double v, double u) { return __fma_rn(2.0, v, -u); }
  static __device__ __forceinline__ float twice_minus(float v, float u) { return (v + v) - u; }
};

// Operator metadata (src/kernels/stencils.c:260-271, plus id 8).
template <int OP> struct OpTraits;
template <> struct OpTraits<0> { static constexpr int R = 4, TO = 2, NC = 5, VAR = 0; };
template <> struct OpTraits<1> { static constexpr int R = 1, TO = 1, NC = 2, VAR = 0; };
template <> struct OpTraits<2> { static constexpr int R = 1, TO = 1, NC = 2, VAR = 1; };
template <> struct OpTraits<3> { static constexpr int R = 1, TO = 1, NC = 4, VAR = 1; };
template <> struct OpTraits<4> { static constexpr int R = 4, TO = 1, NC = 13, VAR = 1; };
template <> struct OpTraits<5> { static constexpr int R = 1, TO = 1, NC = 7, VAR = 1; };
template <> struct OpTraits<7> { static constexpr int R = 1, TO = 1, NC = 4, VAR = 0; };
template <> struct OpTraits<8> { static constexpr int R = 1, TO = 2, NC = 2, VAR = 0; };

// Coefficient fetch for variable-coefficient operators: array m at the centre
// point.  Full-precision storage (T) or BF16 with a per-array FP32 scale.
template <class T> struct CoefFull {
  const T *__restrict__ base;
  int64_t stride;  // elements between arrays
  __device__ __forceinline__ T operator()(int m, int64_t c) const { return __ldg(base + m * stride + c); }
};
struct CoefBF16 {
  const __nv_bfloat16 *__restrict__ base;
  int64_t stride;
  const float *__restrict__ scale;  // per array
  __device__ __forceinline__ float operator()(int m, int64_t c) const {
    return __bfloat162float(base[m * stride + c]) * scale[m];
  }
};

// Neighbour access goes through an accessor `V` with V.c() (centre) and
// V.x(d), V.y(d), V.z(d) (offset d along one axis, d may be negative), so that
// each kernel can serve neighbours from registers, shared memory or global
// memory.  A pair sum is (+d) + (-d), the reference's order.
#define GIRIH_PAIR(ax, d) A::add(V.ax(d), V.ax(-(d)))

// Constant-coefficient star Laplacian sum of radius R (operators 0, 1, 8):
// c0*v + c1*(x1) + c1*(y1) + c1*(z1) + c2*(x2) + ... (verification.c:330-350, 367-370).
template <int R, class A, class T, class Vf>
__device__ __forceinline__ T star_const_sum(const T *c, const Vf &V) {
  T s = A::mul(c[0], V.c());
#pragma unroll
  for (int d = 1; d <= R; d++) {
    s = A::add(s, A::mul(c[d], GIRIH_PAIR(x, d)));
    s = A::add(s, A::mul(c[d], GIRIH_PAIR(y, d)));
    s = A::add(s, A::mul(c[d], GIRIH_PAIR(z, d)));
  }
  return s;
}

// The same sum grouped per distance, c0*v + sum_d c_d*((x_d + y_d) + z_d): two
// fewer products per distance.  Used where results need not match the
// reference's association bit for bit (the double-float fused form, held to
// the FP64 parity bound).
template <int R, class A, class T, class Vf>
__device__ __forceinline__ T star_grouped_sum(const T *c, const Vf &V) {
  T s = A::mul(c[0], V.c());
#pragma unroll
  for (int d = 1; d <= R; d++)
    s = A::add(s, A::mul(c[d], A::add(A::add(GIRIH_PAIR(x, d), GIRIH_PAIR(y, d)), GIRIH_PAIR(z, d))));
  return s;
}

// One operator application at the centre point; `uold` is the old value of the
// updated array (time-order-2 operators), `roc2` the per-point roc2 value.
template <int OP, class A, class T, class Vf, class Cf>
__device__ __forceinline__ T apply_op(const T *cc, const Cf &coef, int64_t cidx, const Vf &V,
                                      T uold, T roc2) {
  if constexpr (OP == 0 || OP == 8) {
    constexpr int R = OpTraits<OP>::R;
    T lap = star_const_sum<R, A>(cc, V);
    // u = 2v - u + roc2*lap   (verification.c:344-348)
    return A::add(A::twice_minus(V.c(), uold), A::mul(roc2, lap));
  } else if constexpr (OP == 1) {
    return star_const_sum<1, A>(cc, V);
  } else if constexpr (OP == 2) {  // verification.c:390-393
    T c0 = T(coef(0, cidx)), c1 = T(coef(1, cidx));
    T s = A::mul(c0, V.c());
    s = A::add(s, A::mul(c1, GIRIH_PAIR(x, 1)));
    s = A::add(s, A::mul(c1, GIRIH_PAIR(y, 1)));
    s = A::add(s, A::mul(c1, GIRIH_PAIR(z, 1)));
    return s;
  } else if constexpr (OP == 3) {  // verification.c:413-416
    T s = A::mul(T(coef(0, cidx)), V.c());
    s = A::add(s, A::mul(T(coef(1, cidx)), GIRIH_PAIR(x, 1)));
    s = A::add(s, A::mul(T(coef(2, cidx)), GIRIH_PAIR(y, 1)));
    s = A::add(s, A::mul(T(coef(3, cidx)), GIRIH_PAIR(z, 1)));
    return s;
  } else if constexpr (OP == 4) {  // verification.c:437-449
    T s = A::mul(T(coef(0, cidx)), V.c());
#pragma unroll
    for (int d = 1; d <= 4; d++) {
      s = A::add(s, A::mul(T(coef(3 * d - 2, cidx)), GIRIH_PAIR(x, d)));
      s = A::add(s, A::mul(T(coef(3 * d - 1, cidx)), GIRIH_PAIR(y, d)));
      s = A::add(s, A::mul(T(coef(3 * d, cidx)), GIRIH_PAIR(z, d)));
    }
    return s;
  } else if constexpr (OP == 5) {  // verification.c:468-474
    T s = A::mul(T(coef(0, cidx)), V.c());
    s = A::add(s, A::mul(T(coef(1, cidx)), V.x(-1)));
    s = A::add(s, A::mul(T(coef(2, cidx)), V.x(1)));
    s = A::add(s, A::mul(T(coef(3, cidx)), V.y(-1)));
    s = A::add(s, A::mul(T(coef(4, cidx)), V.y(1)));
    s = A::add(s, A::mul(T(coef(5, cidx)), V.z(-1)));
    s = A::add(s, A::mul(T(coef(6, cidx)), V.z(1)));
    return s;
  } else if constexpr (OP == 7) {  // box, verification.c:797-815: edges and corners via V.xyz()
    T s = A::mul(cc[0], V.c());
    s = A::add(s, A::mul(cc[1], GIRIH_PAIR(x, 1)));
    s = A::add(s, A::mul(cc[1], GIRIH_PAIR(y, 1)));
    s = A::add(s, A::mul(cc[1], GIRIH_PAIR(z, 1)));
    s = A::add(s, A::mul(cc[2], A::add(V.xyz(1, 0, -1), V.xyz(-1, 0, -1))));
    s = A::add(s, A::mul(cc[2], A::add(V.xyz(0, 1, -1), V.xyz(0, -1, -1))));
    s = A::add(s, A::mul(cc[2], A::add(V.xyz(1, 1, 0), V.xyz(-1, -1, 0))));
    s = A::add(s, A::mul(cc[2], A::add(V.xyz(1, -1, 0), V.xyz(-1, 1, 0))));
    s = A::add(s, A::mul(cc[2], A::add(V.xyz(1, 0, 1), V.xyz(-1, 0, 1))));
    s = A::add(s, A::mul(cc[2], A::add(V.xyz(0, 1, 1), V.xyz(0, -1, 1))));
    s = A::add(s, A::mul(cc[3], A::add(V.xyz(1, 1, 1), V.xyz(-1, -1, -1))));
    s = A::add(s, A::mul(cc[3], A::add(V.xyz(1, -1, 1), V.xyz(-1, 1, -1))));
    s = A::add(s, A::mul(cc[3], A::add(V.xyz(-1, -1, 1), V.xyz(1, 1, -1))));
    s = A::add(s, A::mul(cc[3], A::add(V.xyz(-1, 1, 1), V.xyz(1, -1, -1))));
    return s;
  }
  return T(0);
}

#undef GIRIH_PAIR

}  // namespace girih
