// Plain time stepping: one stencil sweep per kernel launch.
//
// This replaces the reference's spatially blocked sweep (src/kernels/stencils_spt_blk.ic:19-48,
// called twice per iteration from src/kernels/nb_naive_ts.c:189,195).  Each thread owns one
// (x, y) column of the interior and streams a chunk of z planes, keeping the 2R+1 values of its
// column in a register queue; x and y neighbours are read through the read-only path (L1).
// Warps run along x over the 128-byte-aligned interior rows, so every row access coalesces.
#include <algorithm>

#include "internal.cuh"
#include "ops.cuh"

namespace girih {

namespace {

constexpr int kBX = 32, kBY = 8;

template <int R, class T> struct ColumnAcc {
  const T *__restrict__ p;  // centre point in v
  int64_t sy;               // row pitch
  int64_t sz;               // plane pitch
  const T (&q)[2 * R + 1];  // column values at planes k-R .. k+R
  __device__ __forceinline__ T c() const { return q[R]; }
  __device__ __forceinline__ T x(int d) const { return __ldg(p + d); }
  __device__ __forceinline__ T y(int d) const { return __ldg(p + d * sy); }
  __device__ __forceinline__ T z(int d) const { return q[R + d]; }
  // off-axis neighbour (box operator)
  __device__ __forceinline__ T xyz(int dx, int dy, int dz) const { return __ldg(p + dx + dy * sy + dz * sz); }
};

template <int OP, class A, class T, class Cf>
__global__ void __launch_bounds__(kBX *kBY) plain_step(StepArgs<T> a, Cf coef, int zchunk) {
  constexpr int R = OpTraits<OP>::R;
  constexpr int TO = OpTraits<OP>::TO;
  const int i = blockIdx.x * kBX + threadIdx.x;
  const int j = blockIdx.y * kBY + threadIdx.y;
  if (i >= a.g.nx || j >= a.g.ny) return;
  const int k0 = blockIdx.z * zchunk;
  const int k1 = min(k0 + zchunk, a.g.nz);
  const int64_t plane = a.g.plane;
  int64_t c = a.g.at(R + i, R + j, R + k0);
  T cc[5];
#pragma unroll
  for (int m = 0; m < 5; m++) cc[m] = a.cc[m];
  T q[2 * R + 1];
#pragma unroll
  for (int d = 0; d < 2 * R; d++) q[d] = __ldg(a.v + c + (int64_t)(d - R) * plane);
  for (int k = k0; k < k1; k++, c += plane) {
    q[2 * R] = __ldg(a.v + c + (int64_t)R * plane);
    ColumnAcc<R, T> acc{a.v + c, a.g.px, plane, q};
    T uold = T(0), r2 = T(0);
    if constexpr (TO == 2) {
      uold = a.u[c];
      r2 = __ldg(a.roc2 + c);
    }
    a.u[c] = apply_op<OP, A>(cc, coef, c, acc, uold, r2);
#pragma unroll
    for (int d = 0; d < 2 * R; d++) q[d] = q[d + 1];
  }
}

template <int OP, class A, class T, class Cf>
cudaError_t launch_one(const StepArgs<T> &a, Cf coef, cudaStream_t s) {
  constexpr int R = OpTraits<OP>::R;
  dim3 block(kBX, kBY);
  int gx = (a.g.nx + kBX - 1) / kBX, gy = (a.g.ny + kBY - 1) / kBY;
  // enough CTAs for several waves on 152 SMs, z chunks long enough that the
  // 2R re-read planes per chunk stay a small fraction
  const int64_t want = 8 * 152;
  int64_t cols = (int64_t)gx * gy;
  int nchunks = (int)std::max<int64_t>(1, (want + cols - 1) / cols);
  int zchunk = (a.g.nz + nchunks - 1) / nchunks;
  zchunk = std::max(zchunk, std::min(a.g.nz, 8 * R));
  int gz = (a.g.nz + zchunk - 1) / zchunk;
  plain_step<OP, A, T, Cf><<<dim3(gx, gy, gz), block, 0, s>>>(a, coef, zchunk);
  return cudaGetLastError();
}

template <int OP, class T>
cudaError_t dispatch(const StepArgs<T> &a, bool exact, bool bf16coef, cudaStream_t s) {
  if constexpr (OpTraits<OP>::VAR) {
    if constexpr (sizeof(T) == 4) {
      if (bf16coef) {
        CoefBF16 cf{static_cast<const __nv_bfloat16 *>(a.coef), a.g.elems, a.scale};
        return exact ? launch_one<OP, ExactArith>(a, cf, s) : launch_one<OP, FastArith>(a, cf, s);
      }
    }
    CoefFull<T> cf{static_cast<const T *>(a.coef), a.g.elems};
    return exact ? launch_one<OP, ExactArith>(a, cf, s) : launch_one<OP, FastArith>(a, cf, s);
  } else {
    CoefFull<T> cf{nullptr, 0};
    return exact ? launch_one<OP, ExactArith>(a, cf, s) : launch_one<OP, FastArith>(a, cf, s);
  }
}

}  // namespace

template <class T>
cudaError_t launch_plain_sweep(const StepArgs<T> &a, bool exact, bool bf16coef, cudaStream_t s);

// Source point of one sweep, after the sweep (nb_naive_ts.c:190,196): one
// thread adds the value in the arithmetic of the sweep.
template <class A, class T> __global__ void add_source(T *u, int64_t off, const double *src) {
  u[off] = A::add(u[off], (T)src[0]);
}

template <class T>
cudaError_t launch_plain(const StepArgs<T> &a, bool exact, bool bf16coef, cudaStream_t s) {
  cudaError_t e = launch_plain_sweep(a, exact, bf16coef, s);
  if (e != cudaSuccess || a.src == nullptr) return e;
  if (exact) add_source<ExactArith, T><<<1, 1, 0, s>>>(a.u, a.src_off, a.src);
  else add_source<FastArith, T><<<1, 1, 0, s>>>(a.u, a.src_off, a.src);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_plain_sweep(const StepArgs<T> &a, bool exact, bool bf16coef, cudaStream_t s) {
  switch (a.g.op) {
    case 0: return dispatch<0>(a, exact, bf16coef, s);
    case 1: return dispatch<1>(a, exact, bf16coef, s);
    case 2: return dispatch<2>(a, exact, bf16coef, s);
    case 3: return dispatch<3>(a, exact, bf16coef, s);
    case 4: return dispatch<4>(a, exact, bf16coef, s);
    case 5: return dispatch<5>(a, exact, bf16coef, s);
    case 7: return dispatch<7>(a, exact, bf16coef, s);
    case 8: return dispatch<8>(a, exact, bf16coef, s);
  }
  return cudaErrorInvalidValue;
}

const char *plain_kernel_name(int op) {
  (void)op;
  return "plain_step";
}

template cudaError_t launch_plain<double>(const StepArgs<double> &, bool, bool, cudaStream_t);
template cudaError_t launch_plain<float>(const StepArgs<float> &, bool, bool, cudaStream_t);

}  // namespace girih
