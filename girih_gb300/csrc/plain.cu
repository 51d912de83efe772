// Plain time stepping: one stencil sweep per kernel launch.
//
// This replaces the reference's spatially blocked sweep (src/kernels/stencils_spt_blk.ic:19-48,
// called twice per iteration from src/kernels/nb_naive_ts.c:189,195).  Each thread owns one
// (x, y) column of the interior and streams a chunk of z planes, keeping the 2R+1 values of its
// column in a register queue; x and y neighbours are read through the read-only path (L1).
// Warps run along x over the 128-byte-aligned interior rows, so every row access coalesces.
//
// FP32 star operators use x quads instead: each thread owns 4 consecutive columns, moves
// every row segment as one 16-byte vector (its own quad, the y-neighbour rows, the z
// plane, the old value, roc2) and takes the x neighbours beyond its quad from the
// adjacent quads, and variable coefficients as one vector per array: per 4 updates
// roughly a quarter of the load instructions of the one-column sweep.
#include <algorithm>

#include "check.cuh"
#include "internal.cuh"
#include "ops.cuh"
#include "vec.cuh"

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
  // checked build: the point's whole neighbourhood block, planes k-R..k+R
  const int64_t reach = R * plane + R * (int64_t)a.g.px + R;
#pragma unroll
  for (int d = 0; d < 2 * R; d++) q[d] = T(0);
  if (in_array(c - reach, 2 * reach + 1, a.g.elems, a.flag))
#pragma unroll
    for (int d = 0; d < 2 * R; d++) q[d] = __ldg(a.v + c + (int64_t)(d - R) * plane);
  for (int k = k0; k < k1; k++, c += plane) {
    if (!in_array(c - reach, 2 * reach + 1, a.g.elems, a.flag)) continue;
    q[2 * R] = __ldg(a.v + c + (int64_t)R * plane);
    ColumnAcc<R, T> acc{a.v + c, a.g.px, plane, q};
    T uold = T(0), r2 = T(0);
    if constexpr (TO == 2) {
      uold = a.u[c];
      r2 = __ldg(a.roc2 + c);
    }
    a.u[c] = apply_op<OP, A>(cc, coef, c, acc, uold, r2);
    count_writes(a.cov, c, 1);
#pragma unroll
    for (int d = 0; d < 2 * R; d++) q[d] = q[d + 1];
  }
}

// Accessor of column V of a thread's quad at the current plane.
template <int R, class T, int VX, int V> struct QuadAcc {
  const T (&q)[2 * R + 1][VX];  // z queue: planes k-R .. k+R of the quad's columns
  const T (&xl)[VX], (&xr)[VX];  // the quads left and right of this one (current plane)
  const T (&yv)[2 * R][VX];      // y neighbour rows: [d-1] = +d, [R+d-1] = -d
  __device__ __forceinline__ T c() const { return q[R][V]; }
  __device__ __forceinline__ T x(int d) const {
    const int pos = V + d;
    if (pos >= 0 && pos < VX) return q[R][pos < 0 ? 0 : (pos >= VX ? VX - 1 : pos)];
    return pos < 0 ? xl[pos < -VX ? 0 : pos + VX] : xr[pos >= 2 * VX ? VX - 1 : pos - VX];
  }
  __device__ __forceinline__ T y(int d) const { return d > 0 ? yv[d - 1][V] : yv[R - d - 1][V]; }
  __device__ __forceinline__ T z(int d) const { return q[R + d][V]; }
};

template <class T, int VX> __device__ __forceinline__ void vload(const T *p, T (&e)[VX]) {
  VecU<T, VX> u;
  u.v = __ldg(reinterpret_cast<const decltype(u.v) *>(p));
#pragma unroll
  for (int k = 0; k < VX; k++) e[k] = u.e[k];
}

// One sweep with x quads (FP32, radius <= 4): a thread owns columns i0..i0+3 of
// row j and streams a z chunk.  Reads past the last interior column stay in the
// array (the row is followed by halo rows or planes) and feed only columns that
// are not written.
template <int OP, class A, class T, bool BF16>
__global__ void __launch_bounds__(kBX *kBY) plain_step_quad(StepArgs<T> a, int zchunk) {
  constexpr int R = OpTraits<OP>::R, TO = OpTraits<OP>::TO, VX = 4;
  constexpr bool VAR = OpTraits<OP>::VAR;
  constexpr int NC = VAR ? OpTraits<OP>::NC : 1;
  const int i0 = (blockIdx.x * kBX + threadIdx.x) * VX;
  const int j = blockIdx.y * kBY + threadIdx.y;
  if (i0 >= a.g.nx || j >= a.g.ny) return;
  const int k0 = blockIdx.z * zchunk;
  const int k1 = min(k0 + zchunk, a.g.nz);
  const int64_t plane = a.g.plane, px = a.g.px;
  int64_t c = a.g.at(R + i0, R + j, R + k0);  // 16-byte aligned: the interior starts on 128 bytes
  T cc[5];
#pragma unroll
  for (int m = 0; m < 5; m++) cc[m] = a.cc[m];
  T q[2 * R + 1][VX];
  // Loads: the normal build addresses every vector as a.v + c +/- offset (with
  // the negative offsets written as subtractions: the radius-4 kernel then
  // compiles to 76 registers, three CTAs per SM, against 90-127 for other
  // spellings of the same addresses); the checked build first tests each
  // vector range against the array and skips a load outside it (values zero).
#if GIRIH_CHECKED
  unsigned *const flag = a.flag;
  const int64_t n = a.g.elems;
  auto ld = [&](int64_t off, T(&e)[VX]) {
    if (in_array(off, VX, n, flag)) {
      vload<T, VX>(a.v + off, e);
    } else {
#pragma unroll
      for (int v = 0; v < VX; v++) e[v] = T(0);
    }
  };
#define GIRIH_QLD(off, e) ld(c + (off), e)
#define GIRIH_QLD_M(off, e) ld(c - (off), e)
#else
#define GIRIH_QLD(off, e) vload<T, VX>(a.v + c + (off), e)
#define GIRIH_QLD_M(off, e) vload<T, VX>(a.v + c - (off), e)
#endif
#pragma unroll
  for (int d = 0; d < 2 * R; d++) GIRIH_QLD((int64_t)(d - R) * plane, q[d]);
  const bool full = i0 + VX <= a.g.nx;
  for (int k = k0; k < k1; k++, c += plane) {
    GIRIH_QLD((int64_t)R * plane, q[2 * R]);
    T xl[VX], xr[VX], yv[2 * R][VX];
    GIRIH_QLD_M(VX, xl);
    GIRIH_QLD(VX, xr);
#pragma unroll
    for (int d = 1; d <= R; d++) {
      GIRIH_QLD(d * px, yv[d - 1]);
      GIRIH_QLD_M(d * px, yv[R + d - 1]);
    }
#undef GIRIH_QLD
#undef GIRIH_QLD_M
#if GIRIH_CHECKED
    if (!in_array(c, VX, n, flag)) continue;  // the old value, roc2, coefficients and the store
#endif
    T uo[VX], r2[VX];
    if constexpr (TO == 2) {
      VecU<T, VX> u;
      u.v = *reinterpret_cast<const decltype(u.v) *>(a.u + c);
#pragma unroll
      for (int v = 0; v < VX; v++) uo[v] = u.e[v];
      vload<T, VX>(a.roc2 + c, r2);
    }
    T cf[NC][VX];
    if constexpr (VAR) load_coef_group<T, BF16, NC, VX>(a.coef, a.g.elems, a.scale, c, cf);
    T out[VX];
#pragma unroll
    for (int v = 0; v < VX; v++) out[v] = T(0);
    // static unroll over the quad's columns
#define GIRIH_QUAD_COLUMN(V)                                                                   \
    {                                                                                          \
      QuadAcc<R, T, VX, V> acc{q, xl, xr, yv};                                                 \
      CoefGroup<T, NC, VX, V> cg{cf};                                                          \
      if constexpr (TO == 2) out[V] = apply_op<OP, A>(cc, cg, 0, acc, uo[V], r2[V]);            \
      else out[V] = apply_op<OP, A>(cc, cg, 0, acc, T(0), T(0));                               \
    }
    GIRIH_QUAD_COLUMN(0)
    GIRIH_QUAD_COLUMN(1)
    GIRIH_QUAD_COLUMN(2)
    GIRIH_QUAD_COLUMN(3)
#undef GIRIH_QUAD_COLUMN
    if (full) {
      VecU<T, VX> u;
#pragma unroll
      for (int v = 0; v < VX; v++) u.e[v] = out[v];
      *reinterpret_cast<decltype(u.v) *>(a.u + c) = u.v;
      count_writes(a.cov, c, VX);
    } else {
#pragma unroll
      for (int v = 0; v < VX; v++)
        if (i0 + v < a.g.nx) {
          a.u[c + v] = out[v];
          count_writes(a.cov, c + v, 1);
        }
    }
#pragma unroll
    for (int d = 0; d < 2 * R; d++)
#pragma unroll
      for (int v = 0; v < VX; v++) q[d][v] = q[d + 1][v];
  }
}

template <int OP, class A, class T, bool BF16>
cudaError_t launch_quad(const StepArgs<T> &a, cudaStream_t s) {
  constexpr int R = OpTraits<OP>::R;
  dim3 block(kBX, kBY);
  const int cols = kBX * 4;
  int gx = (a.g.nx + cols - 1) / cols, gy = (a.g.ny + kBY - 1) / kBY;
  const int64_t want = 8 * 152;
  int64_t blocks = (int64_t)gx * gy;
  int nchunks = (int)std::max<int64_t>(1, (want + blocks - 1) / blocks);
  int zchunk = (a.g.nz + nchunks - 1) / nchunks;
  zchunk = std::max(zchunk, std::min(a.g.nz, 8 * R));
  int gz = (a.g.nz + zchunk - 1) / zchunk;
  plain_step_quad<OP, A, T, BF16><<<dim3(gx, gy, gz), block, 0, s>>>(a, zchunk);
  return cudaGetLastError();
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
  if constexpr (sizeof(T) == 4 && OP != 7) {  // FP32 star operators: x quads
    if constexpr (OpTraits<OP>::VAR) {
      if (bf16coef)
        return exact ? launch_quad<OP, ExactArith, T, true>(a, s) : launch_quad<OP, FastArith, T, true>(a, s);
    }
    return exact ? launch_quad<OP, ExactArith, T, false>(a, s) : launch_quad<OP, FastArith, T, false>(a, s);
  }
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
