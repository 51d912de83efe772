// Time-fused stencil kernel: TT time steps per pass over HBM.
//
// Replaces the reference's Multi-core Wavefront Diamond temporal blocking
// (src/kernels/stencils_mwf.ic:19-161, scheduled by src/kernels/diamond_ts.c:871-976)
// with a GPU schedule: overlapped x-y tiles (each CTA recomputes a halo of
// TT*R columns instead of synchronising with its neighbours) and a z wavefront
// inside the CTA.  Time level l trails level l-1 by D = R+1 planes, so level l
// computes plane p = s - l*D at z step s from
//   * the z neighbours p-R..p+R of level l-1, held in a per-thread register
//     queue (the reference's wavefront "frontline", stencils_mwf.ic:119-147),
//   * the x/y neighbours of level l-1 at plane p, read from shared memory that
//     every thread filled at step s-1 (double buffered: one barrier per step).
// Only level 0 is read from HBM and only the last two levels are written, so a
// pass moves the bytes of one step while advancing TT steps.
//
// Points outside the interior (halo columns, halo planes) keep their initial
// value at every level, as the reference never writes halos.  All field
// buffers carry the same fixed halo, so a halo value can be copied from the
// level below.
#pragma once
#include <algorithm>
#include <utility>

#include "fused.cuh"
#include "ops.cuh"

namespace girih {

template <class T> struct FusedArgs {
  Geom g;
  const T *prev, *cur, *roc2;
  T *out_prev, *out_cur;
  T cc[5];
  int zchunk;
  int write_prev;
};

// z-queue slot of plane p: planes are stored at p mod QL, so advancing a step
// renames registers instead of moving them (the step loop is unrolled QL times
// and every slot index below is a compile-time constant).
template <int QL> __host__ __device__ constexpr int qslot(int x) { return ((x % QL) + QL) % QL; }

template <int R, class T, int QL, int BASE> struct FusedAcc {
  const T *__restrict__ s;  // shared-memory element of the centre (level l-1, plane p)
  const T (&q)[QL];         // z queue of level l-1; plane p sits in slot BASE
  int ld;                   // shared-memory row length
  __device__ __forceinline__ T c() const { return q[qslot<QL>(BASE)]; }
  __device__ __forceinline__ T x(int d) const { return s[d]; }
  __device__ __forceinline__ T y(int d) const { return s[d * ld]; }
  __device__ __forceinline__ T z(int d) const { return q[qslot<QL>(BASE + d)]; }
};

template <class F, int... I>
__device__ __forceinline__ void static_for_impl(F &f, std::integer_sequence<int, I...>) {
  (f(std::integral_constant<int, I>{}), ...);
}
template <int N, class F> __device__ __forceinline__ void static_for(F &&f) {
  static_for_impl(f, std::make_integer_sequence<int, N>{});
}

// Compensated leapfrog update 2v - u + roc2*lap: the cancellation 2v - u is
// computed exactly as s + e (two-sum), e is folded into the small term, and the
// result is rounded once.
__device__ __forceinline__ float leapfrog_compensated(float v, float u, float r2, float lap) {
  const float a = 2.f * v;
  const float s = __fsub_rn(a, u);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(-u, bb));
  return __fadd_rn(s, fmaf(r2, lap, e));
}

template <int OP, class T, bool COMP, int TT, int NTX, int NTY, int CY>
__global__ void __launch_bounds__(NTX *NTY) fused_pass(FusedArgs<T> a) {
  constexpr int R = OpTraits<OP>::R;
  constexpr int TO = OpTraits<OP>::TO;
  constexpr int D = R + 1;
  constexpr int QL = TO == 2 ? 2 * R + 2 : 2 * R + 1;
  constexpr int RY = NTY * CY;
  constexpr int H = TT * R;
  constexpr int BX = NTX - 2 * H;
  constexpr int BY = RY - 2 * H;
  static_assert(BX > 0 && BY > 0, "tile too small for the fusion depth");
  static_assert(TT * CY <= 32, "activity mask holds 32 (level, row) pairs");

  extern __shared__ __align__(16) unsigned char smraw[];
  T *sm = reinterpret_cast<T *>(smraw);  // [2][TT][RY][NTX]

  const Geom &g = a.g;
  const int64_t plane = g.plane;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int X0 = blockIdx.x * BX, Y0 = blockIdx.y * BY;
  const int Z0 = R + blockIdx.z * a.zchunk;
  const int Z1 = min(Z0 + a.zchunk, g.nnz - R);
  const int sb = max(0, Z0 - H);
  const int se = Z1 - 1 + TT * D;
  const int s0 = sb - sb % QL;  // aligned so that plane p lives in slot p mod QL

  const int xi = X0 - H + tx;  // interior x index of this column
  const int i = xi + R;        // reference x index
  const bool x_dom = i >= 0 && i < g.nnx;
  const bool x_int = xi >= 0 && xi < g.nx;
  const bool x_out = tx >= H && tx < NTX - H && xi < g.nx;

  bool y_dom[CY], y_out[CY];
  int64_t col[CY];
  unsigned act_mask = 0;  // bit (l-1)*CY + c: level l of row c lies in the shrinking valid region
#pragma unroll
  for (int c = 0; c < CY; c++) {
    const int ry = ty + c * NTY;
    const int yj = Y0 - H + ry;
    const int j = yj + R;
    y_dom[c] = j >= 0 && j < g.nny;
    const bool y_int = yj >= 0 && yj < g.ny;
    y_out[c] = x_out && ry >= H && ry < RY - H && yj < g.ny;
    col[c] = (x_dom && y_dom[c]) ? (int64_t)j * g.px + g.ox + i : 0;
#pragma unroll
    for (int l = 1; l <= TT; l++)
      if (x_int && y_int && tx >= l * R && tx < NTX - l * R && ry >= l * R && ry < RY - l * R)
        act_mask |= 1u << ((l - 1) * CY + c);
  }

  T cc[5];
#pragma unroll
  for (int m = 0; m < 5; m++) cc[m] = a.cc[m];

  T q[TT][CY][QL];
#pragma unroll
  for (int l = 0; l < TT; l++)
#pragma unroll
    for (int c = 0; c < CY; c++)
#pragma unroll
      for (int e = 0; e < QL; e++) q[l][c][e] = T(0);

  for (int sbase = s0; sbase <= se; sbase += QL) {
    static_for<QL>([&](auto ph_c) {
      constexpr int PH = decltype(ph_c)::value;
      const int s = sbase + PH;
      if (s > se) return;  // uniform over the CTA
      const int rb = (s - 1) & 1, wb = s & 1;
      const int64_t soff = (int64_t)s * plane;
      // levels TT..1, highest first: level l reads level l-1's queue before
      // level l-1 stores this step's plane
      static_for<TT>([&](auto li_c) {
        constexpr int L = TT - decltype(li_c)::value;  // TT, TT-1, ..., 1
        constexpr int SL = qslot<QL>(PH - L * D);        // slot of plane p in every queue
        const int p = s - L * D;
        const bool p_int = p >= R && p < g.nnz - R;
        const bool p_out = p_int && p >= Z0 && p < Z1;
        const int64_t poff = soff - (int64_t)(L * D) * plane;
        const T *smr = sm + (size_t)((rb * TT + (L - 1)) * RY) * NTX;
#pragma unroll
        for (int c = 0; c < CY; c++) {
          const int ry = ty + c * NTY;
          T val = q[L - 1][c][SL];
          if (p_int && (act_mask >> ((L - 1) * CY + c) & 1u)) {
            const int64_t at = poff + col[c];
            FusedAcc<R, T, QL, SL> acc{smr + ry * NTX + tx, q[L - 1][c], NTX};
            if constexpr (TO == 2) {
              T uold;
              if constexpr (L >= 2) uold = q[L - 2][c][SL];
              else uold = a.prev[at];
              const T r2 = __ldg(a.roc2 + at);
              if constexpr (COMP) {
                const float lap = star_const_sum<R, FastArith>(cc, acc);
                val = leapfrog_compensated(val, uold, r2, lap);
              } else {
                CoefFull<T> none{nullptr, 0};
                val = apply_op<OP, FastArith>(cc, none, 0, acc, uold, r2);
              }
            } else {
              CoefFull<T> none{nullptr, 0};
              val = apply_op<OP, FastArith>(cc, none, 0, acc, T(0), T(0));
            }
          }
          if (p_out && y_out[c]) {
            if constexpr (L == TT) a.out_cur[poff + col[c]] = val;
            if constexpr (L == TT - 1) {
              if (a.write_prev) a.out_prev[poff + col[c]] = val;
            }
          }
          if constexpr (L < TT) q[L][c][SL] = val;
        }
      });
      // level 0: stream plane s from HBM
      const bool s_in = s < g.nnz;
#pragma unroll
      for (int c = 0; c < CY; c++) {
        T v = T(0);
        if (s_in && x_dom && y_dom[c]) v = __ldg(a.cur + soff + col[c]);
        q[0][c][qslot<QL>(PH)] = v;
        if constexpr (TT == 1) {
          if (a.write_prev && s >= R && s < g.nnz - R && s >= Z0 && s < Z1 && y_out[c])
            a.out_prev[soff + col[c]] = v;
        }
      }
      // publish each level's centre plane (s - l*D - R) for the x/y neighbours of step s+1
#pragma unroll
      for (int l = 0; l < TT; l++)
#pragma unroll
        for (int c = 0; c < CY; c++)
          sm[(size_t)((wb * TT + l) * RY + ty + c * NTY) * NTX + tx] = q[l][c][qslot<QL>(PH - l * D - R)];
      __syncthreads();
    });
  }
}

template <int NTX, int NTY, int CY> struct VariantShape {
  static constexpr int ntx = NTX, nty = NTY, cy = CY;
};

template <int OP, class T, bool COMP, int TT, int NTX, int NTY, int CY>
cudaError_t launch_tt(const Geom &g, const FusedLaunch &L, cudaStream_t s) {
  constexpr int R = OpTraits<OP>::R;
  constexpr int RY = NTY * CY, H = TT * R, BX = NTX - 2 * H, BY = RY - 2 * H;
  auto kern = fused_pass<OP, T, COMP, TT, NTX, NTY, CY>;
  const size_t smem = (size_t)2 * TT * RY * NTX * sizeof(T);
  static bool attr_set = false;  // per instantiation, host side
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  int occ = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, NTX * NTY, smem);
  if (occ < 1) occ = 1;
  const int gx = (g.nx + BX - 1) / BX, gy = (g.ny + BY - 1) / BY;
  const int64_t tiles = (int64_t)gx * gy;
  int nsm = 152;
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  }
  const int64_t cap = (int64_t)nsm * occ;
  // choose the number of z chunks: minimise waves x (chunk + pipeline overhead)
  const int over = TT * R + TT * (R + 1);
  int best_n = 1;
  double best_cost = 1e300;
  for (int n = 1; n <= 64 && n <= g.nz; n++) {
    int chunk = (g.nz + n - 1) / n;
    int64_t ctas = tiles * n;
    int64_t waves = (ctas + cap - 1) / cap;
    double cost = (double)waves * (chunk + over);
    if (cost < best_cost * 0.999) {
      best_cost = cost;
      best_n = n;
    }
  }
  const int zchunk = (g.nz + best_n - 1) / best_n;
  const int nz_ch = (g.nz + zchunk - 1) / zchunk;
  FusedArgs<T> a{};
  a.g = g;
  a.prev = static_cast<const T *>(L.prev);
  a.cur = static_cast<const T *>(L.cur);
  a.roc2 = static_cast<const T *>(L.roc2);
  a.out_prev = static_cast<T *>(L.out_prev);
  a.out_cur = static_cast<T *>(L.out_cur);
  for (int m = 0; m < 5; m++) a.cc[m] = (T)L.cc[m];
  a.zchunk = zchunk;
  a.write_prev = L.write_prev;
  kern<<<dim3(gx, gy, nz_ch), dim3(NTX, NTY), smem, s>>>(a);
  return cudaGetLastError();
}

template <int OP, class T, bool COMP, int NTX, int NTY, int CY, int TMAX>
cudaError_t launch_variant(const Geom &g, const FusedLaunch &L, cudaStream_t s) {
  switch (L.steps) {
    case 1: return launch_tt<OP, T, COMP, 1, NTX, NTY, CY>(g, L, s);
    case 2: if constexpr (TMAX >= 2) return launch_tt<OP, T, COMP, 2, NTX, NTY, CY>(g, L, s); break;
    case 3: if constexpr (TMAX >= 3) return launch_tt<OP, T, COMP, 3, NTX, NTY, CY>(g, L, s); break;
    case 4: if constexpr (TMAX >= 4) return launch_tt<OP, T, COMP, 4, NTX, NTY, CY>(g, L, s); break;
    case 5: if constexpr (TMAX >= 5) return launch_tt<OP, T, COMP, 5, NTX, NTY, CY>(g, L, s); break;
    case 6: if constexpr (TMAX >= 6) return launch_tt<OP, T, COMP, 6, NTX, NTY, CY>(g, L, s); break;
  }
  return cudaErrorInvalidValue;
}

// Maximum fusion depth instantiated per operator radius and element type.
template <int OP, class T> constexpr int fused_tmax() {
  return OpTraits<OP>::R == 4 ? 2 : (sizeof(T) == 8 ? 4 : 6);
}

template <int OP, class T, bool COMP>
cudaError_t launch_fused_op_impl(const Geom &g, const FusedConfig &cfg, const FusedLaunch &L,
                                 cudaStream_t s) {
  constexpr int TM = fused_tmax<OP, T>();
  if (cfg.variant == FV_64x16x2) return launch_variant<OP, T, COMP, 64, 16, 2, TM>(g, L, s);
  return launch_variant<OP, T, COMP, 32, 16, 4, TM>(g, L, s);
}

}  // namespace girih
