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
#include <atomic>
#include <cstdint>
#include <type_traits>
#include <utility>

#include "check.cuh"
#include "df64.cuh"
#include "fused.cuh"
#include "ops.cuh"
#include "tma.cuh"
#include "vec.cuh"

namespace girih {

// Arguments of one fused pass over one grid.  S is the storage type in HBM
// (float, double, or Df64 pairs: the double-float form streams FP64 fields as
// FP32 pairs, split from and joined to FP64 around the run).
template <class S> struct FusedArgs {
  Geom g;
  const S *prev, *cur, *roc2;
  S *out_prev, *out_cur;
  double cc[5];
  float cch[5], ccl[5];  // cc split on the host: hi = nearest FP32, lo = nearest FP32 of the rest
  int zchunk;      // z chunk of a (tile, chunk) grid; plane split k of a persistent one (for_each_piece)
  int write_prev;
  unsigned *range_flag;  // error flags (bit 1: a TMA copy timed out)
  const void *coef;      // variable coefficients: nc arrays of g.elems (S, or BF16 in the mixed form)
  const float *cscale;   // per-array scales of BF16 coefficients
  const double *src;     // source point values per step (null: none)
  int src_off, src_t0, src_n;
  unsigned *cov_prev, *cov_cur;  // checked build: write counters of out_prev / out_cur (else null)
};

// Storage type of a compute type (every compute type is stored as itself).
template <class T> struct StorageOf { using type = T; };

// Conversions between storage and compute values.
template <class T, class S> __device__ __forceinline__ T to_compute(S v, unsigned &bad) {
  (void)bad;
  if constexpr (std::is_same<T, S>::value) return v;
  else return (T)v;
}
template <class S, class T> __device__ __forceinline__ S to_storage(T v) {
  if constexpr (std::is_same<T, S>::value) return v;
  else return (S)v;
}
// Constant coefficient m in the compute type, from the host-split copies (no
// FP64 conversion in the kernel, which the compiler may otherwise repeat inside
// the z loop on the scarce FP64 pipe instead of holding the value).
template <class T, class S> __device__ __forceinline__ T coef_arg(const FusedArgs<S> &a, int m) {
  if constexpr (std::is_same<T, Df64>::value) return Df64(a.cch[m], a.ccl[m]);
  else if constexpr (std::is_same<T, float>::value) return a.cch[m];
  else return (T)a.cc[m];
}

inline void split_coefs(const double *cc, float *hi, float *lo) {
  for (int m = 0; m < 5; m++) {
    hi[m] = (float)cc[m];
    lo[m] = (float)(cc[m] - (double)hi[m]);
  }
}

template <class T> __device__ __forceinline__ T coef_to_compute(double c) {
  if constexpr (std::is_same<T, Df64>::value) {
    const float h = __double2float_rn(c);
    return Df64(h, __double2float_rn(c - (double)h));
  } else {
    return (T)c;
  }
}

// One element through the read-only path (pairs as one 8-byte load).
template <class S> __device__ __forceinline__ S ldg_elem(const S *p) {
  if constexpr (std::is_same<S, Df64>::value) {
    const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
    return Df64(v.x, v.y);
  } else {
    return __ldg(p);
  }
}

// z-queue slot of plane p: planes are stored at p mod QL, so advancing a step
// renames registers instead of moving them (the step loop is unrolled QL times
// and every slot index below is a compile-time constant).
template <int QL> __host__ __device__ constexpr int qslot(int x) { return ((x % QL) + QL) % QL; }

// VX consecutive x elements (one thread owns VX columns) in the compute type.
template <class T, int VX> struct Pack {
  T e[VX];
  // shared memory (compute type)
  __device__ __forceinline__ void load(const T *p) {
    VecU<T, VX> u;
    u.v = *reinterpret_cast<const decltype(u.v) *>(p);
#pragma unroll
    for (int k = 0; k < VX; k++) e[k] = u.e[k];
  }
  __device__ __forceinline__ void store(T *p) const {
    VecU<T, VX> u;
#pragma unroll
    for (int k = 0; k < VX; k++) u.e[k] = e[k];
    *reinterpret_cast<decltype(u.v) *>(p) = u.v;
  }
  // global memory (storage type S), read-only path
  template <class S> __device__ __forceinline__ void ldg(const S *p, unsigned &bad) {
    VecU<S, VX> u;
    u.v = __ldg(reinterpret_cast<const decltype(u.v) *>(p));
#pragma unroll
    for (int k = 0; k < VX; k++) e[k] = to_compute<T>(u.e[k], bad);
  }
  template <class S> __device__ __forceinline__ void stg(S *p) const {
    VecU<S, VX> u;
#pragma unroll
    for (int k = 0; k < VX; k++) u.e[k] = to_storage<S>(e[k]);
    *reinterpret_cast<decltype(u.v) *>(p) = u.v;
  }
};

// Neighbour accessor of element V of a thread's x-group at level l-1, plane p
// (slot BASE of the z queues): x neighbours inside the group come from
// registers, the others from the shared-memory row; y neighbours from the
// pre-loaded shared-memory vectors; z neighbours from the z queue.
// x neighbours beyond the thread's group come from the two adjacent groups,
// loaded as vectors, when the radius fits in one group and exceeds one column
// (radius 4 with x quads: 2 vector loads instead of 8 scalar ones per quad);
// at radius 1 the two scalar loads measured faster.
__host__ __device__ constexpr bool fused_x_groups(int r, int vx) { return r > 1 && r <= vx; }

// XE (radius 1): the two x neighbours across the group's edges come from xe[0]
// (left) and xe[1] (right), taken from the neighbouring lanes' registers by warp
// shuffles, instead of from the shared-memory row.
template <int R, class T, int QL, int BASE, int VX, int V, bool XE = false> struct FusedAcc {
  const T *__restrict__ srow;             // shared-memory row of level l-1 at this thread's first column
  const T (&q)[VX][QL];                   // z queues of the thread's columns (level l-1)
  const T (&yv)[2 * R][VX];               // y neighbours: [d-1] = +d, [R+d-1] = -d
  const T (&xl)[VX], (&xr)[VX];           // fused_x_groups: the x groups left and right of this one
  const T *xe = nullptr;                  // XE: {left, right} neighbours across the group's edges
  static_assert(!XE || R == 1, "edge shuffles serve radius-1 operators");
  __device__ __forceinline__ T c() const { return q[V][qslot<QL>(BASE)]; }
  __device__ __forceinline__ T x(int d) const {
    const int pos = V + d;
    if (pos >= 0 && pos < VX) return q[pos < 0 ? 0 : (pos >= VX ? VX - 1 : pos)][qslot<QL>(BASE)];
    if constexpr (XE) return pos < 0 ? xe[0] : xe[1];
    else if constexpr (fused_x_groups(R, VX)) return pos < 0 ? xl[pos < -VX ? 0 : pos + VX] : xr[pos >= 2 * VX ? VX - 1 : pos - VX];
    else return srow[pos];
  }
  __device__ __forceinline__ T y(int d) const { return d > 0 ? yv[d - 1][V] : yv[R - d - 1][V]; }
  __device__ __forceinline__ T z(int d) const { return q[V][qslot<QL>(BASE + d)]; }
};

// The accessors of two neighbouring double-float columns as one, returning
// their values as packed pairs (Df2).
template <class A0, class A1> struct PairAcc {
  const A0 &a0;
  const A1 &a1;
  __device__ __forceinline__ Df2 c() const { return df2(a0.c(), a1.c()); }
  __device__ __forceinline__ Df2 x(int d) const { return df2(a0.x(d), a1.x(d)); }
  __device__ __forceinline__ Df2 y(int d) const { return df2(a0.y(d), a1.y(d)); }
  __device__ __forceinline__ Df2 z(int d) const { return df2(a0.z(d), a1.z(d)); }
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

// Packed FP32 pairs: sm_100-class GPUs execute f32x2 add / multiply / FMA as
// one FMA-pipe instruction for two values, each rounded as its scalar
// counterpart.  The radius-1 constant-coefficient levels run a thread's
// columns two at a time with the scalar code's association order (the
// compiler contracts s + c*p into fma(c, p, s)); a - b is fma(-1, b, a), the
// same single rounding as __fsub_rn.
__device__ __forceinline__ float2 f2_sub(float2 a, float2 b) {
  return __ffma2_rn(make_float2(-1.f, -1.f), b, a);
}

// star_const_sum<1, FastArith> on two columns: c0 v + c1 x + c1 y + c1 z.
__device__ __forceinline__ float2 star1_sum2(const float *cc, float2 v, float2 px, float2 py, float2 pz) {
  const float2 c1 = make_float2(cc[1], cc[1]);
  float2 s = __fmul2_rn(make_float2(cc[0], cc[0]), v);
  s = __ffma2_rn(c1, px, s);
  s = __ffma2_rn(c1, py, s);
  return __ffma2_rn(c1, pz, s);
}

// leapfrog_compensated on two columns; -u - bb is -(u + bb), exactly.
__device__ __forceinline__ float2 leapfrog_compensated2(float2 v, float2 u, float2 r2, float2 lap) {
  const float2 a = __fadd2_rn(v, v);
  const float2 s = f2_sub(a, u);
  const float2 bb = f2_sub(s, a);
  const float2 e = f2_sub(f2_sub(a, f2_sub(s, bb)), __fadd2_rn(u, bb));
  return __fadd2_rn(s, __ffma2_rn(r2, lap, e));
}

__device__ __forceinline__ int pmod(int a, int m) { return ((a % m) + m) % m; }


template <int OP, class T, bool COMP, int TT, int NTX, int NTY, int CY, int VX, bool TMA = false>
struct FusedShape {
  using ST = typename StorageOf<T>::type;
  static constexpr int R = OpTraits<OP>::R;
  static constexpr int TO = OpTraits<OP>::TO;
  static constexpr int D = R + 1;                            // planes between time levels
  static constexpr int QL = TO == 2 ? 2 * R + 2 : 2 * R + 1;  // z-queue length
  static constexpr int U = QL % 2 == 0 ? QL : 2 * QL;         // z-loop unroll: even multiple of QL
  static constexpr int RW = NTX * VX, RY = NTY * CY;          // column region
  static constexpr int RP = (R + VX - 1) / VX * VX;           // column padding, a whole number of x groups
  static constexpr int PW = RW + 2 * RP, PR = RY + 2 * R;     // shared rows padded by RP, rows by R
  static constexpr int H = TT * R;
  // x alignment of the region start: one x group, or 16 bytes for TMA boxes
  static constexpr int ALIGN = TMA ? (16 / (int)sizeof(ST) > VX ? 16 / (int)sizeof(ST) : VX) : VX;
  // output tile width: without TMA a multiple of ALIGN when that loses no
  // more columns than an arbitrary start does (every tile then starts aligned,
  // the region start X0 - H is off by the same MIS columns in every tile, and
  // each x group lies wholly inside or outside the output); otherwise any
  // width with up to ALIGN-1 columns of alignment slack (fused_tile_width in
  // fused.cu computes the same)
  static constexpr int MIS = ((-H) % ALIGN + ALIGN) % ALIGN;
  static constexpr int BXA = (RW - 2 * H - MIS) / ALIGN * ALIGN, BXU = RW - 2 * H - (ALIGN - 1);
  // (double-float tiles keep the general width too: their one-column and x-group
  // variants share regions, and an output tile names one variant)
  static constexpr bool ALIGNED_W = !TMA && !std::is_same<T, Df64>::value;
  static constexpr int BX = ALIGNED_W && BXA >= BXU ? BXA : BXU, BY = RY - 2 * H;  // output tile
  static constexpr size_t field_bytes = (size_t)2 * TT * PR * PW * sizeof(T);
  // TMA rings: NB planes of the input state (and the old state), NR planes of roc2
  static constexpr int NB = fused_tma_nb(R, TT, RW * RY);
  static constexpr int NR = fused_tma_nr(R, TT, NB);
  static constexpr size_t plane_bytes = (size_t)RW * RY * sizeof(ST);
  static constexpr size_t off_cur = (field_bytes + 127) / 128 * 128;
  static constexpr size_t off_prev = off_cur + NB * plane_bytes;
  static constexpr size_t off_roc2 = off_prev + (TO == 2 ? NB * plane_bytes : 0);
  static constexpr size_t off_bar = off_roc2 + (TO == 2 ? NR * plane_bytes : 0);
  static constexpr size_t smem_bytes = TMA ? off_bar + NB * sizeof(uint64_t) : field_bytes;
};

// One CTA-tile of a fused pass: tile (bxi, byi) of the x-y tiling, z chunk bzi
// (planes [R + bzi*zchunk, ...)), or, with zlo >= 0, planes [zlo, zhi),
// executed by the NTX*NTY threads of the calling CTA (thread (tx, ty)).  Used by
// the single-grid persistent kernels below (one call per piece of work; `first`
// on the CTA's first, later calls re-initialise the TMA barriers) and by the
// batched persistent kernel.
template <int OP, class T, bool COMP, int TT, int NTX, int NTY, int CY, int VX, bool TMA = false, bool SRC = false>
__device__ __forceinline__ void fused_tile(const FusedArgs<typename StorageOf<T>::type> &a, int bxi, int byi,
                                           int bzi, int tx, int ty, unsigned char *smraw,
                                           const TmaMaps *maps = nullptr, int zlo = -1, int zhi = -1,
                                           bool first = true) {
  using Sh = FusedShape<OP, T, COMP, TT, NTX, NTY, CY, VX, TMA>;
  using ST = typename StorageOf<T>::type;
  constexpr int R = Sh::R, TO = Sh::TO, D = Sh::D, QL = Sh::QL, U = Sh::U;
  constexpr int RW = Sh::RW, RY = Sh::RY, RP = Sh::RP, PW = Sh::PW, PR = Sh::PR, H = Sh::H, BX = Sh::BX,
                BY = Sh::BY;
  unsigned range_bad = 0;
  unsigned *const flag = a.range_flag;               // checked build: bounds violations
  constexpr int64_t SMB = (int64_t)Sh::smem_bytes;   // shared allocation of the CTA
  static_assert(PW % VX == 0 && RP % VX == 0, "x groups must stay vector-aligned in shared memory");
  static_assert(BX > 0 && BY > 0, "tile too small for the fusion depth");
  static_assert(TT * CY * VX <= 32, "activity mask holds 32 (level, row, column) bits");

  // [2 buffers][TT levels][PR rows][PW columns]; the padding is never written and
  // only feeds values that are discarded, so every neighbour read stays in bounds
  T *sm = reinterpret_cast<T *>(smraw);

  const Geom &g = a.g;
  // 32-bit element offsets: fused_supported() limits the fused schedule to
  // grids of fewer than 2^31 elements per array
  const int plane = (int)g.plane;
  const int X0 = bxi * BX, Y0 = byi * BY;
  const int Z0 = zlo >= 0 ? zlo : R + bzi * a.zchunk;
  const int Z1 = zlo >= 0 ? zhi : min(Z0 + a.zchunk, g.nnz - R);
  const int sb = max(0, Z0 - H);
  const int se = Z1 - 1 + TT * D;
  const int s0 = sb - sb % U;  // plane p lives in queue slot p mod QL; buffer parity = PH parity

  // region start, aligned so that every thread's x-group is one aligned vector
  // in memory (and, for TMA, so that the box starts on a 16-byte boundary)
  const int xs = X0 - H - pmod(X0 - H + R + g.ox, Sh::ALIGN);
  const int xi0 = xs + tx * VX;  // interior x index of the thread's first column

  bool x_dom[VX], x_outc[VX];
  unsigned x_act = 0;  // bit (l-1)*VX + v: column v inside level l's valid x range
#pragma unroll
  for (int v = 0; v < VX; v++) {
    const int xi = xi0 + v;
    x_dom[v] = xi + R >= 0 && xi + R < g.nnx;
    const bool x_int = xi >= 0 && xi < g.nx;
    x_outc[v] = x_int && xi >= X0 && xi < X0 + BX;
#pragma unroll
    for (int l = 1; l <= TT; l++)
      if (x_int && xi >= X0 - (TT - l) * R && xi < X0 + BX + (TT - l) * R) x_act |= 1u << ((l - 1) * VX + v);
  }
  const bool xg_dom = x_dom[0] && x_dom[VX - 1];

  bool y_dom[CY], y_outr[CY];
  int col[CY];
  unsigned act = 0;  // bit ((l-1)*CY + c)*VX + v
#pragma unroll
  for (int c = 0; c < CY; c++) {
    const int yj = Y0 - H + ty + c * NTY;
    y_dom[c] = yj + R >= 0 && yj + R < g.nny;
    const bool y_int = yj >= 0 && yj < g.ny;
    y_outr[c] = y_int && yj >= Y0 && yj < Y0 + BY;
    col[c] = (yj + R) * g.px + g.ox + (xi0 + R);
#pragma unroll
    for (int l = 1; l <= TT; l++)
      if (y_int && yj >= Y0 - (TT - l) * R && yj < Y0 + BY + (TT - l) * R)
#pragma unroll
        for (int v = 0; v < VX; v++)
          if (x_act >> ((l - 1) * VX + v) & 1u) act |= 1u << (((l - 1) * CY + c) * VX + v);
  }

  T cc[5];
#pragma unroll
  for (int m = 0; m < 5; m++) cc[m] = coef_arg<T>(a, m);
  // the same coefficients as packed pairs, for the double-float column pairs
  [[maybe_unused]] Df2 cc2[5];
  if constexpr (std::is_same<T, Df64>::value) {
#pragma unroll
    for (int m = 0; m < 5; m++) cc2[m] = df2(cc[m], cc[m]);
  }
  // variable coefficients (operators 2-5): full precision, or BF16 with a
  // per-array scale in the mixed form (COMP selects BF16 for these operators)
  constexpr bool VAR = OpTraits<OP>::VAR;

  // source point: its plane, and per row the position inside this thread's
  // x group (-1: not this thread's)
  int src_z = -(1 << 30), src_v[CY];
#pragma unroll
  for (int c = 0; c < CY; c++) src_v[c] = -1;
  if (SRC && a.src != nullptr) {
    src_z = a.src_off / plane;
    const int xy = a.src_off - src_z * plane;
#pragma unroll
    for (int c = 0; c < CY; c++) src_v[c] = (xy - col[c] >= 0 && xy - col[c] < VX) ? xy - col[c] : -1;
  }

  T q[TT][CY][VX][QL];
#pragma unroll
  for (int l = 0; l < TT; l++)
#pragma unroll
    for (int c = 0; c < CY; c++)
#pragma unroll
      for (int v = 0; v < VX; v++)
#pragma unroll
        for (int e = 0; e < QL; e++) q[l][c][v][e] = T(0);

  // shared-memory element of this thread's first column, row c, level l, buffer b:
  //   sm + thr + ((b*TT + l)*PR + c*NTY)*PW   (compile-time offsets from thr)
  T *const thr = sm + (ty + R) * PW + tx * VX + RP;

  // TMA: one thread streams whole region planes into shared-memory rings,
  // NB-1 planes ahead of the z step that consumes them
  constexpr int NB = Sh::NB, NR = Sh::NR;
  const int tid = ty * NTX + tx;
  ST *const ring_cur = reinterpret_cast<ST *>(smraw + Sh::off_cur);
  ST *const ring_prev = reinterpret_cast<ST *>(smraw + Sh::off_prev);
  ST *const ring_roc2 = reinterpret_cast<ST *>(smraw + Sh::off_roc2);
  uint64_t *const bars = reinterpret_cast<uint64_t *>(smraw + Sh::off_bar);
  const int xg = xs + R + g.ox, yg = Y0 - H + R;  // global x / row of the region origin
  unsigned tma_timeout = 0;
  auto tma_issue = [&](int t) {  // input planes of z step t (thread 0 only)
    if constexpr (TMA) {
      const int k = (t - s0) & (NB - 1);
      unsigned bytes = (unsigned)Sh::plane_bytes;
      if constexpr (TO == 2) bytes *= 3;
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(&bars[k], bytes);
      tma_load_3d(ring_cur + (size_t)k * RW * RY, &maps->cur, xg, yg, t, &bars[k]);
      if constexpr (TO == 2) {
        tma_load_3d(ring_prev + (size_t)k * RW * RY, &maps->prev, xg, yg, t - D, &bars[k]);
        tma_load_3d(ring_roc2 + (size_t)((t - s0) & (NR - 1)) * RW * RY, &maps->roc2, xg, yg, t - D, &bars[k]);
      }
    }
  };
  if constexpr (TMA) {
    if (tid == 0) {  // every phase restarts at 0; a barrier of an earlier piece is invalidated first
      for (int k = 0; k < NB; k++) {
        if (!first) mbar_inval(&bars[k]);
        mbar_init(&bars[k], 1);
      }
      mbar_init_fence();
    }
    __syncthreads();
    if (tid == 0)
      for (int t = s0; t < s0 + NB - 1 && t <= se; t++) tma_issue(t);
  }

  for (int sbase = s0; sbase <= se; sbase += U) {
    static_for<U>([&](auto ph_c) {
      constexpr int PH = decltype(ph_c)::value;
      constexpr int RB = (PH + 1) & 1, WB = PH & 1;  // read buffer (s-1) and write buffer (s)
      const int s = sbase + PH;
      if (s > se) return;  // uniform over the CTA
      const int soff = s * plane;

      if constexpr (TMA) {
        if (tid == 0 && s + NB - 1 <= se) tma_issue(s + NB - 1);
        if (!mbar_wait(&bars[(s - s0) & (NB - 1)], ((s - s0) / NB) & 1, 1u << 26)) tma_timeout = 1;
      }
      // roc2 (and, for level 1, the old state) of every level: from the TMA rings,
      // or issued before the level loop so that their latency overlaps the higher
      // levels' arithmetic
      Pack<T, VX> r2c[TO == 2 ? TT : 1][CY], pvc[CY];
      if constexpr (TO == 2 && TMA) {
#pragma unroll
        for (int l = TT; l >= 1; l--) {
          const int kr = (s - s0 - (l - 1) * D + NR) & (NR - 1);
#pragma unroll
          for (int c = 0; c < CY; c++) {
            const size_t off = (size_t)(ty + c * NTY) * RW + tx * VX;
            Pack<ST, VX> raw;
#pragma unroll
            for (int v = 0; v < VX; v++) raw.e[v] = ST(0);
            const ST *pr = ring_roc2 + (size_t)kr * RW * RY + off;
            if (in_shared(pr, VX * sizeof(ST), smraw, SMB, flag)) raw.load(pr);
#pragma unroll
            for (int v = 0; v < VX; v++) r2c[l - 1][c].e[v] = to_compute<T>(raw.e[v], range_bad);
            if (l == 1) {
              const ST *pp = ring_prev + (size_t)((s - s0) & (NB - 1)) * RW * RY + off;
              if (in_shared(pp, VX * sizeof(ST), smraw, SMB, flag)) raw.load(pp);
#pragma unroll
              for (int v = 0; v < VX; v++) pvc[c].e[v] = to_compute<T>(raw.e[v], range_bad);
            }
          }
        }
      } else if constexpr (TO == 2) {
#pragma unroll
        for (int l = TT; l >= 1; l--) {
          const int p = s - l * D;
          const bool p_int = p >= R && p < g.nnz - R;
#pragma unroll
          for (int c = 0; c < CY; c++) {
            const int at = p * plane + col[c];
#pragma unroll
            for (int v = 0; v < VX; v++) r2c[l - 1][c].e[v] = T(0);
            if (l == 1)
#pragma unroll
              for (int v = 0; v < VX; v++) pvc[c].e[v] = T(0);
            if (p_int && ((act >> (((l - 1) * CY + c) * VX)) & ((1u << VX) - 1)) &&
                in_array(at, VX, g.elems, flag)) {
              r2c[l - 1][c].ldg(a.roc2 + at, range_bad);
              if (l == 1) pvc[c].ldg(a.prev + at, range_bad);
            }
          }
        }
      }

      // levels TT..1, highest first: level l reads level l-1's queues before
      // level l-1 stores this step's plane
      static_for<TT>([&](auto li_c) {
        constexpr int L = TT - decltype(li_c)::value;  // TT, TT-1, ..., 1
        constexpr int SL = qslot<QL>(PH - L * D);        // slot of plane p in every queue
        const int p = s - L * D;
        const bool p_int = p >= R && p < g.nnz - R;
        const bool p_out = p_int && p >= Z0 && p < Z1;
        const int poff = soff - L * D * plane;
#pragma unroll
        for (int c = 0; c < CY; c++) {
          const T *srow = thr + ((RB * TT + (L - 1)) * PR + c * NTY) * PW;
          T val[VX];
          // radius-1 constant-coefficient levels in FP32 or double-float: column
          // pairs in packed f32x2 arithmetic (below)
          constexpr bool PAIRS = std::is_same<T, float>::value && R == 1 && !VAR && (OP == 1 || OP == 8) &&
                                 VX % 2 == 0;
          constexpr bool DPAIRS = std::is_same<T, Df64>::value && R == 1 && !VAR && (OP == 1 || OP == 8) &&
                                  VX % 2 == 0;
          // their x neighbours across the group's edges are the last column of the
          // lane to the left and the first column of the lane to the right, read by
          // warp shuffles while the warp is still converged (at the region's x edges,
          // and across a warp's row boundary, the value is one that the tile discards,
          // as the unwritten shared-memory padding is)
          [[maybe_unused]] T xe[2];
          if constexpr (PAIRS || DPAIRS) {
            constexpr unsigned kAll = 0xffffffffu;
            if constexpr (PAIRS) {
              xe[0] = __shfl_up_sync(kAll, q[L - 1][c][VX - 1][SL], 1);
              xe[1] = __shfl_down_sync(kAll, q[L - 1][c][0][SL], 1);
            } else {
              xe[0] = T(__shfl_up_sync(kAll, q[L - 1][c][VX - 1][SL].hi, 1),
                        __shfl_up_sync(kAll, q[L - 1][c][VX - 1][SL].lo, 1));
              xe[1] = T(__shfl_down_sync(kAll, q[L - 1][c][0][SL].hi, 1),
                        __shfl_down_sync(kAll, q[L - 1][c][0][SL].lo, 1));
            }
          }
          // rows outside level L's valid band (or halo planes) only carry their
          // value: a warp covers whole rows, so this branch is warp-uniform except
          // at the two x edges of the region
          const bool row_on = p_int && ((act >> (((L - 1) * CY + c) * VX)) & ((1u << VX) - 1)) &&
                              in_shared(srow - R * PW - RP, (int64_t)(2 * R * PW + VX + 2 * RP) * sizeof(T), smraw,
                                        SMB, flag) &&
                              (!VAR || in_array(poff + col[c], VX, g.elems, flag));
          if (!row_on) {
#pragma unroll
            for (int v = 0; v < VX; v++) val[v] = q[L - 1][c][v][SL];
          } else {
          T yv[2 * R][VX];
#pragma unroll
          for (int d = 1; d <= R; d++) {
            Pack<T, VX> up, dn;
            up.load(srow + d * PW);
            dn.load(srow - d * PW);
#pragma unroll
            for (int v = 0; v < VX; v++) {
              yv[d - 1][v] = up.e[v];
              yv[R + d - 1][v] = dn.e[v];
            }
          }
          // variable coefficients of the group at this plane: one vector load per
          // array (the row is interior, so the whole group lies inside the array)
          constexpr int NCF = VAR ? OpTraits<OP>::NC : 1;
          T cf[NCF][VX];
          if constexpr (VAR) load_coef_group<T, COMP, NCF, VX>(a.coef, g.elems, a.cscale, poff + col[c], cf);
          // x neighbours outside the group: the neighbouring groups as two vector loads
          Pack<T, VX> xlp, xrp;
          if constexpr (fused_x_groups(R, VX)) {
            xlp.load(srow - VX);
            xrp.load(srow + VX);
          }
          // radius-1 constant-coefficient operators in FP32: column pairs in f32x2
          if constexpr (PAIRS) {
            static_for<VX / 2>([&](auto p_c) {
              constexpr int V0 = 2 * decltype(p_c)::value, V1 = V0 + 1;
              const FusedAcc<R, T, QL, SL, VX, V0, true> a0{srow, q[L - 1][c], yv, xlp.e, xrp.e, xe};
              const FusedAcc<R, T, QL, SL, VX, V1, true> a1{srow, q[L - 1][c], yv, xlp.e, xrp.e, xe};
              const float2 v2 = make_float2(a0.c(), a1.c());
              const float2 lap = star1_sum2(cc, v2, __fadd2_rn(make_float2(a0.x(1), a1.x(1)), make_float2(a0.x(-1), a1.x(-1))),
                                            __fadd2_rn(make_float2(a0.y(1), a1.y(1)), make_float2(a0.y(-1), a1.y(-1))),
                                            __fadd2_rn(make_float2(a0.z(1), a1.z(1)), make_float2(a0.z(-1), a1.z(-1))));
              float2 cand;
              if constexpr (TO == 2) {
                float2 uold;
                if constexpr (L >= 2) uold = make_float2(q[L - 2][c][V0][SL], q[L - 2][c][V1][SL]);
                else uold = make_float2(pvc[c].e[V0], pvc[c].e[V1]);
                const float2 r2 = make_float2(r2c[L - 1][c].e[V0], r2c[L - 1][c].e[V1]);
                if constexpr (COMP) cand = leapfrog_compensated2(v2, uold, r2, lap);
                else cand = __ffma2_rn(r2, lap, f2_sub(__fadd2_rn(v2, v2), uold));  // (2v - u) + roc2*lap
              } else {
                cand = lap;
              }
              const bool on0 = p_int && (act >> (((L - 1) * CY + c) * VX + V0) & 1u);
              const bool on1 = p_int && (act >> (((L - 1) * CY + c) * VX + V1) & 1u);
              val[V0] = on0 ? cand.x : v2.x;  // halo and out-of-region points keep their value
              val[V1] = on1 ? cand.y : v2.y;
            });
          } else if constexpr (DPAIRS) {
            // double-float radius-1 constant-coefficient levels: column pairs with
            // packed f32x2 arithmetic, each lane the scalar Df64 code's operations
            static_for<VX / 2>([&](auto p_c) {
              constexpr int V0 = 2 * decltype(p_c)::value, V1 = V0 + 1;
              const FusedAcc<R, T, QL, SL, VX, V0, true> a0{srow, q[L - 1][c], yv, xlp.e, xrp.e, xe};
              const FusedAcc<R, T, QL, SL, VX, V1, true> a1{srow, q[L - 1][c], yv, xlp.e, xrp.e, xe};
              const PairAcc<FusedAcc<R, T, QL, SL, VX, V0, true>, FusedAcc<R, T, QL, SL, VX, V1, true>> acc2{a0, a1};
              const Df2 centre = acc2.c();
              const Df2 lap = star_grouped_sum<R, FastArith>(cc2, acc2);
              Df2 cand;
              if constexpr (TO == 2) {
                Df2 uold;
                if constexpr (L >= 2) uold = df2(q[L - 2][c][V0][SL], q[L - 2][c][V1][SL]);
                else uold = df2(pvc[c].e[V0], pvc[c].e[V1]);
                cand = (twice(centre) - uold) + df2(r2c[L - 1][c].e[V0], r2c[L - 1][c].e[V1]) * lap;
              } else {
                cand = lap;
              }
              cand = df_norm(cand);
              const bool on0 = p_int && (act >> (((L - 1) * CY + c) * VX + V0) & 1u);
              const bool on1 = p_int && (act >> (((L - 1) * CY + c) * VX + V1) & 1u);
              val[V0] = on0 ? df2_x(cand) : df2_x(centre);  // halo and out-of-region points keep their value
              val[V1] = on1 ? df2_y(cand) : df2_y(centre);
            });
          } else
          static_for<VX>([&](auto v_c) {
            constexpr int V = decltype(v_c)::value;
            const T centre = q[L - 1][c][V][SL];
            // with one column per thread the row test above already decided
            const bool on = VX == 1 || (p_int && (act >> (((L - 1) * CY + c) * VX + V) & 1u));
            // double-float arithmetic is ~10x the FP32 work: skip inactive points
            // with a branch there; the FP32/FP64 paths stay branch-free
            constexpr bool heavy = std::is_same<T, Df64>::value;
            if (heavy && !on) {
              val[V] = centre;
              return;
            }
            FusedAcc<R, T, QL, SL, VX, V> acc{srow, q[L - 1][c], yv, xlp.e, xrp.e};
            T cand;
            if constexpr (heavy && !VAR) {
              const T lap = star_grouped_sum<R, FastArith>(cc, acc);
              if constexpr (TO == 2) {
                T uold;
                if constexpr (L >= 2) uold = q[L - 2][c][V][SL];
                else uold = pvc[c].e[V];
                cand = twice_minus(centre, uold) + r2c[L - 1][c].e[V] * lap;
              } else {
                cand = lap;
              }
            } else if constexpr (TO == 2) {
              T uold;
              if constexpr (L >= 2) uold = q[L - 2][c][V][SL];
              else uold = pvc[c].e[V];
              const T r2 = r2c[L - 1][c].e[V];
              if constexpr (COMP) {
                cand = leapfrog_compensated(centre, uold, r2, star_const_sum<R, FastArith>(cc, acc));
              } else {
                CoefFull<T> none{nullptr, 0};
                cand = apply_op<OP, FastArith>(cc, none, 0, acc, uold, r2);
              }
            } else if constexpr (VAR) {
              CoefGroup<T, NCF, VX, V> cg{cf};
              cand = apply_op<OP, FastArith>(cc, cg, 0, acc, T(0), T(0));
            } else {
              CoefFull<T> none{nullptr, 0};
              cand = apply_op<OP, FastArith>(cc, none, 0, acc, T(0), T(0));
            }
            if constexpr (heavy) val[V] = df_norm(cand);  // inactive points took the branch above
            else val[V] = on ? cand : centre;  // halo and out-of-region points keep their value
          });
          }
          // source point of step src_t0 + L - 1, added after the update's rounding
          // (every tile holding the point adds it, so overlapping halos agree)
          if (SRC && p == src_z && src_v[c] >= 0) {
            const int st = a.src_t0 + L - 1;
            if (st < a.src_n) {
              const T sv = coef_to_compute<T>(a.src[st]);
              static_for<VX>([&](auto v_c) {
                constexpr int V = decltype(v_c)::value;
                if (V == src_v[c]) {
                  if constexpr (std::is_same<T, Df64>::value) val[V] = df_norm(val[V] + sv);
                  else val[V] = val[V] + sv;
                }
              });
            }
          }
          if constexpr (L == TT || L == TT - 1) {
            if (p_out && y_outr[c] && (L == TT || a.write_prev) && in_array(poff + col[c], VX, g.elems, flag)) {
              ST *dst = (L == TT ? a.out_cur : a.out_prev) + poff + col[c];
              unsigned *cov = L == TT ? a.cov_cur : a.cov_prev;
              if (x_outc[0] && x_outc[VX - 1]) {
                Pack<T, VX> o;
#pragma unroll
                for (int v = 0; v < VX; v++) o.e[v] = val[v];
                o.stg(dst);
                count_writes(cov, poff + col[c], VX);
              } else {
#pragma unroll
                for (int v = 0; v < VX; v++)
                  if (x_outc[v]) {
                    dst[v] = to_storage<ST>(val[v]);
                    count_writes(cov, poff + col[c] + v, 1);
                  }
              }
            }
          }
          if constexpr (L < TT) {
#pragma unroll
            for (int v = 0; v < VX; v++) q[L][c][v][SL] = val[v];
          }
        }
      });
      // level 0: stream plane s from HBM
      const bool s_in = s < g.nnz;
#pragma unroll
      for (int c = 0; c < CY; c++) {
        Pack<T, VX> in;
#pragma unroll
        for (int v = 0; v < VX; v++) in.e[v] = T(0);
        if constexpr (TMA) {
          Pack<ST, VX> raw;  // out-of-range boxes are zero-filled by the copy
#pragma unroll
          for (int v = 0; v < VX; v++) raw.e[v] = ST(0);
          const ST *pc = ring_cur + (size_t)((s - s0) & (NB - 1)) * RW * RY + (size_t)(ty + c * NTY) * RW + tx * VX;
          if (in_shared(pc, VX * sizeof(ST), smraw, SMB, flag)) raw.load(pc);
#pragma unroll
          for (int v = 0; v < VX; v++) in.e[v] = to_compute<T>(raw.e[v], range_bad);
        } else if (s_in && y_dom[c]) {
          if (xg_dom) {
            if (in_array(soff + col[c], VX, g.elems, flag)) in.ldg(a.cur + soff + col[c], range_bad);
          } else {
#pragma unroll
            for (int v = 0; v < VX; v++)
              if (x_dom[v] && in_array(soff + col[c] + v, 1, g.elems, flag))
                in.e[v] = to_compute<T>(ldg_elem(a.cur + soff + col[c] + v), range_bad);
          }
        }
#pragma unroll
        for (int v = 0; v < VX; v++) q[0][c][v][qslot<QL>(PH)] = in.e[v];
        if constexpr (TT == 1) {
          if (a.write_prev && s >= R && s < g.nnz - R && s >= Z0 && s < Z1 && y_outr[c])
#pragma unroll
            for (int v = 0; v < VX; v++)
              if (x_outc[v] && in_array(soff + col[c] + v, 1, g.elems, flag)) {
                a.out_prev[soff + col[c] + v] = to_storage<ST>(in.e[v]);
                count_writes(a.cov_prev, soff + col[c] + v, 1);
              }
        }
      }
      // publish each level's centre plane (s - l*D - R) for the x/y neighbours of step s+1
#pragma unroll
      for (int l = 0; l < TT; l++)
#pragma unroll
        for (int c = 0; c < CY; c++) {
          Pack<T, VX> o;
#pragma unroll
          for (int v = 0; v < VX; v++) o.e[v] = q[l][c][v][qslot<QL>(PH - l * D - R)];
          T *const dst = thr + ((WB * TT + l) * PR + c * NTY) * PW;
          if (in_shared(dst, VX * sizeof(T), smraw, SMB, flag)) o.store(dst);
        }
      __syncthreads();
    });
  }
  if constexpr (TMA) {
    if (tma_timeout && a.range_flag) atomicOr(a.range_flag, 2u);  // a copy never completed
  }
}

// Persistent schedule of a single-grid pass over gx*gy tiles (row-major) and
// nz planes on gridDim.x CTAs, as pieces (tile, planes [za, zb)) handed to
// f(bxi, byi, za, zb, first):
//   phase 1: CTA b takes whole tiles b, b + C, b + 2C, ... (C = gridDim.x) while
//     C of them remain, so that all CTAs stream the same planes at the same time
//     and neighbouring tiles share their overlapping halo boxes in L2;
//   phase 2: each of the `rest` remaining tiles is split into k equal plane
//     ranges (k from fused_phase2_parts), pieces numbered tile by tile and
//     dealt in rounds of C, so that the pieces of neighbouring tiles over the
//     same planes run at the same time; the pieces of a last, partial round go
//     to CTAs spread evenly over the grid (piece q of Q to CTA q*C/Q), not to
//     the first Q, which the hardware would place on neighbouring SMs.
// Each piece pays the z pipeline's fill once (against once per z chunk of a
// (tile, chunk) grid).  32-bit work indices: tiles x planes <= points < 2^31
// (fused_supported).
template <class F> __device__ __forceinline__ void for_each_piece(int gx, int gy, int nz, int k, F &&f) {
  const int tiles = gx * gy, C = gridDim.x, b = blockIdx.x;
  const int full = tiles / C;
  bool first = true;
  for (int r = 0; r < full; r++) {
    const int t = r * C + b;
    f(t % gx, t / gx, 0, nz, first);
    first = false;
  }
  const int rest = tiles - full * C;
  if (rest == 0) return;
  k = max(1, min(nz, k));
  const int P = k * rest;
  for (int base = 0; base < P; base += C) {
    const int Q = min(C, P - base);
    const int q = (int)(((int64_t)b * Q + C - 1) / C);  // the one piece q with q*C/Q == b, if any
    if (q < Q && (int)((int64_t)q * C / Q) == b) {
      const int p = base + q, t = full * C + p / k, part = p % k;
      f(t % gx, t / gx, part * nz / k, (part + 1) * nz / k, first);
      first = false;
    }
  }
}

template <int OP, class T, bool COMP, int TT, int NTX, int NTY, int CY, int VX, bool TMA, bool SRC>
__device__ __forceinline__ void fused_pieces(const FusedArgs<typename StorageOf<T>::type> &a, unsigned char *smraw,
                                             const TmaMaps *maps) {
  using Sh = FusedShape<OP, T, COMP, TT, NTX, NTY, CY, VX, TMA>;
  const Geom &g = a.g;
  for_each_piece((g.nx + Sh::BX - 1) / Sh::BX, (g.ny + Sh::BY - 1) / Sh::BY, g.nz, a.zchunk,
                 [&](int bxi, int byi, int za, int zb, bool first) {
                   fused_tile<OP, T, COMP, TT, NTX, NTY, CY, VX, TMA, SRC>(a, bxi, byi, 0, threadIdx.x, threadIdx.y,
                                                                          smraw, maps, Sh::R + za, Sh::R + zb, first);
                 });
}

template <int OP, class T, bool COMP, int TT, int NTX, int NTY, int CY, int VX, bool SRC = false>
__global__ void __launch_bounds__(NTX *NTY) fused_pass(FusedArgs<typename StorageOf<T>::type> a) {
  extern __shared__ __align__(128) unsigned char smraw[];
  fused_pieces<OP, T, COMP, TT, NTX, NTY, CY, VX, false, SRC>(a, smraw, nullptr);
}

// The same pass with the input planes staged by TMA; the tensor maps travel as
// grid constants.  This one keeps a grid of (tile, z chunk) CTAs, x fastest:
// the CTAs running at one time are neighbouring tiles at the same z, whose
// overlapping halo boxes then come from L2 (the persistent order above ran
// the 512^3 mixed leapfrog at 451 against 550 GLUP/s).
template <int OP, class T, bool COMP, int TT, int NTX, int NTY, int CY, int VX>
__global__ void __launch_bounds__(NTX *NTY)
    fused_pass_tma(FusedArgs<typename StorageOf<T>::type> a, const __grid_constant__ TmaMaps maps) {
  extern __shared__ __align__(128) unsigned char smraw[];
  fused_tile<OP, T, COMP, TT, NTX, NTY, CY, VX, true>(a, blockIdx.x, blockIdx.y, blockIdx.z, threadIdx.x,
                                                      threadIdx.y, smraw, &maps);
}

// CTAs of a persistent pass (for_each_piece) over `tiles` x-y tiles and nz
// planes with `cap` resident CTAs: every resident slot, as long as each gets
// at least one plane.
inline int64_t fused_persistent_ctas(const Geom &g, int64_t tiles, int64_t cap) {
  return std::max<int64_t>(1, std::min<int64_t>(cap, tiles * g.nz));
}

// Plane split k of the tiles left after the whole-tile rounds of a persistent
// pass on C CTAs: the k (<= 64) with the fewest rounds x (planes per piece +
// the pipeline's `over` fill planes), the smaller k on a tie.
inline int fused_phase2_parts(int64_t tiles, int64_t C, int nz, int over) {
  const int64_t rest = tiles % C;
  if (rest == 0) return 1;
  int best_k = 1;
  int64_t best = INT64_MAX;
  for (int k = 1; k <= 64 && k <= nz; k++) {
    const int64_t rounds = (rest * k + C - 1) / C, cost = rounds * ((nz + k - 1) / k + over);
    if (cost < best) {
      best = cost;
      best_k = k;
    }
  }
  return best_k;
}

// z chunk length of a (tile, z chunk) grid: split the z range so that waves x
// (chunk + pipeline overhead `over` planes) is smallest over `tiles` x-y tiles
// and `cap` resident CTAs.
inline int fused_zchunk(const Geom &g, int64_t tiles, int64_t cap, int over) {
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
  return (g.nz + best_n - 1) / best_n;
}

// Prepare a fused kernel for launch on the current device: opt in to its
// dynamic shared memory (a function attribute of each device, set once per
// (kernel, device) from any host thread) and return its resident CTAs per SM.
inline cudaError_t fused_kernel_setup(const void *kern, size_t smem, int threads,
                                      std::atomic<unsigned long long> &attr_set, int *occ_out, int *nsm_out) {
  int dev = 0;
  cudaGetDevice(&dev);
  const unsigned long long dev_bit = 1ull << (dev & 63);
  if (!(attr_set.load(std::memory_order_acquire) & dev_bit)) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_set.fetch_or(dev_bit, std::memory_order_release);
  }
  int occ = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, smem);
  *occ_out = occ < 1 ? 1 : occ;
  int nsm = 152;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  *nsm_out = nsm;
  return cudaSuccess;
}

// Kernel arguments of one fused pass.
template <class ST> FusedArgs<ST> make_fused_args(const Geom &g, const FusedLaunch &L, int zchunk) {
  FusedArgs<ST> a{};
  a.g = g;
  a.prev = static_cast<const ST *>(L.prev);
  a.cur = static_cast<const ST *>(L.cur);
  a.roc2 = static_cast<const ST *>(L.roc2);
  a.out_prev = static_cast<ST *>(L.out_prev);
  a.out_cur = static_cast<ST *>(L.out_cur);
  for (int m = 0; m < 5; m++) a.cc[m] = L.cc[m];
  split_coefs(a.cc, a.cch, a.ccl);
  a.range_flag = L.range_flag;
  a.coef = L.coef;
  a.cscale = L.cscale;
  a.src = L.src;
  a.src_off = L.src_off;
  a.src_t0 = L.src_t0;
  a.src_n = L.src_n;
  a.cov_prev = L.cov_prev;
  a.cov_cur = L.cov_cur;
  a.zchunk = zchunk;
  a.write_prev = L.write_prev;
  return a;
}

template <int OP, class T, bool COMP, int TT, int NTX, int NTY, int CY, int VX, bool TMA, bool SRC = false>
cudaError_t launch_tt(const Geom &g, const FusedLaunch &L, cudaStream_t s) {
  using S = FusedShape<OP, T, COMP, TT, NTX, NTY, CY, VX, TMA>;
  constexpr int R = S::R, BX = S::BX, BY = S::BY;
  void *kern;
  if constexpr (TMA) kern = (void *)fused_pass_tma<OP, T, COMP, TT, NTX, NTY, CY, VX>;
  else kern = (void *)fused_pass<OP, T, COMP, TT, NTX, NTY, CY, VX, SRC>;
  const size_t smem = S::smem_bytes;
  static std::atomic<unsigned long long> attr_set{0};
  int occ = 1, nsm = 152;
  cudaError_t e = fused_kernel_setup(kern, smem, NTX * NTY, attr_set, &occ, &nsm);
  if (e != cudaSuccess) return e;
  const int gx = (g.nx + BX - 1) / BX, gy = (g.ny + BY - 1) / BY;
  int64_t ctas = 1;
  int zchunk = 1, nz_ch = 1;
  if constexpr (TMA) {
    zchunk = fused_zchunk(g, (int64_t)gx * gy, (int64_t)nsm * occ, TT * R + TT * (R + 1));
    nz_ch = (g.nz + zchunk - 1) / zchunk;
  } else {
    ctas = fused_persistent_ctas(g, (int64_t)gx * gy, (int64_t)nsm * occ);
    zchunk = fused_phase2_parts((int64_t)gx * gy, ctas, g.nz, TT * R + TT * (R + 1));
  }
  using ST = typename StorageOf<T>::type;
  FusedArgs<ST> a = make_fused_args<ST>(g, L, zchunk);
  if constexpr (TMA) {
    if (!L.tma_cur || !L.tma_roc2 || !L.tma_prev) return cudaErrorInvalidValue;
    // the copies must fill exactly the ring slots this shape sizes
    if (L.tma_box_w != S::RW || L.tma_box_h != S::RY) return cudaErrorInvalidValue;
    TmaMaps maps;
    maps.cur = *static_cast<const CUtensorMap *>(L.tma_cur);
    maps.prev = *static_cast<const CUtensorMap *>(L.tma_prev);
    maps.roc2 = *static_cast<const CUtensorMap *>(L.tma_roc2);
    fused_pass_tma<OP, T, COMP, TT, NTX, NTY, CY, VX><<<dim3(gx, gy, nz_ch), dim3(NTX, NTY), smem, s>>>(a, maps);
  } else {
    fused_pass<OP, T, COMP, TT, NTX, NTY, CY, VX, SRC><<<(unsigned)ctas, dim3(NTX, NTY), smem, s>>>(a);
  }
  return cudaGetLastError();
}

template <int OP, class T, bool COMP, int NTX, int NTY, int CY, int VX, int TMAX, bool TMA = false, bool SRC = false>
cudaError_t launch_variant(const Geom &g, const FusedLaunch &L, cudaStream_t s) {
  switch (L.steps) {
    case 1: return launch_tt<OP, T, COMP, 1, NTX, NTY, CY, VX, TMA, SRC>(g, L, s);
    case 2: if constexpr (TMAX >= 2) return launch_tt<OP, T, COMP, 2, NTX, NTY, CY, VX, TMA, SRC>(g, L, s); break;
    case 3: if constexpr (TMAX >= 3) return launch_tt<OP, T, COMP, 3, NTX, NTY, CY, VX, TMA, SRC>(g, L, s); break;
    case 4: if constexpr (TMAX >= 4) return launch_tt<OP, T, COMP, 4, NTX, NTY, CY, VX, TMA, SRC>(g, L, s); break;
  }
  return cudaErrorInvalidValue;
}

// Maximum fusion depth instantiated per operator radius and element type.
template <int OP, class T> constexpr int fused_tmax() {
  if constexpr (std::is_same<T, Df64>::value) return OpTraits<OP>::R == 4 ? 2 : 3;
  if constexpr (OpTraits<OP>::VAR) return OpTraits<OP>::R == 4 ? 2 : 3;
  return OpTraits<OP>::R == 4 ? 2 : (sizeof(T) == 8 ? 2 : 4);
}

template <int OP, class T, bool COMP>
cudaError_t launch_fused_op_impl(const Geom &g, const FusedConfig &cfg, const FusedLaunch &L,
                                 cudaStream_t s) {
  constexpr int TM = fused_tmax<OP, T>();
  // TMA variants (2, 3) are built for FP32 storage, where the rings fit shared
  // memory, and for the constant-coefficient operators
  constexpr bool kTma = std::is_same<T, float>::value && !OpTraits<OP>::VAR;
  // with a source point every pass runs the source-enabled build of the first
  // tile variant (the update is compiled out of the others); the kernel
  // derives its tiling from its own shape
  if (L.src != nullptr) {
    if constexpr (std::is_same<T, Df64>::value || OpTraits<OP>::R != 1)
      return launch_variant<OP, T, COMP, 64, 16, 2, 1, TM, false, true>(g, L, s);
    else
      return launch_variant<OP, T, COMP, 32, 16, 2, 2, TM, false, true>(g, L, s);
  }
  if constexpr (std::is_same<T, Df64>::value) {  // one column per thread: pairs already fill 8 bytes
    switch (cfg.variant) {
      case 0: return launch_variant<OP, T, COMP, 64, 16, 2, 1, TM>(g, L, s);  // 64 x 32 region, 1024 threads
      case 1: return launch_variant<OP, T, COMP, 32, 16, 2, 1, TM>(g, L, s);  // 32 x 32 region, 512 threads
      case 2:  // 64 x 16 region, 1024 threads (radius 1)
        if constexpr (OpTraits<OP>::R == 1) return launch_variant<OP, T, COMP, 64, 16, 1, 1, TM>(g, L, s);
        break;
      case 3:  // x pairs: 64 x 32 region, 512 threads (radius 1)
        if constexpr (OpTraits<OP>::R == 1) return launch_variant<OP, T, COMP, 32, 16, 2, 2, TM>(g, L, s);
        break;
      case 4:  // x pairs: 32 x 64 region, 1024 threads (radius 1)
        if constexpr (OpTraits<OP>::R == 1) return launch_variant<OP, T, COMP, 16, 64, 1, 2, TM>(g, L, s);
        break;
      case 5:  // TMA-staged 32 x 32 and 32 x 64 regions (fused_df_tma.cu; operator 0: fused_df_tma4.cu)
      case 6:
        if constexpr (OP == 1 || OP == 8) return launch_fused_df_tma<OP>(g, cfg, L, s);
        if constexpr (OP == 0) return launch_fused_df_tma4(g, cfg, L, s);
        break;
    }
  } else if constexpr (OpTraits<OP>::R == 1) {  // x pairs: vector loads, stores and shared-memory traffic
    switch (cfg.variant) {
      case 0: return launch_variant<OP, T, COMP, 32, 16, 2, 2, TM>(g, L, s);  // 64 x 32 region, 512 threads
      case 1: return launch_variant<OP, T, COMP, 16, 64, 1, 2, TM>(g, L, s);  // 32 x 64 region, 1024 threads
      case 2:  // 64 x 32 region, 512 threads: x quads at depth 4, x pairs below (same tile: 4-column alignment)
        if constexpr (kTma) {
          if (L.steps == 4) return launch_tt<OP, T, COMP, 4, 16, 32, 1, 4, true>(g, L, s);
          return launch_variant<OP, T, COMP, 32, 16, 2, 2, 3, true>(g, L, s);
        }
        break;
      case 3:  // depth <= 2: 64 x 64 region with x quads, 1024 threads; deeper: 32 x 64 with x pairs
        if constexpr (kTma) {
          if (cfg.depth <= 2) return launch_variant<OP, T, COMP, 16, 64, 1, 4, 2, true>(g, L, s);
          return launch_variant<OP, T, COMP, 16, 64, 1, 2, TM, true>(g, L, s);
        }
        break;
    }
  } else {  // radius 4: 10-plane queues leave no registers for wider groups beyond depth 1
    switch (cfg.variant) {
      case 0: return launch_variant<OP, T, COMP, 64, 16, 2, 1, TM>(g, L, s);  // 64 x 32 region, 1024 threads
      case 1: return launch_variant<OP, T, COMP, 32, 32, 2, 1, TM>(g, L, s);  // 32 x 64 region, 1024 threads
      case 2:  // 64 x 32 region: x quads at depth 1 (the x neighbours are the adjacent quads), columns above
        if constexpr (kTma) {
          if (L.steps == 1) return launch_tt<OP, T, COMP, 1, 16, 32, 1, 4, true>(g, L, s);
          return launch_variant<OP, T, COMP, 64, 16, 2, 1, TM, true>(g, L, s);
        }
        break;
      case 3: if constexpr (kTma) return launch_variant<OP, T, COMP, 32, 32, 2, 1, TM, true>(g, L, s); break;
      case 5:  // one-step TMA pass of operator 0, 32 x 32 tile (fused_df_tma4.cu)
        if constexpr (OP == 0 && std::is_same<T, float>::value) return launch_fused_f32_tma4<COMP>(g, cfg, L, s);
        break;
    }
  }
  return cudaErrorInvalidValue;
}

}  // namespace girih
