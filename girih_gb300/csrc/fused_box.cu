// Time-fused passes of the 27-point box operator (operator 7,
// box_ref_2space_1time, src/kernels/stencils.c:227-242; serial form
// src/verification.c:786-819): TT time steps per HBM pass, in FP64, FP32 and
// double-float.
//
// The star kernels read the x/y neighbours of a level from one shared-memory
// plane; the box operator also needs the x/y neighbours of the planes above and
// below.  It is evaluated through per-plane partial sums instead: for level l-1
// and plane q let
//     F(q) = the 4 in-plane face neighbours  (x+-1, y) and (x, y+-1),
//     E(q) = the 4 in-plane diagonal neighbours (x+-1, y+-1),
// so that the 26 neighbours of (x, y, p) group as
//     faces   = F(p) + v(p-1) + v(p+1)
//     edges   = E(p) + F(p-1) + F(p+1)
//     corners = E(p-1) + E(p+1)
// and  u = c0 v + c1 faces + c2 edges + c3 corners.  Each thread computes F and
// E once per plane and column (8 shared-memory reads) and keeps the last three
// planes' values, and its column's values, in registers.  The association
// order differs from the reference's, so results agree within the rounding of
// the form (the FP64 parity bound 1e-12 for FP64 and double-float), not bit for
// bit; the plain FP64 kernel in `exact` mode keeps the reference's order.
//
// Schedule (as the star kernels): overlapped x-y tiles with a halo of TT
// columns, a z wavefront inside the CTA where level l computes plane
// p = s - 2l at z step s.  At the end of step s every level publishes its
// newest plane (level 0: plane s read from HBM; level l: plane s - 2l) into a
// double-buffered shared-memory plane, from which level l+1 takes F and E of
// plane p+1 at step s+1.  Points outside the interior keep their value.
#include "fused_impl.cuh"

namespace girih {
namespace {

template <class T, int TT, int NTX, int NTY, int CY> struct BoxShape {
  static constexpr int QL = 3;                     // planes p-1, p, p+1 in registers
  static constexpr int U = 6;                      // z-loop unroll: a multiple of QL, even (buffer parity)
  static constexpr int RW = NTX, RY = NTY * CY;    // column region
  static constexpr int PW = RW + 2, PR = RY + 2;   // shared plane padded by one column / row
  static constexpr int H = TT;                     // halo: one column per level
  static constexpr int BX = RW - 2 * H, BY = RY - 2 * H;  // output tile
  static constexpr size_t smem_bytes = (size_t)2 * TT * PR * PW * sizeof(T);
};

template <class T, int TT, int NTX, int NTY, int CY>
__global__ void __launch_bounds__(NTX *NTY) fused_box_pass(FusedArgs<typename StorageOf<T>::type> a) {
  using Sh = BoxShape<T, TT, NTX, NTY, CY>;
  using ST = typename StorageOf<T>::type;
  constexpr int QL = Sh::QL, U = Sh::U, PW = Sh::PW, PR = Sh::PR, H = Sh::H, BX = Sh::BX, BY = Sh::BY;
  static_assert(BX > 0 && BY > 0, "tile too small for the fusion depth");
  extern __shared__ __align__(128) unsigned char smraw[];
  T *sm = reinterpret_cast<T *>(smraw);  // [2 buffers][TT levels][PR rows][PW columns]
  unsigned range_bad = 0;
  unsigned *const flag = a.range_flag;                   // checked build: bounds violations
  constexpr int64_t SMB = (int64_t)Sh::smem_bytes;

  const Geom &g = a.g;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int plane = (int)g.plane;  // fused_supported(): fewer than 2^31 elements per array
  const int X0 = blockIdx.x * BX, Y0 = blockIdx.y * BY;
  const int Z0 = 1 + blockIdx.z * a.zchunk;
  const int Z1 = min(Z0 + a.zchunk, g.nnz - 1);
  const int sb = max(0, Z0 - H);
  const int se = Z1 - 1 + 2 * TT;
  const int s0 = sb - sb % U;  // plane q sits in register slot q mod 3; buffer parity = step parity

  const int xi = X0 - H + tx;  // interior x index of the thread's column
  const bool x_dom = xi + 1 >= 0 && xi + 1 < g.nnx;
  const bool x_int = xi >= 0 && xi < g.nx;
  const bool x_out = x_int && xi >= X0 && xi < X0 + BX;
  bool y_dom[CY], y_out[CY];
  int col[CY];
  unsigned act = 0;  // bit (l-1)*CY + c: the point is inside level l's valid band
#pragma unroll
  for (int c = 0; c < CY; c++) {
    const int yj = Y0 - H + ty + c * NTY;
    y_dom[c] = yj + 1 >= 0 && yj + 1 < g.nny;
    const bool y_int = yj >= 0 && yj < g.ny;
    y_out[c] = y_int && yj >= Y0 && yj < Y0 + BY;
    col[c] = (yj + 1) * g.px + g.ox + (xi + 1);
#pragma unroll
    for (int l = 1; l <= TT; l++)
      if (x_int && y_int && xi >= X0 - (TT - l) && xi < X0 + BX + (TT - l) && yj >= Y0 - (TT - l) &&
          yj < Y0 + BY + (TT - l))
        act |= 1u << ((l - 1) * CY + c);
  }
  // source point: its plane and, per row, whether it is this thread's column
  int src_z = -(1 << 30);
  bool src_here[CY];
#pragma unroll
  for (int c = 0; c < CY; c++) src_here[c] = false;
  if (a.src != nullptr) {
    src_z = a.src_off / plane;
#pragma unroll
    for (int c = 0; c < CY; c++) src_here[c] = a.src_off - src_z * plane == col[c];
  }

  T cc[4];
#pragma unroll
  for (int m = 0; m < 4; m++) cc[m] = coef_arg<T>(a, m);

  // v: each level's values of the thread's column (planes mod 3); f, e: the
  // partial sums F and E of level L-1 that level L uses (planes mod 3)
  T v[TT][CY][QL], f[TT][CY][QL], e[TT][CY][QL];
#pragma unroll
  for (int l = 0; l < TT; l++)
#pragma unroll
    for (int c = 0; c < CY; c++)
#pragma unroll
      for (int q = 0; q < QL; q++) v[l][c][q] = f[l][c][q] = e[l][c][q] = T(0);

  // shared element of this thread's column, row c, level l, buffer b:
  //   thr + ((b*TT + l)*PR + c*NTY)*PW
  T *const thr = sm + (ty + 1) * PW + tx + 1;

  for (int sbase = s0; sbase <= se; sbase += U) {
    static_for<U>([&](auto ph_c) {
      constexpr int PH = decltype(ph_c)::value;
      constexpr int RB = (PH + 1) & 1, WB = PH & 1;  // read buffer (written at s-1), write buffer
      const int s = sbase + PH;
      if (s > se) return;  // uniform over the CTA
      // levels TT..1, highest first: level L reads level L-1's registers before
      // level L-1 replaces them with this step's plane
      static_for<TT>([&](auto li_c) {
        constexpr int L = TT - decltype(li_c)::value;
        constexpr int SM = qslot<QL>(PH - 2 * L - 1), S0 = qslot<QL>(PH - 2 * L), SP = qslot<QL>(PH - 2 * L + 1);
        const int p = s - 2 * L;
        const bool p_int = p >= 1 && p < g.nnz - 1;
#pragma unroll
        for (int c = 0; c < CY; c++) {
          // F and E of level L-1 at plane p+1 (published at step s-1)
          const T *q = thr + ((RB * TT + (L - 1)) * PR + c * NTY) * PW;
          if (in_shared(q - PW - 1, (int64_t)(2 * PW + 3) * sizeof(T), smraw, SMB, flag)) {
            f[L - 1][c][SP] = (q[-1] + q[1]) + (q[-PW] + q[PW]);
            e[L - 1][c][SP] = (q[-PW - 1] + q[PW + 1]) + (q[-PW + 1] + q[PW - 1]);
          }
          const T centre = v[L - 1][c][S0];
          T val = centre;
          if (p_int && (act >> ((L - 1) * CY + c) & 1u)) {
            const T faces = f[L - 1][c][S0] + (v[L - 1][c][SM] + v[L - 1][c][SP]);
            const T edges = e[L - 1][c][S0] + (f[L - 1][c][SM] + f[L - 1][c][SP]);
            const T corners = e[L - 1][c][SM] + e[L - 1][c][SP];
            T u = cc[0] * centre + cc[1] * faces + cc[2] * edges + cc[3] * corners;
            // source point of step src_t0 + L - 1, added after the update's rounding
            if (p == src_z && src_here[c] && a.src_t0 + L - 1 < a.src_n) {
              if constexpr (std::is_same<T, Df64>::value) u = df_norm(u);
              u = u + coef_to_compute<T>(a.src[a.src_t0 + L - 1]);
            }
            if constexpr (std::is_same<T, Df64>::value) val = df_norm(u);
            else val = u;
          }
          if constexpr (L == TT || L == TT - 1) {
            if (p_int && p >= Z0 && p < Z1 && x_out && y_out[c] && (L == TT || a.write_prev) &&
                in_array(p * plane + col[c], 1, g.elems, flag)) {
              (L == TT ? a.out_cur : a.out_prev)[p * plane + col[c]] = to_storage<ST>(val);
              count_writes(L == TT ? a.cov_cur : a.cov_prev, p * plane + col[c], 1);
            }
          }
          if constexpr (L < TT) v[L][c][S0] = val;  // level L's newest plane is p
        }
      });
      // level 0: plane s from HBM
      const bool s_in = s < g.nnz;
#pragma unroll
      for (int c = 0; c < CY; c++) {
        T in = T(0);
        if (s_in && x_dom && y_dom[c] && in_array(s * plane + col[c], 1, g.elems, flag))
          in = to_compute<T>(ldg_elem(a.cur + s * plane + col[c]), range_bad);
        v[0][c][qslot<QL>(PH)] = in;
        if constexpr (TT == 1) {
          if (a.write_prev && s >= 1 && s < g.nnz - 1 && s >= Z0 && s < Z1 && x_out && y_out[c] &&
              in_array(s * plane + col[c], 1, g.elems, flag)) {
            a.out_prev[s * plane + col[c]] = to_storage<ST>(in);
            count_writes(a.cov_prev, s * plane + col[c], 1);
          }
        }
      }
      // publish every level's newest plane (level l: plane s - 2l) for step s+1
#pragma unroll
      for (int l = 0; l < TT; l++)
#pragma unroll
        for (int c = 0; c < CY; c++) {
          T *const dst = thr + ((WB * TT + l) * PR + c * NTY) * PW;
          if (in_shared(dst, sizeof(T), smraw, SMB, flag)) *dst = v[l][c][qslot<QL>(PH - 2 * l)];
        }
      __syncthreads();
    });
  }
}

template <class T, int TT, int NTX, int NTY, int CY>
cudaError_t launch_box_tt(const Geom &g, const FusedLaunch &L, cudaStream_t s) {
  using S = BoxShape<T, TT, NTX, NTY, CY>;
  using ST = typename StorageOf<T>::type;
  void *kern = (void *)fused_box_pass<T, TT, NTX, NTY, CY>;
  const size_t smem = S::smem_bytes;
  static std::atomic<unsigned long long> attr_set{0};
  int dev = 0;
  cudaGetDevice(&dev);
  const unsigned long long dev_bit = 1ull << (dev & 63);
  if (!(attr_set.load(std::memory_order_acquire) & dev_bit)) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_set.fetch_or(dev_bit, std::memory_order_release);
  }
  int occ = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, NTX * NTY, smem);
  if (occ < 1) occ = 1;
  const int gx = (g.nx + S::BX - 1) / S::BX, gy = (g.ny + S::BY - 1) / S::BY;
  int nsm = 152;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int64_t cap = (int64_t)nsm * occ, tiles = (int64_t)gx * gy;
  // z chunks: minimise waves x (chunk + pipeline fill)
  const int over = 3 * TT;
  int best_n = 1;
  double best_cost = 1e300;
  for (int n = 1; n <= 64 && n <= g.nz; n++) {
    const int chunk = (g.nz + n - 1) / n;
    const double cost = (double)((tiles * n + cap - 1) / cap) * (chunk + over);
    if (cost < best_cost * 0.999) {
      best_cost = cost;
      best_n = n;
    }
  }
  const int zchunk = (g.nz + best_n - 1) / best_n;
  FusedArgs<ST> a{};
  a.g = g;
  a.cur = static_cast<const ST *>(L.cur);
  a.out_prev = static_cast<ST *>(L.out_prev);
  a.out_cur = static_cast<ST *>(L.out_cur);
  for (int m = 0; m < 5; m++) a.cc[m] = L.cc[m];
  split_coefs(a.cc, a.cch, a.ccl);
  a.range_flag = L.range_flag;
  a.src = L.src;
  a.src_off = L.src_off;
  a.src_t0 = L.src_t0;
  a.src_n = L.src_n;
  a.cov_prev = L.cov_prev;
  a.cov_cur = L.cov_cur;
  a.zchunk = zchunk;
  a.write_prev = L.write_prev;
  fused_box_pass<T, TT, NTX, NTY, CY>
      <<<dim3(gx, gy, (g.nz + zchunk - 1) / zchunk), dim3(NTX, NTY), smem, s>>>(a);
  return cudaGetLastError();
}

template <class T, int NTX, int NTY, int CY, int TMAX>
cudaError_t launch_box_variant(const Geom &g, const FusedLaunch &L, cudaStream_t s) {
  switch (L.steps) {
    case 1: return launch_box_tt<T, 1, NTX, NTY, CY>(g, L, s);
    case 2: if constexpr (TMAX >= 2) return launch_box_tt<T, 2, NTX, NTY, CY>(g, L, s); break;
    case 3: if constexpr (TMAX >= 3) return launch_box_tt<T, 3, NTX, NTY, CY>(g, L, s); break;
    case 4: if constexpr (TMAX >= 4) return launch_box_tt<T, 4, NTX, NTY, CY>(g, L, s); break;
  }
  return cudaErrorInvalidValue;
}

// Variant 0: 32 x 32 region (32x16 threads, two rows each, 512 threads);
// variant 1: 64 x 16 region (64x16 threads, one row each, 1024 threads).
// Depth: up to 4 in FP32, 3 (variant 0) or 2 (variant 1) in double-float, 2 in
// FP64 -- the deepest passes whose three register queues per level fit the
// registers a thread has at that block size.
template <class T>
cudaError_t launch_box(const Geom &g, const FusedConfig &cfg, const FusedLaunch &L, cudaStream_t s) {
  constexpr bool F32 = std::is_same<T, float>::value, DF = std::is_same<T, Df64>::value;
  switch (cfg.variant) {
    case 0: return launch_box_variant<T, 32, 16, 2, F32 ? 4 : (DF ? 3 : 2)>(g, L, s);
    case 1: return launch_box_variant<T, 64, 16, 1, F32 ? 4 : 2>(g, L, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace

template <>
cudaError_t launch_fused_op<7, double, false>(const Geom &g, const FusedConfig &cfg, const FusedLaunch &L,
                                              cudaStream_t s) {
  return launch_box<double>(g, cfg, L, s);
}
template <>
cudaError_t launch_fused_op<7, float, false>(const Geom &g, const FusedConfig &cfg, const FusedLaunch &L,
                                             cudaStream_t s) {
  return launch_box<float>(g, cfg, L, s);
}
template <>
cudaError_t launch_fused_op<7, Df64, false>(const Geom &g, const FusedConfig &cfg, const FusedLaunch &L,
                                            cudaStream_t s) {
  return launch_box<Df64>(g, cfg, L, s);
}

}  // namespace girih
