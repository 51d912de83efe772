// Double-float time-fused pass for the radius-1 constant-coefficient operators
// 1 (7-point Jacobi-type sweep) and 8 (7-point leapfrog), with every input
// plane staged into shared memory by TMA.
//
// The double-float form is bound by instruction issue, not by HBM: its update
// is ~81 FP32 operations (df64.cuh), and in the general fused kernel
// (fused_impl.cuh) the addressing, activity tests and global loads around it
// added ~60 more instructions per update.  This kernel keeps the same
// arithmetic, in the same order (results are bit-identical to the general
// kernel's double-float passes), and strips the rest:
//   * all input planes (state t, state t-1, roc2) arrive by TMA into rings
//     whose slots, like the z-queue slots and the double-buffer parity, are
//     compile-time constants of the unrolled z loop: every shared-memory access
//     is a fixed offset from one per-thread base;
//   * level 1 reads its x/y neighbours straight from the input ring (state t
//     needs no copy into a published plane);
//   * a thread owns one column and two ADJACENT rows, so one y neighbour of
//     each row is the other row's register;
//   * x/y activity and output ownership are bit masks computed once per tile;
//   * the CTAs are persistent (for_each_piece): whole tiles in rounds, all
//     CTAs at the same planes so that neighbouring tiles share their halo
//     boxes in L2, then the remaining tiles split into plane ranges, each piece
//     paying the z pipeline's fill once.
// Measured at 512^3 (7-point leapfrog): 132 instead of 152 thread instructions
// per update, 164 -> 220 GLUP/s.
//
// CTA: NTX x NTY threads over a region of NTX columns x 2*NTY rows; the output
// tile is the region less a halo of TT columns/rows per side (the region start
// is kept on a 16-byte boundary for the TMA boxes).  Level l (1..TT) of z step s
// updates plane s - l*D, D = 2, exactly as the general kernel does.
#include "fused_impl.cuh"

namespace girih {

__host__ __device__ constexpr int df_gcd(int a, int b) { return b == 0 ? a : df_gcd(b, a % b); }
__host__ __device__ constexpr int df_lcm(int a, int b) { return a / df_gcd(a, b) * b; }

template <int OP, int TT, int NTX, int NTY> struct DfTmaShape {
  static constexpr int R = 1, D = 2, TO = OpTraits<OP>::TO;
  static constexpr int QL = TO == 2 ? 4 : 3;  // z-queue length (planes p-1 .. p+2, and p+... for uold)
  static constexpr int NB = df_tma_nb(TO);    // input-state ring
  static constexpr int NP = 2;                // old-state ring (time order 2)
  static constexpr int NR = df_tma_nr(TT);    // roc2 ring (time order 2)
  // z-loop unroll: every queue slot, ring slot and buffer parity is a constant
  static constexpr int U = df_lcm(df_lcm(QL, 2), df_lcm(NB, TO == 2 ? df_lcm(NP, NR) : 1));
  static constexpr int RW = NTX, RY = 2 * NTY, H = TT;
  static constexpr int PLANE = RW * RY;  // elements of one ring slot / published plane
  // output tile: the aligned width when every tile start is then even, else the
  // general width (fused_tile_width(NTX, TT, 2) on the host)
  static constexpr int MIS = H & 1;
  static constexpr int BXA = (RW - 2 * H - MIS) / 2 * 2, BXU = RW - 2 * H - 1;
  static constexpr int BX = BXA >= BXU ? BXA : BXU, BY = RY - 2 * H;
  static constexpr size_t field_bytes = (size_t)2 * (TT - 1) * PLANE * sizeof(Df64);
  static constexpr size_t off_cur = (field_bytes + 127) / 128 * 128;
  static constexpr size_t off_prev = off_cur + (size_t)NB * PLANE * sizeof(Df64);
  static constexpr size_t off_roc2 = off_prev + (TO == 2 ? (size_t)NP * PLANE * sizeof(Df64) : 0);
  static constexpr size_t off_bar = off_roc2 + (TO == 2 ? (size_t)NR * PLANE * sizeof(Df64) : 0);
  static constexpr size_t smem_bytes = off_bar + NB * sizeof(uint64_t);
  static_assert(smem_bytes == df_tma_smem(TO, TT, RW, RY), "host and device shared-memory layouts differ");
  static_assert(TT >= 1 && TT <= 2, "depth 1 or 2");
  static_assert(BX > 0 && BY > 0, "tile too small for the fusion depth");
  static_assert(U % NB == 0 && U % QL == 0 && U % 2 == 0, "unroll must cover every period");
};

__host__ __device__ constexpr int df_pmod(int a, int m) { return ((a % m) + m) % m; }

// One piece of work: output tile (bxi, byi), planes [Z0, Z1).  `first`: the
// CTA's first piece (its mbarriers are initialised, not re-initialised).
// Returns with every copy it issued consumed and a barrier passed.
template <int OP, int TT, int NTX, int NTY>
__device__ __forceinline__ unsigned df_tma_piece(const FusedArgs<Df64> &a, const TmaMaps &maps, int bxi, int byi,
                                                 int Z0, int Z1, bool first, unsigned char *smraw) {
  using S = DfTmaShape<OP, TT, NTX, NTY>;
  constexpr int R = S::R, D = S::D, TO = S::TO, QL = S::QL, U = S::U, NB = S::NB, NP = S::NP, NR = S::NR;
  constexpr int RW = S::RW, H = S::H, BX = S::BX, BY = S::BY, PLANE = S::PLANE;
  unsigned *const flag = a.range_flag;
  constexpr int64_t SMB = (int64_t)S::smem_bytes;

  const Geom &g = a.g;
  const int plane = (int)g.plane;  // 32-bit offsets: fused_supported() bounds the grid
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * NTX + tx;
  const int X0 = bxi * BX, Y0 = byi * BY;
  const int sb = max(0, Z0 - H);
  const int se = Z1 - 1 + TT * D;
  const int s0 = sb - sb % U;  // every plane index below is taken relative to a multiple of U

  // region origin (interior coordinates), its x on a 16-byte boundary
  const int xs = X0 - H - df_pmod(X0 - H + R + g.ox, 2);
  const int xi = xs + tx;
  const bool x_int = xi >= 0 && xi < g.nx;

  // act bit (l-1)*2 + c: row c of this thread is updated at level l; out bit c:
  // row c is in the output tile
  unsigned act = 0, outb = 0;
  int col[2];
#pragma unroll
  for (int c = 0; c < 2; c++) {
    const int yj = Y0 - H + 2 * ty + c;
    const bool y_int = yj >= 0 && yj < g.ny;
    col[c] = (yj + R) * g.px + g.ox + xi + R;
#pragma unroll
    for (int l = 1; l <= TT; l++) {
      const int m = TT - l;
      if (x_int && y_int && xi >= X0 - m && xi < X0 + BX + m && yj >= Y0 - m && yj < Y0 + BY + m)
        act |= 1u << ((l - 1) * 2 + c);
    }
    if (x_int && y_int && xi >= X0 && xi < X0 + BX && yj >= Y0 && yj < Y0 + BY) outb |= 1u << c;
  }

  const Df64 c0 = Df64(a.cch[0], a.ccl[0]), c1 = Df64(a.cch[1], a.ccl[1]);

  // shared memory: published planes [2 buffers][levels 1..TT-1][RY][RW], then
  // the rings and one mbarrier per input slot
  Df64 *const field = reinterpret_cast<Df64 *>(smraw);
  Df64 *const ring_cur = reinterpret_cast<Df64 *>(smraw + S::off_cur);
  Df64 *const ring_prev = reinterpret_cast<Df64 *>(smraw + S::off_prev);
  Df64 *const ring_roc2 = reinterpret_cast<Df64 *>(smraw + S::off_roc2);
  uint64_t *const bars = reinterpret_cast<uint64_t *>(smraw + S::off_bar);
  const int toff = 2 * ty * RW + tx;  // this thread's row-0 element inside a plane
  auto lds = [&](const Df64 *p) -> Df64 {
    if (in_shared(p, sizeof(Df64), smraw, SMB, flag)) {
      const float2 v = *reinterpret_cast<const float2 *>(p);
      return Df64(v.x, v.y);
    }
    return Df64(0.f, 0.f);
  };

  Df64 q[TT][2][QL];  // z queues of levels 0..TT-1: plane p in slot p mod QL
#pragma unroll
  for (int l = 0; l < TT; l++)
#pragma unroll
    for (int c = 0; c < 2; c++)
#pragma unroll
      for (int e = 0; e < QL; e++) q[l][c][e] = Df64(0.f, 0.f);

  // TMA: thread 0 streams the region's planes one z step ahead
  const int xg = xs + R + g.ox, yg = Y0 - H + R;  // box origin in array coordinates
  constexpr unsigned kBytes = (unsigned)(PLANE * sizeof(Df64)) * (TO == 2 ? 3u : 1u);
  unsigned timeout = 0;
  if (tid == 0) {  // every phase restarts at 0; a barrier of an earlier piece is invalidated first
    for (int k = 0; k < NB; k++) {
      if (!first) mbar_inval(&bars[k]);
      mbar_init(&bars[k], 1);
    }
    mbar_init_fence();
  }
  __syncthreads();
  if (tid == 0) {  // plane s0 into slot 0 of every ring
    mbar_arrive_expect_tx(&bars[0], kBytes);
    tma_load_3d(ring_cur, &maps.cur, xg, yg, s0, &bars[0]);
    if constexpr (TO == 2) {
      tma_load_3d(ring_prev, &maps.prev, xg, yg, s0 - D, &bars[0]);
      tma_load_3d(ring_roc2, &maps.roc2, xg, yg, s0 - D, &bars[0]);
    }
  }

  for (int sbase = s0, it = 0; sbase <= se; sbase += U, it++) {
    static_for<U>([&](auto ph_c) {
      constexpr int PH = decltype(ph_c)::value;
      const int s = sbase + PH;
      if (s > se) return;  // uniform over the CTA
      constexpr int RB = (PH + 1) & 1, WB = PH & 1;  // published planes: read (step s-1) / write (step s)
      constexpr int KB = PH % NB;

      // next plane in flight, then wait for this one
      if (tid == 0 && s + 1 <= se) {
        constexpr int KB1 = (PH + 1) % NB, KP1 = (PH + 1) % NP, KR1 = (PH + 1) % NR;
        fence_proxy_async_smem();  // earlier generic reads of the slots before the async writes
        mbar_arrive_expect_tx(&bars[KB1], kBytes);
        tma_load_3d(ring_cur + KB1 * PLANE, &maps.cur, xg, yg, s + 1, &bars[KB1]);
        if constexpr (TO == 2) {
          tma_load_3d(ring_prev + KP1 * PLANE, &maps.prev, xg, yg, s + 1 - D, &bars[KB1]);
          tma_load_3d(ring_roc2 + KR1 * PLANE, &maps.roc2, xg, yg, s + 1 - D, &bars[KB1]);
        }
      }
      if (!mbar_wait(&bars[KB], (unsigned)(it * (U / NB) + PH / NB) & 1u, 1u << 26)) timeout = 1;

      // levels TT..1, highest first: level l reads level l-1's queues before
      // level l-1 stores this step's plane
      static_for<TT>([&](auto li_c) {
        constexpr int L = TT - decltype(li_c)::value;
        constexpr int SP = qslot<QL>(PH - L * D), SU = qslot<QL>(PH - L * D + 1), SD = qslot<QL>(PH - L * D - 1);
        const int p = s - L * D;
        const bool p_int = p >= R && p < g.nnz - R;
        const bool p_out = p_int && p >= Z0 && p < Z1;
        // level L-1 at plane p: the input ring (L = 1) or the plane published at step s-1
        const Df64 *src;
        if constexpr (L == 1) src = ring_cur + df_pmod(PH - D, NB) * PLANE + toff;
        else src = field + (RB * (TT - 1) + (L - 2)) * PLANE + toff;
#pragma unroll
        for (int c = 0; c < 2; c++) {
          const Df64 centre = q[L - 1][c][SP];
          Df64 val = centre;  // halo, out-of-region and inactive points keep their value
          if (p_int && (act >> ((L - 1) * 2 + c) & 1u)) {
            const Df64 *sr = src + c * RW;
            const Df64 xl = lds(sr - 1), xr = lds(sr + 1);
            const Df64 yup = c == 0 ? q[L - 1][1][SP] : lds(sr + RW);
            const Df64 ydn = c == 0 ? lds(sr - RW) : q[L - 1][0][SP];
            // star_grouped_sum<1>: c0 v + c1 ((x pair + y pair) + z pair)
            const Df64 lap = c0 * centre + c1 * (((xr + xl) + (yup + ydn)) + (q[L - 1][c][SU] + q[L - 1][c][SD]));
            Df64 cand;
            if constexpr (TO == 2) {
              Df64 uold;
              if constexpr (L == 1) uold = lds(ring_prev + (PH % NP) * PLANE + toff + c * RW);
              else uold = q[L - 2][c][SP];
              // roc2 of plane p arrived with input plane s - (L-1)*D
              const Df64 r2 = lds(ring_roc2 + df_pmod(PH - (L - 1) * D, NR) * PLANE + toff + c * RW);
              cand = twice_minus(centre, uold) + r2 * lap;
            } else {
              cand = lap;
            }
            val = df_norm(cand);
          }
          if constexpr (L == TT || L == TT - 1) {
            if (p_out && (outb >> c & 1u) && (L == TT || a.write_prev) &&
                in_array((int64_t)p * plane + col[c], 1, g.elems, flag)) {
              Df64 *dst = (L == TT ? a.out_cur : a.out_prev) + p * plane + col[c];
              *reinterpret_cast<float2 *>(dst) = make_float2(val.hi, val.lo);
              count_writes(L == TT ? a.cov_cur : a.cov_prev, (int64_t)p * plane + col[c], 1);
            }
          }
          if constexpr (L < TT) q[L][c][SP] = val;
        }
      });

      // level 0: plane s from the input ring
      constexpr int S0 = qslot<QL>(PH);
#pragma unroll
      for (int c = 0; c < 2; c++) {
        q[0][c][S0] = lds(ring_cur + KB * PLANE + toff + c * RW);
        if constexpr (TT == 1) {  // the pass's state t+TT-1 is its input
          if (a.write_prev && s >= R && s < g.nnz - R && s >= Z0 && s < Z1 && (outb >> c & 1u) &&
              in_array((int64_t)s * plane + col[c], 1, g.elems, flag)) {
            *reinterpret_cast<float2 *>(a.out_prev + s * plane + col[c]) = make_float2(q[0][c][S0].hi, q[0][c][S0].lo);
            count_writes(a.cov_prev, (int64_t)s * plane + col[c], 1);
          }
        }
      }
      // publish each level l >= 1's plane s - l*D - 1 for level l+1 at step s+1
#pragma unroll
      for (int l = 1; l < TT; l++)
#pragma unroll
        for (int c = 0; c < 2; c++) {
          Df64 *dst = field + (WB * (TT - 1) + (l - 1)) * PLANE + toff + c * RW;
          const Df64 v = q[l][c][qslot<QL>(PH - l * D - 1)];
          if (in_shared(dst, sizeof(Df64), smraw, SMB, flag)) *reinterpret_cast<float2 *>(dst) = make_float2(v.hi, v.lo);
        }
      __syncthreads();
    });
  }
  return timeout;
}

// Persistent pass: the pieces of for_each_piece (whole tiles while every CTA
// can take one, then the remaining tiles' planes split evenly), each paying
// the z pipeline's fill (~TT*D + TT planes) once.
template <int OP, int TT, int NTX, int NTY>
__global__ void __launch_bounds__(NTX *NTY, NTX * NTY <= 512 ? 2 : 1)
    fused_df_tma(FusedArgs<Df64> a, const __grid_constant__ TmaMaps maps) {
  using S = DfTmaShape<OP, TT, NTX, NTY>;
  extern __shared__ __align__(128) unsigned char smraw[];
  const Geom &g = a.g;
  unsigned timeout = 0;
  for_each_piece((g.nx + S::BX - 1) / S::BX, (g.ny + S::BY - 1) / S::BY, g.nz, a.zchunk,
                 [&](int bxi, int byi, int za, int zb, bool first) {
                   timeout |= df_tma_piece<OP, TT, NTX, NTY>(a, maps, bxi, byi, S::R + za, S::R + zb, first, smraw);
                 });
  if (timeout && a.range_flag) atomicOr(a.range_flag, 2u);  // a copy never completed within the wait bound
}

template <int OP, int TT, int NTX, int NTY>
cudaError_t launch_df_tma_tt(const Geom &g, const FusedLaunch &L, cudaStream_t s) {
  using S = DfTmaShape<OP, TT, NTX, NTY>;
  const void *kern = (const void *)fused_df_tma<OP, TT, NTX, NTY>;
  static std::atomic<unsigned long long> attr_set{0};
  int occ = 1, nsm = 152;
  cudaError_t e = fused_kernel_setup(kern, S::smem_bytes, NTX * NTY, attr_set, &occ, &nsm);
  if (e != cudaSuccess) return e;
  if (!L.tma_cur || !L.tma_prev || !L.tma_roc2) return cudaErrorInvalidValue;
  // the copies must fill exactly the ring slots this shape sizes
  if (L.tma_box_w != S::RW || L.tma_box_h != S::RY) return cudaErrorInvalidValue;
  // persistent grid: one CTA per resident slot
  const int gx = (g.nx + S::BX - 1) / S::BX, gy = (g.ny + S::BY - 1) / S::BY;
  const int64_t ctas = fused_persistent_ctas(g, (int64_t)gx * gy, (int64_t)nsm * occ);
  const int parts = fused_phase2_parts((int64_t)gx * gy, ctas, g.nz, TT * S::R + TT * S::D);
  FusedArgs<Df64> a = make_fused_args<Df64>(g, L, parts);
  TmaMaps maps;
  maps.cur = *static_cast<const CUtensorMap *>(L.tma_cur);
  maps.prev = *static_cast<const CUtensorMap *>(L.tma_prev);
  maps.roc2 = *static_cast<const CUtensorMap *>(L.tma_roc2);
  fused_df_tma<OP, TT, NTX, NTY><<<(unsigned)ctas, dim3(NTX, NTY), S::smem_bytes, s>>>(a, maps);
  return cudaGetLastError();
}

template <int OP>
cudaError_t launch_fused_df_tma(const Geom &g, const FusedConfig &cfg, const FusedLaunch &L, cudaStream_t s) {
  if (L.src != nullptr || L.steps < 1 || L.steps > cfg.depth) return cudaErrorInvalidValue;
  if (cfg.variant == 5) {  // 32 x 32 region, 512 threads
    if (L.steps == 1) return launch_df_tma_tt<OP, 1, 32, 16>(g, L, s);
    if (L.steps == 2) return launch_df_tma_tt<OP, 2, 32, 16>(g, L, s);
  } else if (cfg.variant == 6) {  // 64 x 32 region, 1024 threads
    if (L.steps == 1) return launch_df_tma_tt<OP, 1, 64, 16>(g, L, s);
    if (L.steps == 2) return launch_df_tma_tt<OP, 2, 64, 16>(g, L, s);
  }
  return cudaErrorInvalidValue;
}

template cudaError_t launch_fused_df_tma<1>(const Geom &, const FusedConfig &, const FusedLaunch &, cudaStream_t);
template cudaError_t launch_fused_df_tma<8>(const Geom &, const FusedConfig &, const FusedLaunch &, cudaStream_t);

}  // namespace girih
