// TMA-staged one-step passes of the 25-point leapfrog (operator 0, radius 4;
// src/kernels/stencils.c:27-41): double-float values, or FP32 storage with FP32
// or compensated (mixed) arithmetic, every input plane staged into shared
// memory by TMA.
//
// At radius 4 the overlapped time-fused tiles recompute more halo than they
// save, so these forms run one time step per pass.  The general kernel
// (fused_impl.cuh) then spends most of its issue slots around the arithmetic:
// the region's threads include the halo, and each of the 25 neighbours goes
// through the general addressing.  This kernel:
//   * covers the output tile only (32 x 32: one column and two adjacent rows
//     per thread, 512 threads); the input state's TMA boxes are the tile plus
//     the radius-4 halo (40 x 40 per plane);
//   * keeps the 2R + 1 planes an update reads, and the one in flight, in a
//     10-slot ring of the input state, so that every neighbour, z included, is
//     one shared-memory load; the old state and roc2 of the updated plane,
//     read at the point only, come with the same copy as tile-sized boxes
//     (2-slot rings);
//   * carries the ring bookkeeping (slot, barrier parity, the window of z
//     slots) from step to step: recomputing it with divisions by the 10-slot
//     ring cost ~20 instructions per update;
//   * computes exactly the general kernel's update, in the same order
//     (double-float: star_grouped_sum<4>, twice_minus(v, u) + roc2 lap,
//     df_norm; FP32: apply_op<0>; mixed: leapfrog_compensated of
//     star_const_sum<4>), so results are bit-identical;
//   * runs persistent CTAs over the (tile, plane range) pieces of
//     for_each_piece, each piece paying the ring fill (2R planes) once
//     (double-float: one CTA per SM, 161 KB of shared memory; FP32: two, 80 KB
//     each).
// At step s of a piece the copy of plane s + 1 is issued and plane s - R is
// updated; a CTA barrier per step protects the slots the next copy overwrites.
#include "fused_impl.cuh"

namespace girih {

template <class T, int NTX, int NTY> struct Tma4Shape {
  static constexpr int R = 4;
  static constexpr int BX = NTX, BY = 2 * NTY;                // output tile
  static constexpr int BW = BX + 2 * R, BH = BY + 2 * R;      // TMA box
  static constexpr int PLANE = BW * BH;                       // elements of one input-ring slot
  static constexpr int PLANE2 = BX * BY;                      // of one old-state / roc2 slot
  static constexpr int NB = tma4_nb(), NP = 2;                // input ring; old-state and roc2 rings
  static constexpr size_t ES = sizeof(T);                     // Df64: an FP32 pair
  static constexpr size_t off_prev = (size_t)NB * PLANE * ES;
  static constexpr size_t off_roc2 = off_prev + (size_t)NP * PLANE2 * ES;
  static constexpr size_t off_bar = off_roc2 + (size_t)NP * PLANE2 * ES;
  static constexpr size_t smem_bytes = off_bar + NB * sizeof(uint64_t);
  static_assert(NB == 2 * R + 2, "the ring holds planes p - R .. p + R and the one in flight");
  static_assert(BX == tma4_tile() && BY == tma4_tile() && BW == tma4_box() && BH == tma4_box(),
                "host and device tiles differ");
  static_assert(smem_bytes == tma4_smem((int)ES), "host and device shared-memory layouts differ");
  static_assert(off_prev % 128 == 0 && (PLANE * ES) % 128 == 0 && (PLANE2 * ES) % 128 == 0,
                "TMA destinations on 128 bytes");
};

// One ring element (checked build: inside the CTA's shared memory).
template <class T>
__device__ __forceinline__ T tma4_ld(const T *p, const unsigned char *smraw, int64_t smb, unsigned *flag) {
  if (!in_shared(p, sizeof(T), smraw, smb, flag)) return T(0.f);
  if constexpr (std::is_same<T, Df64>::value) {
    const float2 v = *reinterpret_cast<const float2 *>(p);
    return Df64(v.x, v.y);
  } else {
    return *p;
  }
}

// Neighbour accessor of the operator bodies (ops.cuh) over the rings: x and y
// in the box of plane p, z in the slots of planes p - R .. p + R.
template <class T, int R, int BW> struct Tma4Acc {
  const T *cp;                 // the point in the slot of plane p
  const T *zp;                 // the point's offset from the ring base (slot 0)
  const int (&zs)[2 * R + 1];  // slot offsets of planes p - R .. p + R
  const unsigned char *smraw;
  int64_t smb;
  unsigned *flag;
  __device__ __forceinline__ T c() const { return tma4_ld(cp, smraw, smb, flag); }
  __device__ __forceinline__ T x(int d) const { return tma4_ld(cp + d, smraw, smb, flag); }
  __device__ __forceinline__ T y(int d) const { return tma4_ld(cp + d * BW, smraw, smb, flag); }
  __device__ __forceinline__ T z(int d) const { return tma4_ld(zp + zs[R + d], smraw, smb, flag); }
};

// One piece: output tile (bxi, byi), planes [Z0, Z1) (array coordinates).
// `first`: the CTA's first piece (its mbarriers are initialised, not
// re-initialised).  Returns with every copy it issued consumed and a barrier
// passed; the return value is 1 if a copy did not arrive within the wait bound.
template <class T, bool COMP, int NTX, int NTY>
__device__ __forceinline__ unsigned tma4_piece(const FusedArgs<T> &a, const TmaMaps &maps, int bxi, int byi,
                                               int Z0, int Z1, bool first, unsigned char *smraw) {
  using S = Tma4Shape<T, NTX, NTY>;
  constexpr int R = S::R, NB = S::NB, BW = S::BW, PLANE = S::PLANE, PLANE2 = S::PLANE2;
  constexpr int64_t SMB = (int64_t)S::smem_bytes;
  unsigned *const flag = a.range_flag;
  const Geom &g = a.g;
  const int plane = (int)g.plane;  // 32-bit offsets: fused_supported() bounds the grid
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * NTX + tx;
  const int X0 = bxi * S::BX, Y0 = byi * S::BY;
  const int sb = Z0 - R, se = Z1 - 1 + R;  // plane s arrives at step s; plane s - R is updated there

  // bit c: row c of this thread is an interior point of the tile
  const int xi = X0 + tx;
  unsigned act = 0;
  int col[2];
#pragma unroll
  for (int c = 0; c < 2; c++) {
    const int yj = Y0 + 2 * ty + c;
    col[c] = (yj + R) * g.px + g.ox + xi + R;
    if (xi < g.nx && yj < g.ny) act |= 1u << c;
  }
  T cc[5];
#pragma unroll
  for (int m = 0; m < 5; m++) cc[m] = coef_arg<T>(a, m);

  T *const ring_cur = reinterpret_cast<T *>(smraw);
  T *const ring_prev = reinterpret_cast<T *>(smraw + S::off_prev);
  T *const ring_roc2 = reinterpret_cast<T *>(smraw + S::off_roc2);
  uint64_t *const bars = reinterpret_cast<uint64_t *>(smraw + S::off_bar);
  const int toff = (2 * ty + R) * BW + tx + R;  // this thread's row-0 point inside an input box
  const int toff2 = 2 * ty * S::BX + tx;         // and inside an old-state / roc2 box
  auto lds = [&](const T *p) -> T { return tma4_ld(p, smraw, SMB, flag); };

  // box origins: interior points (X0 - R, Y0 - R) of the input box and (X0, Y0)
  // of the others in array coordinates; their x sit on 16 bytes (the host
  // admits this shape only when g.ox and g.ox + R do)
  const int xg = X0 + g.ox, yg = Y0, xg2 = xg + R, yg2 = Y0 + R;
  constexpr unsigned kBytes = (unsigned)((PLANE + 2 * PLANE2) * S::ES);
  unsigned timeout = 0;
  if (tid == 0) {  // every phase restarts at 0; a barrier of an earlier piece is invalidated first
    for (int k = 0; k < NB; k++) {
      if (!first) mbar_inval(&bars[k]);
      mbar_init(&bars[k], 1);
    }
    mbar_init_fence();
  }
  __syncthreads();
  if (tid == 0) {  // plane sb, with the old state and roc2 of plane sb - R
    mbar_arrive_expect_tx(&bars[0], kBytes);
    tma_load_3d(ring_cur, &maps.cur, xg, yg, sb, &bars[0]);
    tma_load_3d(ring_prev, &maps.prev, xg2, yg2, sb - R, &bars[0]);
    tma_load_3d(ring_roc2, &maps.roc2, xg2, yg2, sb - R, &bars[0]);
  }

  // ring bookkeeping carried from step to step (uniform values): kb = slot of
  // plane s, ph = the parity its barrier completes with, kpo = offset (0 or
  // PLANE2) of the old-state / roc2 slot of plane s - R, zs[d] = offset of the
  // slot of plane s - 2R + d (valid once 2R + 1 planes have arrived)
  int kb = 0, kpo = 0;
  unsigned ph = 0;
  int zs[2 * R + 1];
#pragma unroll
  for (int d = 0; d <= 2 * R; d++) zs[d] = 0;
  for (int s = sb; s <= se; s++) {
#pragma unroll
    for (int d = 0; d < 2 * R; d++) zs[d] = zs[d + 1];
    zs[2 * R] = kb * PLANE;
    const int kb1 = kb + 1 == NB ? 0 : kb + 1;
    // next plane in flight (its slots were last read at step s - 1, before that
    // step's barrier), then wait for this one
    if (tid == 0 && s + 1 <= se) {
      fence_proxy_async_smem();  // earlier generic reads of the slots before the async writes
      mbar_arrive_expect_tx(&bars[kb1], kBytes);
      tma_load_3d(ring_cur + kb1 * PLANE, &maps.cur, xg, yg, s + 1, &bars[kb1]);
      tma_load_3d(ring_prev + (PLANE2 - kpo), &maps.prev, xg2, yg2, s + 1 - R, &bars[kb1]);
      tma_load_3d(ring_roc2 + (PLANE2 - kpo), &maps.roc2, xg2, yg2, s + 1 - R, &bars[kb1]);
    }
    if (!mbar_wait(&bars[kb], ph, 1u << 26)) timeout = 1;

    const int p = s - R;
    if (p >= Z0) {  // 2R + 1 planes have arrived: planes p - R .. p + R are in zs[0 .. 2R]
      const T *const base = ring_cur + toff;
#pragma unroll
      for (int c = 0; c < 2; c++) {
        if (!(act >> c & 1u)) continue;
        const T *const cp = base + zs[R] + c * BW;
        const T centre = lds(cp);
        const T uold = lds(ring_prev + kpo + toff2 + c * S::BX);
        const T r2 = lds(ring_roc2 + kpo + toff2 + c * S::BX);
        T val;
        if constexpr (std::is_same<T, Df64>::value) {
          // star_grouped_sum<4>: c0 v + sum_d c_d ((x pair + y pair) + z pair)
          Df64 lap = cc[0] * centre;
#pragma unroll
          for (int d = 1; d <= R; d++) {
            const Df64 xp = lds(cp + d) + lds(cp - d);
            const Df64 yp = lds(cp + d * BW) + lds(cp - d * BW);
            const Df64 zq = lds(base + zs[R + d] + c * BW) + lds(base + zs[R - d] + c * BW);
            lap = lap + cc[d] * ((xp + yp) + zq);
          }
          val = df_norm(twice_minus(centre, uold) + r2 * lap);
        } else {
          const Tma4Acc<T, R, BW> V{cp, base + c * BW, zs, smraw, SMB, flag};
          if constexpr (COMP) {
            val = leapfrog_compensated(centre, uold, r2, star_const_sum<R, FastArith>(cc, V));
          } else {
            CoefFull<T> none{nullptr, 0};
            val = apply_op<0, FastArith>(cc, none, 0, V, uold, r2);
          }
        }
        const int64_t o = (int64_t)p * plane + col[c];
        if (in_array(o, 1, g.elems, flag)) {
          if constexpr (std::is_same<T, Df64>::value) {
            *reinterpret_cast<float2 *>(a.out_cur + o) = make_float2(val.hi, val.lo);
          } else {
            a.out_cur[o] = val;
          }
          count_writes(a.cov_cur, o, 1);
          if (a.write_prev) {  // the pass's state t is its input
            if constexpr (std::is_same<T, Df64>::value) {
              *reinterpret_cast<float2 *>(a.out_prev + o) = make_float2(centre.hi, centre.lo);
            } else {
              a.out_prev[o] = centre;
            }
            count_writes(a.cov_prev, o, 1);
          }
        }
      }
    }
    __syncthreads();
    kb = kb1;
    ph ^= kb == 0 ? 1u : 0u;
    kpo = PLANE2 - kpo;
  }
  return timeout;
}

template <class T, bool COMP, int NTX, int NTY>
__device__ __forceinline__ void tma4_pass(const FusedArgs<T> &a, const TmaMaps &maps, unsigned char *smraw) {
  using S = Tma4Shape<T, NTX, NTY>;
  const Geom &g = a.g;
  unsigned timeout = 0;
  for_each_piece((g.nx + S::BX - 1) / S::BX, (g.ny + S::BY - 1) / S::BY, g.nz, a.zchunk,
                 [&](int bxi, int byi, int za, int zb, bool first) {
                   timeout |= tma4_piece<T, COMP, NTX, NTY>(a, maps, bxi, byi, S::R + za, S::R + zb, first, smraw);
                 });
  if (timeout && a.range_flag) atomicOr(a.range_flag, 2u);  // a copy never completed within the wait bound
}

// Double-float: one CTA per SM (161 KB of shared memory).
template <int NTX, int NTY>
__global__ void __launch_bounds__(NTX *NTY, 1) fused_df_tma4(FusedArgs<Df64> a, const __grid_constant__ TmaMaps maps) {
  extern __shared__ __align__(128) unsigned char smraw[];
  tma4_pass<Df64, false, NTX, NTY>(a, maps, smraw);
}

// FP32 storage: two CTAs per SM (80 KB each).
template <bool COMP, int NTX, int NTY>
__global__ void __launch_bounds__(NTX *NTY, 2) fused_f32_tma4(FusedArgs<float> a, const __grid_constant__ TmaMaps maps) {
  extern __shared__ __align__(128) unsigned char smraw[];
  tma4_pass<float, COMP, NTX, NTY>(a, maps, smraw);
}

template <class T, int NTX, int NTY>
static cudaError_t launch_tma4(const void *kern, std::atomic<unsigned long long> &attr_set, const Geom &g,
                               const FusedConfig &cfg, const FusedLaunch &L, cudaStream_t s) {
  using S = Tma4Shape<T, NTX, NTY>;
  if (L.src != nullptr || L.steps != 1 || cfg.depth != 1 || cfg.variant != 5 || g.op != 0) return cudaErrorInvalidValue;
  if (!L.tma_cur || !L.tma_prev || !L.tma_roc2) return cudaErrorInvalidValue;
  // the copies must fill exactly the ring slots this shape sizes, from 16-byte x offsets
  if (L.tma_box_w != S::BW || L.tma_box_h != S::BH || L.tma_box2_w != S::BX || L.tma_box2_h != S::BY ||
      (g.ox * (int)S::ES) % 16 || ((g.ox + S::R) * (int)S::ES) % 16)
    return cudaErrorInvalidValue;
  int occ = 1, nsm = 152;
  cudaError_t e = fused_kernel_setup(kern, S::smem_bytes, NTX * NTY, attr_set, &occ, &nsm);
  if (e != cudaSuccess) return e;
  const int gx = (g.nx + S::BX - 1) / S::BX, gy = (g.ny + S::BY - 1) / S::BY;
  const int64_t ctas = fused_persistent_ctas(g, (int64_t)gx * gy, (int64_t)nsm * occ);
  const int parts = fused_phase2_parts((int64_t)gx * gy, ctas, g.nz, 2 * S::R);
  FusedArgs<T> a = make_fused_args<T>(g, L, parts);
  TmaMaps maps;
  maps.cur = *static_cast<const CUtensorMap *>(L.tma_cur);
  maps.prev = *static_cast<const CUtensorMap *>(L.tma_prev);
  maps.roc2 = *static_cast<const CUtensorMap *>(L.tma_roc2);
  void *args[] = {&a, &maps};
  e = cudaLaunchKernel(kern, dim3((unsigned)ctas), dim3(NTX, NTY), args, S::smem_bytes, s);
  return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_fused_df_tma4(const Geom &g, const FusedConfig &cfg, const FusedLaunch &L, cudaStream_t s) {
  static std::atomic<unsigned long long> attr_set{0};
  return launch_tma4<Df64, 32, 16>((const void *)fused_df_tma4<32, 16>, attr_set, g, cfg, L, s);
}

template <bool COMP>
cudaError_t launch_fused_f32_tma4(const Geom &g, const FusedConfig &cfg, const FusedLaunch &L, cudaStream_t s) {
  static std::atomic<unsigned long long> attr_set{0};
  return launch_tma4<float, 32, 16>((const void *)fused_f32_tma4<COMP, 32, 16>, attr_set, g, cfg, L, s);
}

template cudaError_t launch_fused_f32_tma4<false>(const Geom &, const FusedConfig &, const FusedLaunch &, cudaStream_t);
template cudaError_t launch_fused_f32_tma4<true>(const Geom &, const FusedConfig &, const FusedLaunch &, cudaStream_t);

}  // namespace girih
