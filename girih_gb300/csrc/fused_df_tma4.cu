// Double-float one-step pass of the 25-point leapfrog (operator 0, radius 4;
// src/kernels/stencils.c:27-41), every input plane staged into shared memory
// by TMA.
//
// At radius 4 the overlapped time-fused tiles recompute more halo than they
// save, so the double-float form of operator 0 runs one time step per pass.
// The general kernel (fused_impl.cuh) then spends most of its issue slots
// around the arithmetic: the region's threads include the halo, and each of
// the 25 neighbours goes through the general addressing.  This kernel:
//   * covers the output tile only (32 x 32: one column and two adjacent rows
//     per thread, 512 threads); the TMA boxes are the tile plus the radius-4
//     halo (40 x 40 per plane);
//   * keeps the 2R + 1 planes an update reads, and the one in flight, in a
//     10-slot ring of the input state, so that every neighbour, z included, is
//     one shared-memory load; the old state and roc2 of the updated plane come
//     with the same copy (2-slot rings);
//   * indexes the ring slots at run time: a few integer operations against the
//     ~235 FP32 operations of a double-float update, where an unrolled z loop
//     (lcm of the ring periods) would not fit the instruction cache;
//   * computes exactly the general kernel's double-float update
//     (star_grouped_sum<4>, then twice_minus(v, u) + roc2 lap, then df_norm), in
//     the same order, so results are bit-identical;
//   * runs persistent CTAs over the (tile, plane range) pieces of
//     for_each_piece, each piece paying the ring fill (2R planes) once.
// At step s of a piece the copy of plane s + 1 is issued and plane s - R is
// updated; a CTA barrier per step protects the slots the next copy overwrites.
#include "fused_impl.cuh"

namespace girih {

template <int NTX, int NTY> struct DfTma4Shape {
  static constexpr int R = 4;
  static constexpr int BX = NTX, BY = 2 * NTY;                // output tile
  static constexpr int BW = BX + 2 * R, BH = BY + 2 * R;      // TMA box
  static constexpr int PLANE = BW * BH;                       // elements of one ring slot
  static constexpr int NB = df_tma4_nb(), NP = 2;             // input ring; old-state and roc2 rings
  static constexpr size_t off_prev = (size_t)NB * PLANE * sizeof(Df64);
  static constexpr size_t off_roc2 = off_prev + (size_t)NP * PLANE * sizeof(Df64);
  static constexpr size_t off_bar = off_roc2 + (size_t)NP * PLANE * sizeof(Df64);
  static constexpr size_t smem_bytes = off_bar + NB * sizeof(uint64_t);
  static_assert(NB == 2 * R + 2, "the ring holds planes p - R .. p + R and the one in flight");
  static_assert(BX == df_tma4_tile() && BY == df_tma4_tile() && BW == df_tma4_box() && BH == df_tma4_box(),
                "host and device tiles differ");
  static_assert(smem_bytes == df_tma4_smem(), "host and device shared-memory layouts differ");
  static_assert(off_prev % 128 == 0 && (PLANE * sizeof(Df64)) % 128 == 0, "TMA destinations on 128 bytes");
};

// One piece: output tile (bxi, byi), planes [Z0, Z1) (array coordinates).
// `first`: the CTA's first piece (its mbarriers are initialised, not
// re-initialised).  Returns with every copy it issued consumed and a barrier
// passed; the return value is 1 if a copy did not arrive within the wait bound.
template <int NTX, int NTY>
__device__ __forceinline__ unsigned df_tma4_piece(const FusedArgs<Df64> &a, const TmaMaps &maps, int bxi, int byi,
                                                  int Z0, int Z1, bool first, unsigned char *smraw) {
  using S = DfTma4Shape<NTX, NTY>;
  constexpr int R = S::R, NB = S::NB, NP = S::NP, BW = S::BW, PLANE = S::PLANE;
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
  Df64 cc[R + 1];
#pragma unroll
  for (int m = 0; m <= R; m++) cc[m] = coef_arg<Df64>(a, m);

  Df64 *const ring_cur = reinterpret_cast<Df64 *>(smraw);
  Df64 *const ring_prev = reinterpret_cast<Df64 *>(smraw + S::off_prev);
  Df64 *const ring_roc2 = reinterpret_cast<Df64 *>(smraw + S::off_roc2);
  uint64_t *const bars = reinterpret_cast<uint64_t *>(smraw + S::off_bar);
  const int toff = (2 * ty + R) * BW + tx + R;  // this thread's row-0 point inside a box
  auto lds = [&](const Df64 *p) -> Df64 {
    if (in_shared(p, sizeof(Df64), smraw, SMB, flag)) {
      const float2 v = *reinterpret_cast<const float2 *>(p);
      return Df64(v.x, v.y);
    }
    return Df64(0.f, 0.f);
  };

  // box origin: interior point (X0 - R, Y0 - R) in array coordinates; its x is
  // even (the host admits this shape only when g.ox is), a 16-byte boundary
  const int xg = X0 + g.ox, yg = Y0;
  constexpr unsigned kBytes = (unsigned)(PLANE * sizeof(Df64)) * 3u;
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
    tma_load_3d(ring_prev, &maps.prev, xg, yg, sb - R, &bars[0]);
    tma_load_3d(ring_roc2, &maps.roc2, xg, yg, sb - R, &bars[0]);
  }

  // ring bookkeeping carried from step to step (uniform values; recomputing
  // them with divisions by the 10-slot ring cost ~30 instructions per update):
  // kb = slot of plane s, ph = the parity its barrier completes with, kpo =
  // offset of the old-state / roc2 slot of plane s - R, zs[d] = offset of the
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
      tma_load_3d(ring_prev + (PLANE - kpo), &maps.prev, xg, yg, s + 1 - R, &bars[kb1]);
      tma_load_3d(ring_roc2 + (PLANE - kpo), &maps.roc2, xg, yg, s + 1 - R, &bars[kb1]);
    }
    if (!mbar_wait(&bars[kb], ph, 1u << 26)) timeout = 1;

    const int p = s - R;
    if (p >= Z0) {  // 2R + 1 planes have arrived: planes p - R .. p + R are in zs[0 .. 2R]
      const Df64 *const base = ring_cur + toff;
#pragma unroll
      for (int c = 0; c < 2; c++) {
        if (!(act >> c & 1u)) continue;
        const Df64 *const cp = base + zs[R] + c * BW;
        const Df64 centre = lds(cp);
        // star_grouped_sum<4>: c0 v + sum_d c_d ((x pair + y pair) + z pair)
        Df64 lap = cc[0] * centre;
#pragma unroll
        for (int d = 1; d <= R; d++) {
          const Df64 xp = lds(cp + d) + lds(cp - d);
          const Df64 yp = lds(cp + d * BW) + lds(cp - d * BW);
          const Df64 zp = lds(base + zs[R + d] + c * BW) + lds(base + zs[R - d] + c * BW);
          lap = lap + cc[d] * ((xp + yp) + zp);
        }
        const Df64 uold = lds(ring_prev + kpo + toff + c * BW);
        const Df64 r2 = lds(ring_roc2 + kpo + toff + c * BW);
        const Df64 val = df_norm(twice_minus(centre, uold) + r2 * lap);
        const int64_t o = (int64_t)p * plane + col[c];
        if (in_array(o, 1, g.elems, flag)) {
          *reinterpret_cast<float2 *>(a.out_cur + o) = make_float2(val.hi, val.lo);
          count_writes(a.cov_cur, o, 1);
          if (a.write_prev) {  // the pass's state t is its input
            *reinterpret_cast<float2 *>(a.out_prev + o) = make_float2(centre.hi, centre.lo);
            count_writes(a.cov_prev, o, 1);
          }
        }
      }
    }
    __syncthreads();
    kb = kb1;
    ph ^= kb == 0 ? 1u : 0u;
    kpo = PLANE - kpo;
  }
  return timeout;
}

template <int NTX, int NTY>
__global__ void __launch_bounds__(NTX *NTY, 1) fused_df_tma4(FusedArgs<Df64> a, const __grid_constant__ TmaMaps maps) {
  using S = DfTma4Shape<NTX, NTY>;
  extern __shared__ __align__(128) unsigned char smraw[];
  const Geom &g = a.g;
  unsigned timeout = 0;
  for_each_piece((g.nx + S::BX - 1) / S::BX, (g.ny + S::BY - 1) / S::BY, g.nz, a.zchunk,
                 [&](int bxi, int byi, int za, int zb, bool first) {
                   timeout |= df_tma4_piece<NTX, NTY>(a, maps, bxi, byi, S::R + za, S::R + zb, first, smraw);
                 });
  if (timeout && a.range_flag) atomicOr(a.range_flag, 2u);  // a copy never completed within the wait bound
}

cudaError_t launch_fused_df_tma4(const Geom &g, const FusedConfig &cfg, const FusedLaunch &L, cudaStream_t s) {
  constexpr int NTX = 32, NTY = 16;
  using S = DfTma4Shape<NTX, NTY>;
  if (L.src != nullptr || L.steps != 1 || cfg.depth != 1 || g.op != 0) return cudaErrorInvalidValue;
  if (!L.tma_cur || !L.tma_prev || !L.tma_roc2) return cudaErrorInvalidValue;
  // the copies must fill exactly the ring slots this shape sizes, from an even x
  if (L.tma_box_w != S::BW || L.tma_box_h != S::BH || (g.ox & 1)) return cudaErrorInvalidValue;
  const void *kern = (const void *)fused_df_tma4<NTX, NTY>;
  static std::atomic<unsigned long long> attr_set{0};
  int occ = 1, nsm = 152;
  cudaError_t e = fused_kernel_setup(kern, S::smem_bytes, NTX * NTY, attr_set, &occ, &nsm);
  if (e != cudaSuccess) return e;
  const int gx = (g.nx + S::BX - 1) / S::BX, gy = (g.ny + S::BY - 1) / S::BY;
  const int64_t ctas = fused_persistent_ctas(g, (int64_t)gx * gy, (int64_t)nsm * occ);
  const int parts = fused_phase2_parts((int64_t)gx * gy, ctas, g.nz, 2 * S::R);
  FusedArgs<Df64> a = make_fused_args<Df64>(g, L, parts);
  TmaMaps maps;
  maps.cur = *static_cast<const CUtensorMap *>(L.tma_cur);
  maps.prev = *static_cast<const CUtensorMap *>(L.tma_prev);
  maps.roc2 = *static_cast<const CUtensorMap *>(L.tma_roc2);
  fused_df_tma4<NTX, NTY><<<(unsigned)ctas, dim3(NTX, NTY), S::smem_bytes, s>>>(a, maps);
  return cudaGetLastError();
}

}  // namespace girih
