// Fused-schedule dispatch: which operators have a time-fused kernel, the tile
// and depth for a grid, and the launch routed to the per-operator instantiations.
#include "df64.cuh"
#include "fused.cuh"

namespace girih {

bool fused_supported(const Geom &g, int precision) {
  // the fused kernels index with 32-bit element offsets
  if (g.elems >= ((int64_t)1 << 31)) return false;
  if (g.op == 0 || g.op == 1 || g.op == 7 || g.op == 8) return true;
  // variable coefficients: FP32 fields (FP32 or BF16 coefficients); their FP64
  // form is bound by the FP64 pipe, where fusion cannot help
  return (g.op >= 2 && g.op <= 5) && (precision == GIRIH_FP32 || precision == GIRIH_MIXED);
}

int fused_max_depth(const Geom &g, int precision) {
  if (g.r == 4) return 2;
  if (g.var) return 3;
  if (precision == GIRIH_FP64_DF) return 3;
  return precision == GIRIH_FP64 ? 2 : 4;
}

// Column region of one CTA (every thread owns an x pair):
//   radius 1 (x pairs per thread): variant 0 = 64 x 32 (32x16 threads, 2 rows
//   each), variant 1 = 32 x 64 (16x64 threads, 1 row each);
//   radius 4 (one column per thread): variant 0 = 64 x 32 (64x16 threads, 2
//   rows), variant 1 = 32 x 64 (32x32 threads, 2 rows);
//   variants 2 and 3: 0 and 1 with TMA-staged input planes (variant 2 at
//   depth 4: x quads, 16x32 threads, one row each);
//   double-float: one column per thread in variants 0 = 64 x 32 (64x16 threads,
//   2 rows), 1 = 32 x 32 (32x16 threads, 2 rows), 2 = 64 x 16 (64x16 threads,
//   1 row); x pairs (radius 1) in variants 3 = 64 x 32 (32x16 threads, 2 rows)
//   and 4 = 32 x 64 (16x64 threads, 1 row).  (Double-float x quads, 16x32
//   threads, measured 143 vs 163 GLUP/s for x pairs at depth 2.)
static void variant_shape(int v, int r, int precision, int *ntx, int *ry, int *vx) {
  if (precision == GIRIH_FP64_DF) {
    static const int shape[5][3] = {{64, 32, 1}, {32, 32, 1}, {64, 16, 1}, {64, 32, 2}, {32, 64, 2}};
    *ntx = shape[v][0];
    *ry = shape[v][1];
    *vx = shape[v][2];
    return;
  }
  *ntx = (v % 2) == 0 ? 64 : 32;
  *ry = (v % 2) == 0 ? 32 : 64;
  *vx = r == 1 ? 2 : 1;
}

// Output tile width of a region ntx columns wide with halo h whose start is
// aligned to `align` columns (the kernel's FusedShape::BX): for the
// register/global-load variants a multiple of align when that is at least as
// wide as the general width ntx - 2h - (align-1); the TMA and double-float
// variants keep the general width, so that an output tile names one variant.
int fused_tile_width(int ntx, int h, int align, bool general_only) {
  const int mis = ((-h) % align + align) % align;
  const int aligned = (ntx - 2 * h - mis) / align * align, general = ntx - 2 * h - (align - 1);
  return !general_only && aligned >= general ? aligned : general;
}

// The box operator's own kernel (fused_box.cu): variant 0 = 32 x 32 region
// (32x16 threads, two rows each), variant 1 = 64 x 16 (64x16 threads, one row);
// one column per thread, a halo of one column per level.
static FusedConfig make_box_config(int precision, int depth, int variant) {
  FusedConfig c{};
  if (variant > 1 || (precision == GIRIH_FP64_DF && variant == 1 && depth > 2)) return c;
  const int ntx = variant == 0 ? 32 : 64, ry = variant == 0 ? 32 : 16;
  c.depth = depth;
  c.variant = variant;
  c.bx = ntx - 2 * depth;
  c.by = ry - 2 * depth;
  if (c.bx <= 0 || c.by <= 0) c.depth = 0;
  return c;
}

// Operator 0 (radius 4), variant 5: the TMA-staged one-step pass of
// fused_df_tma4.cu (32 x 32 tile; 40 x 40 boxes of the input state, 32 x 32 of
// the old state and roc2) for `esize`-byte elements; the boxes start at x
// offsets g.ox and g.ox + r, which must sit on 16 bytes.
static FusedConfig make_tma4_config(const Geom &g, int esize, int depth, int variant) {
  FusedConfig c{};
  if (g.op != 0 || depth != 1 || variant != 5 || (g.ox * esize) % 16 || ((g.ox + g.r) * esize) % 16) return c;
  if (tma4_smem(esize) > (size_t)227 * 1024) return c;
  c.depth = 1;
  c.variant = 5;
  c.bx = c.by = tma4_tile();
  c.box_w = c.box_h = tma4_box();
  c.box2_w = c.box2_h = tma4_tile();
  return c;
}

// Double-float radius-1 constant-coefficient operators (1, 8), variants 5 and 6:
// the TMA-staged kernel of fused_df_tma.cu (32 rows, 32 or 64 columns, depth
// <= 2).  Its boxes start on 16 bytes (2 columns), so the tile is the aligned
// width where that loses nothing (depth 2) and the general one else.  Operator
// 0 (radius 4): variant 5 is fused_df_tma4.cu, depth 1, a 32 x 32 tile.
static FusedConfig make_df_tma_config(const Geom &g, int depth, int variant) {
  FusedConfig c{};
  if (g.op == 0) return make_tma4_config(g, 8, depth, variant);
  if (g.r != 1 || g.var || g.op == 7 || depth > 2) return c;
  const int cols = df_tma_cols(variant), rows = df_tma_rows(variant);
  if (df_tma_smem(g.to, depth, cols, rows) > (size_t)227 * 1024) return c;
  c.depth = depth;
  c.variant = variant;
  c.bx = fused_tile_width(cols, depth, 2, false);
  c.by = rows - 2 * depth;
  c.box_w = cols;
  c.box_h = rows;
  return c;
}

FusedConfig make_fused_config(const Geom &g, int precision, int depth, int variant) {
  FusedConfig c{};
  if (!fused_supported(g, precision) || depth < 1 || depth > fused_max_depth(g, precision) ||
      variant < 0 || variant >= FV_COUNT)
    return c;
  if (g.op == 7) return make_box_config(precision, depth, variant);
  if (variant >= 5) return precision == GIRIH_FP64_DF ? make_df_tma_config(g, depth, variant) : make_tma4_config(g, 4, depth, variant);
  int ntx, ry, vx;
  variant_shape(variant, g.r, precision, &ntx, &ry, &vx);
  if (variant == 2 && precision != GIRIH_FP64_DF && ((g.r == 1 && depth == 4) || (g.r == 4 && depth == 1)))
    vx = 4;  // x quads: radius 1 at depth 4, radius 4 at depth 1
  if (variant == 3 && precision != GIRIH_FP64_DF && g.r == 1 && depth <= 2) {
    ntx = 64;  // 64 x 64 region with x quads
    vx = 4;
  }
  // double-buffered shared memory of all levels (rows padded by r), plus the TMA
  // rings of the TMA variants, must fit one CTA (227 KiB)
  const size_t tsz = (precision == GIRIH_FP64 || precision == GIRIH_FP64_DF) ? 8 : 4;
  const bool tma = variant >= 2 && precision != GIRIH_FP64_DF;
  if (tma && (tsz != 4 || g.var)) return c;  // TMA variants: FP32 storage, constant coefficients
  if (precision == GIRIH_FP64_DF && variant >= 2 && g.r != 1) return c;
  if (precision != GIRIH_FP64_DF && variant == 4) return c;
  const int rp = (g.r + vx - 1) / vx * vx;
  size_t smem = (size_t)2 * depth * (ntx + 2 * rp) * (ry + 2 * g.r) * tsz;
  int align = vx;
  if (tma) {
    const int nb = fused_tma_nb(g.r, depth, ntx * ry), nr = fused_tma_nr(g.r, depth, nb);
    const size_t plane = (size_t)ntx * ry * tsz;
    smem = (smem + 127) / 128 * 128 + nb * plane + (g.to == 2 ? (nb + nr) * plane : 0) + nb * 8;
    align = 16 / (int)tsz > vx ? 16 / (int)tsz : vx;
    c.box_w = ntx;
    c.box_h = ry;
  }
  if (smem > (size_t)227 * 1024) return FusedConfig{};
  c.depth = depth;
  c.variant = variant;
  c.bx = fused_tile_width(ntx, depth * g.r, align, tma || precision == GIRIH_FP64_DF);
  c.by = ry - 2 * depth * g.r;
  if (c.bx <= 0 || c.by <= 0) c.depth = 0;
  return c;
}

FusedConfig choose_fused_config(const Geom &g, int precision, int depth, int bx, int by) {
  int d = depth;
  // untuned: the depth that measured fastest per precision (double-float: depth
  // 2, the TMA-staged 64 x 32 region first below; at radius 4 one step per pass,
  // the TMA-staged 32 x 32 tile of operator 0)
  if (d <= 0) {
    if (g.r == 4) d = precision == GIRIH_FP64_DF ? 1 : 2;
    else d = (precision == GIRIH_FP64 || precision == GIRIH_FP64_DF) ? 2 : 4;
  }
  d = d > fused_max_depth(g, precision) ? fused_max_depth(g, precision) : d;
  // double-float: the TMA-staged variants first (the 64 x 32 region, fastest at
  // 512^3, as the untuned choice), so that a tile they share with a register
  // variant (28 x 28 and 60 x 28 at depth 2) selects them
  static const int df_order[FV_COUNT] = {6, 5, 0, 1, 2, 3, 4};
  for (int k = 0; k < FV_COUNT; k++) {
    const int v = precision == GIRIH_FP64_DF ? df_order[k] : k;
    FusedConfig c = make_fused_config(g, precision, d, v);
    if (!c.depth) continue;
    if ((bx && bx != c.bx) || (by && by != c.by)) continue;
    return c;
  }
  return FusedConfig{};
}

cudaError_t launch_fused(const Geom &g, int tsz, int precision, const FusedConfig &cfg,
                         const FusedLaunch &L, cudaStream_t s) {
  const bool comp = precision == GIRIH_MIXED && g.to == 2;
  if (precision == GIRIH_FP64_DF) {
    switch (g.op) {
      case 1: return launch_fused_op<1, Df64, false>(g, cfg, L, s);
      case 8: return launch_fused_op<8, Df64, false>(g, cfg, L, s);
      case 0: return launch_fused_op<0, Df64, false>(g, cfg, L, s);
      case 7: return launch_fused_op<7, Df64, false>(g, cfg, L, s);
    }
    return cudaErrorInvalidValue;
  }
  const bool bf16 = precision == GIRIH_MIXED && g.var;
  switch (g.op) {
    case 2: return bf16 ? launch_fused_op<2, float, true>(g, cfg, L, s) : launch_fused_op<2, float, false>(g, cfg, L, s);
    case 3: return bf16 ? launch_fused_op<3, float, true>(g, cfg, L, s) : launch_fused_op<3, float, false>(g, cfg, L, s);
    case 4: return bf16 ? launch_fused_op<4, float, true>(g, cfg, L, s) : launch_fused_op<4, float, false>(g, cfg, L, s);
    case 5: return bf16 ? launch_fused_op<5, float, true>(g, cfg, L, s) : launch_fused_op<5, float, false>(g, cfg, L, s);
    case 1:
      return tsz == 8 ? launch_fused_op<1, double, false>(g, cfg, L, s)
                      : launch_fused_op<1, float, false>(g, cfg, L, s);
    case 7:
      return tsz == 8 ? launch_fused_op<7, double, false>(g, cfg, L, s)
                      : launch_fused_op<7, float, false>(g, cfg, L, s);
    case 8:
      if (tsz == 8) return launch_fused_op<8, double, false>(g, cfg, L, s);
      return comp ? launch_fused_op<8, float, true>(g, cfg, L, s) : launch_fused_op<8, float, false>(g, cfg, L, s);
    case 0:
      if (tsz == 8) return launch_fused_op<0, double, false>(g, cfg, L, s);
      return comp ? launch_fused_op<0, float, true>(g, cfg, L, s) : launch_fused_op<0, float, false>(g, cfg, L, s);
  }
  return cudaErrorInvalidValue;
}

const char *fused_kernel_name(int op, int precision, const FusedConfig &cfg) {
  if (op == 7) return "fused_box_pass";
  if (precision == GIRIH_FP64_DF && cfg.variant >= 5) return "fused_df_tma";
  if (cfg.variant >= 5) return "fused_f32_tma4";
  return cfg.box_w > 0 ? "fused_pass_tma" : "fused_pass";
}

}  // namespace girih
