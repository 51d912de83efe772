// Internal layout of a girih_gpu_ctx, shared by the single-grid entry points
// (girih_gpu.cu) and the batched entry points (batched.cu).
#pragma once
#include <cuda.h>

#include "fused.cuh"
#include "internal.cuh"

struct girih_gpu_ctx {
  girih_gpu_desc d{};
  girih::Geom g{};
  int tsz = 8, hsz = 8;
  bool bf16coef = false;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  void *f[4] = {nullptr, nullptr, nullptr, nullptr};  // field buffers
  int iu1 = 0, iu2 = 1;                               // buffers holding U1 and U2
  void *roc2 = nullptr;
  // double-float fused form: FP32-pair mirrors of the four field buffers and
  // roc2, split from the FP64 buffers at the start of each run and joined back
  // at its end (the FP64 buffers stay the state every other entry point sees)
  void *dfp[4] = {nullptr, nullptr, nullptr, nullptr};
  void *dfr2 = nullptr;
  void *coef = nullptr;
  float *scale = nullptr;
  // source point: device element offset, value count, device values (FP64)
  int64_t src_off = -1;
  int src_n = 0;
  double *d_src = nullptr;
  int d_src_cap = 0;
  double cc[5] = {0, 0, 0, 0, 0};
  void *staging = nullptr;
  size_t staging_bytes = 0;
  double *acc = nullptr;  // 4 doubles for norms, then flag words
  bool uploaded = false;
  bool halos_equal = false;
  int sched = GIRIH_SCHED_PLAIN;
  girih::FusedConfig fcfg{};
  cudaGraphExec_t gexec = nullptr;
  int g_steps = -1, g_iu1 = -1, g_iu2 = -1;
  int g_launches = 0, g_new_iu1 = 0, g_new_iu2 = 1;
  int last_launches = 0, last_steps = 0;
  double dev_bytes = 0;
  // TMA tensor maps of the four field buffers and roc2 (index 4), per TMA variant (2, 3; double-float 5, 6)
  CUtensorMap tmaps[5][2];
  bool tmap_ok[5][2] = {{false, false}, {false, false}, {false, false}, {false, false}, {false, false}};
  int tmap_box[5][2][2] = {};  // box (x, y) each cached map was encoded with: a variant's box can change with depth
  const void *tmap_base[5][2] = {};  // array each cached map was encoded for
  // checked build: per-buffer write counters (one per element) and the number
  // of times the captured schedule writes each buffer's interior
  unsigned *cov[4] = {nullptr, nullptr, nullptr, nullptr};
  int run_expect[4] = {0, 0, 0, 0};  // of the steps last issued
  int g_expect[4] = {0, 0, 0, 0};    // of the captured graph
};

namespace girih {
// Issue the launches of `steps` time steps of context c on stream st; *iu1/*iu2
// carry the buffers holding U1/U2 in and out.  Defined in girih_gpu.cu.
int issue_steps_on(girih_gpu_ctx *c, int steps, int *launches, int *iu1, int *iu2, cudaStream_t st);
int ensure_fused_buffers_pub(girih_gpu_ctx *c);
}  // namespace girih
