// C-ABI entry points of libgirih_gpu (declared in include/girih_gpu.h).
//
// A context holds one grid on one device: field buffers in the device layout
// (see Geom), roc2, coefficients, a staging buffer for host-layout conversion
// and a stream.  run() replays a captured CUDA graph of the whole time loop
// between two CUDA events on that stream, which replaces the reference's
// MPI_Wtime bracket around the stepper (src/performance.c:74-78).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "internal.cuh"
#include "check.cuh"
#include "fused.cuh"

namespace girih {

static thread_local std::string g_last_error;
void set_error(const std::string &msg) { g_last_error = msg; }

int op_info(int op, int *r, int *to, int *nc, int *var) {
  int R, TO, NC, VAR;
  switch (op) {  // src/kernels/stencils.c:260-271
    case 0: R = 4; TO = 2; NC = 5; VAR = 0; break;
    case 1: R = 1; TO = 1; NC = 2; VAR = 0; break;
    case 2: R = 1; TO = 1; NC = 2; VAR = 1; break;
    case 3: R = 1; TO = 1; NC = 4; VAR = 1; break;
    case 4: R = 4; TO = 1; NC = 13; VAR = 1; break;
    case 5: R = 1; TO = 1; NC = 7; VAR = 1; break;
    case 7: R = 1; TO = 1; NC = 4; VAR = 0; break;
    case 8: R = 1; TO = 2; NC = 2; VAR = 0; break;
    default: return -1;
  }
  if (r) *r = R;
  if (to) *to = TO;
  if (nc) *nc = NC;
  if (var) *var = VAR;
  return 0;
}

Geom make_geom(int op, int nx, int ny, int nz, int hpx, int tsz) {
  Geom g{};
  op_info(op, &g.r, &g.to, &g.nc, &g.var);
  g.op = op;
  g.nx = nx; g.ny = ny; g.nz = nz;
  g.nnx = nx + 2 * g.r; g.nny = ny + 2 * g.r; g.nnz = nz + 2 * g.r;
  g.hpx = hpx;
  const int A = 128 / tsz;  // elements per 128 bytes
  g.ox = (A - (g.r % A)) % A;
  g.px = ((g.ox + g.nnx + A - 1) / A) * A;
  g.plane = (int64_t)g.px * g.nny;
  g.elems = g.plane * g.nnz;
  return g;
}

}  // namespace girih

using namespace girih;

#include "context.cuh"

namespace {

// Autotuner choices, per (operator, precision, size class).
struct TuneChoice {
  int sched, variant, depth;
};
std::mutex g_tune_mutex;
std::map<std::tuple<int, int, int>, TuneChoice> g_tune_cache;

int size_class(const Geom &g) {
  double pts = (double)g.nx * g.ny * g.nz;
  return (int)std::floor(std::log2(pts > 1 ? pts : 1));
}

// Untuned default of the auto schedule, from measurements at 384^3-512^3:
// FP64 arithmetic is bound by the FP64 pipe, where fusion only adds the halo
// recomputation (operator 8: 51 plain vs 36 fused GLUP/s); double-float
// arithmetic exists in the fused passes only; in FP32 fields fusion wins for
// the radius-1 constant operators (operator 8: 512 vs 356, operator 1: 722 vs
// 609) and loses where the overlapped tiles recompute many points or stream
// coefficient arrays (radius 4: 176 vs 237; variable coefficients: 200 vs 268).
bool auto_prefers_fused(const Geom &g, int precision) {
  if (precision == GIRIH_FP64_DF) return true;
  if (precision == GIRIH_FP64) return false;
  return !g.var && g.r == 1;
}

bool cached_choice(const Geom &g, int precision, TuneChoice *out) {
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  auto it = g_tune_cache.find(std::make_tuple(g.op, precision, size_class(g)));
  if (it == g_tune_cache.end()) return false;
  *out = it->second;
  return true;
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

#define CK(...)                                                                    \
  do {                                                                             \
    cudaError_t e_ = (__VA_ARGS__);                                                \
    if (e_ != cudaSuccess) {                                                       \
      set_error(std::string(#__VA_ARGS__) + ": " + cudaGetErrorString(e_));        \
      return e_ == cudaErrorMemoryAllocation ? GIRIH_GPU_ENOMEM : GIRIH_GPU_ECUDA; \
    }                                                                              \
  } while (0)

int fail(int code, const std::string &msg) {
  set_error(msg);
  return code;
}

int dev_alloc(girih_gpu_ctx *c, void **p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(GIRIH_GPU_ENOMEM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed: " +
                                      cudaGetErrorString(e));
  }
  c->dev_bytes += (double)bytes;
  CK(cudaMemsetAsync(*p, 0, bytes, c->st));
  return 0;
}

int ensure_staging(girih_gpu_ctx *c, size_t bytes) {
  if (c->staging_bytes >= bytes) return 0;
  if (c->staging) {
    cudaFree(c->staging);
    c->dev_bytes -= (double)c->staging_bytes;
    c->staging = nullptr;
    c->staging_bytes = 0;
  }
  int e = dev_alloc(c, &c->staging, bytes);
  if (!e) c->staging_bytes = bytes;
  return e;
}

size_t host_array_elems(const girih_gpu_ctx *c) {
  return (size_t)c->d.ldomain_shape[0] * c->d.ldomain_shape[1] * c->d.ldomain_shape[2];
}

// Device address of a host array the GPU can reach directly (pinned or
// registered host memory), else nullptr (pageable memory).
const void *pinned_alias(const void *h) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
    cudaGetLastError();  // clear the sticky-free error of an unknown pointer
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Layout kernel between host-layout src (element hsz) and device-layout dst (tsz).
cudaError_t host_to_device_layout(const girih_gpu_ctx *c, const void *src, void *dst) {
  const Geom &g = c->g;
  if (c->hsz == 8 && c->tsz == 8) return launch_to_device_layout<double, double>(g, (const double *)src, (double *)dst, c->st);
  if (c->hsz == 8) return launch_to_device_layout<double, float>(g, (const double *)src, (float *)dst, c->st);
  if (c->tsz == 8) return launch_to_device_layout<float, double>(g, (const float *)src, (double *)dst, c->st);
  return launch_to_device_layout<float, float>(g, (const float *)src, (float *)dst, c->st);
}
cudaError_t device_to_host_layout(const girih_gpu_ctx *c, const void *src, void *dst) {
  const Geom &g = c->g;
  if (c->hsz == 8 && c->tsz == 8) return launch_to_host_layout<double, double>(g, (const double *)src, (double *)dst, c->st);
  if (c->hsz == 8) return launch_to_host_layout<float, double>(g, (const float *)src, (double *)dst, c->st);
  if (c->tsz == 8) return launch_to_host_layout<double, float>(g, (const double *)src, (float *)dst, c->st);
  return launch_to_host_layout<float, float>(g, (const float *)src, (float *)dst, c->st);
}

// Host (reference layout, element size hsz) -> device layout buffer (tsz).  A
// pinned host array is read by the layout kernel itself (one pass over the
// host link, no staging); a pageable one arrives by one contiguous copy into
// the staging buffer, which the layout kernel then converts.
int upload_field(girih_gpu_ctx *c, const void *h, void *dst) {
  if (const void *dh = pinned_alias(h)) {
    CK(host_to_device_layout(c, dh, dst));
    return 0;
  }
  size_t n = host_array_elems(c);
  int e = ensure_staging(c, n * 8);
  if (e) return e;
  CK(cudaMemcpyAsync(c->staging, h, n * c->hsz, cudaMemcpyHostToDevice, c->st));
  CK(host_to_device_layout(c, c->staging, dst));
  return 0;
}

// Device layout -> host array.  Only the nnx columns of each row are written
// (the caller's x padding is left as it is): directly by the layout kernel into
// a pinned host array, else through the staging buffer and a row-wise copy.
int download_field(girih_gpu_ctx *c, const void *src, void *h) {
  const Geom &g = c->g;
  if (const void *dh = pinned_alias(h)) {
    CK(device_to_host_layout(c, src, const_cast<void *>(dh)));
    return 0;
  }
  size_t n = host_array_elems(c);
  int e = ensure_staging(c, n * 8);
  if (e) return e;
  CK(device_to_host_layout(c, src, c->staging));
  CK(cudaMemcpy2DAsync(h, (size_t)g.hpx * c->hsz, c->staging, (size_t)g.hpx * c->hsz,
                       (size_t)g.nnx * c->hsz, (size_t)g.nny * g.nnz, cudaMemcpyDeviceToHost, c->st));
  return 0;
}

// Quantise coefficient array m (host layout, already in staging as Tin) to BF16.
template <class Tin>
int quantize_from_staging(girih_gpu_ctx *c, int m) {
  unsigned long long *mx = reinterpret_cast<unsigned long long *>(c->acc + 4);
  CK(cudaMemsetAsync(mx, 0, 8, c->st));
  CK(launch_maxabs<Tin>(c->g, (const Tin *)c->staging, mx, c->st));
  unsigned long long bits = 0;
  CK(cudaMemcpyAsync(&bits, mx, 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  double mxv;
  std::memcpy(&mxv, &bits, 8);
  float s = (mxv > 0 && mxv == mxv) ? (float)mxv : 1.0f;
  CK(cudaMemcpyAsync(c->scale + m, &s, 4, cudaMemcpyHostToDevice, c->st));
  __nv_bfloat16 *dst = static_cast<__nv_bfloat16 *>(c->coef) + (size_t)m * c->g.elems;
  CK(launch_quantize_bf16<Tin>(c->g, (const Tin *)c->staging, dst, c->scale + m, c->st));
  CK(cudaStreamSynchronize(c->st));  // the host scale value must outlive the copy
  return 0;
}

int check_halos(girih_gpu_ctx *c) {
  unsigned int *flag = reinterpret_cast<unsigned int *>(c->acc + 5);
  CK(cudaMemsetAsync(flag, 0, 4, c->st));
  CK(launch_halo_equal(c->g, c->f[0], c->f[1], c->tsz, flag, c->st));
  unsigned int h = 1;
  CK(cudaMemcpyAsync(&h, flag, 4, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->halos_equal = (h == 0);
  return 0;
}

void drop_graph(girih_gpu_ctx *c) {
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  c->gexec = nullptr;
  c->g_steps = -1;
}

// TMA tensor map of a device-layout array (3-D: x pitch, rows, planes) with the
// box of a TMA variant; encoded once per (array, variant) and kept in the context.
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    cudaGetLastError();
  }
  return fn;
}

// Tensor map of array `arr` (buffers 0-3, roc2 4) in cache slot v with box bw x bh.
static const CUtensorMap *tensor_map_box(girih_gpu_ctx *c, int arr, const void *base, int v, int bw, int bh) {
  if (v < 0 || v > 1) return nullptr;
  // re-encode when the box or the array changed: a TMA copy of another width
  // would overrun (or under-fill) the ring slots the kernel sized for its own region
  if (!c->tmap_ok[arr][v] || c->tmap_box[arr][v][0] != bw || c->tmap_box[arr][v][1] != bh ||
      c->tmap_base[arr][v] != base) {
    c->tmap_ok[arr][v] = false;
    EncodeTiledFn fn = encode_tiled();
    if (!fn) return nullptr;
    const Geom &g = c->g;
    const cuuint64_t dims[3] = {(cuuint64_t)g.px, (cuuint64_t)g.nny, (cuuint64_t)g.nnz};
    const cuuint64_t strides[2] = {(cuuint64_t)g.px * c->tsz, (cuuint64_t)g.px * g.nny * c->tsz};
    const cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)bh, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(&c->tmaps[arr][v], c->tsz == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                    3, const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return nullptr;
    c->tmap_ok[arr][v] = true;
    c->tmap_box[arr][v][0] = bw;
    c->tmap_box[arr][v][1] = bh;
    c->tmap_base[arr][v] = base;
  }
  return &c->tmaps[arr][v];
}

// The variant's map of `arr`: one cache slot per TMA variant of the context's
// precision, 2 and 3 (FP32 storage) or 5 and 6.  `second`: the old state's and
// roc2's box where the variant gives them their own (operator 0's variant 5,
// which has no variant 6, keeps those maps in the second slot).
const CUtensorMap *tensor_map(girih_gpu_ctx *c, int arr, const void *base, bool second) {
  const int v = c->fcfg.variant >= 5 ? c->fcfg.variant - 5 : c->fcfg.variant - 2;
  if (second && c->fcfg.box2_w > 0) return tensor_map_box(c, arr, base, 1 - v, c->fcfg.box2_w, c->fcfg.box2_h);
  return tensor_map_box(c, arr, base, v, c->fcfg.box_w, c->fcfg.box_h);
}

// Extra field buffers for the fused schedule: inputs and outputs of a fused
// pass must differ because neighbouring tiles read overlapping halos.
int ensure_fused_buffers(girih_gpu_ctx *c) {
  const size_t fb = (size_t)c->g.elems * c->tsz;
  for (int b = 2; b < 4; b++) {
    if (!c->f[b]) {
      int e = dev_alloc(c, &c->f[b], fb);
      if (e) return e;
    }
  }
  if (c->d.precision == GIRIH_FP64_DF) {
    for (int b = 0; b < 4; b++)
      if (!c->dfp[b]) {
        int e = dev_alloc(c, &c->dfp[b], fb);
        if (e) return e;
      }
    if (c->g.to == 2 && !c->dfr2) {
      int e = dev_alloc(c, &c->dfr2, fb);
      if (e) return e;
    }
  }
  return 0;
}

template <class T> StepArgs<T> step_args(girih_gpu_ctx *c, void *u, const void *v) {
  StepArgs<T> a{};
  a.g = c->g;
  a.u = static_cast<T *>(u);
  a.v = static_cast<const T *>(v);
  a.roc2 = static_cast<const T *>(c->roc2);
  a.coef = c->coef;
  a.scale = c->scale;
  for (int m = 0; m < 5; m++) a.cc[m] = (T)c->cc[m];
  return a;
}

// Issue the launches of `steps` time steps on the context stream (captured
// into a graph by the caller).  Plain: U1 <- op(U2), U2 <- op(U1) in place of
// the reference's two sweeps per iteration.  Fused: passes of depth T rotate
// through the four field buffers.
int issue_steps_impl(girih_gpu_ctx *c, int steps, int *launches, int *iu1, int *iu2, cudaStream_t st) {
  *launches = 0;
  const bool exact = c->d.exact != 0;
  unsigned *flag = reinterpret_cast<unsigned *>(c->acc + 6);
  // the checked build's write counters: how often these steps write each buffer
  for (int b = 0; b < 4; b++) c->run_expect[b] = 0;
  if (c->sched == GIRIH_SCHED_PLAIN) {
    for (int s = 0; s < steps; s += 2) {
      for (int h = 0; h < 2; h++) {
        const int ub = h == 0 ? *iu1 : *iu2;
        void *u = c->f[ub];
        const void *v = c->f[h == 0 ? *iu2 : *iu1];
        const int sweep = s + h;
        const double *src = c->d_src && sweep < c->src_n ? c->d_src + sweep : nullptr;
        c->run_expect[ub]++;
        cudaError_t e;
        if (c->tsz == 8) {
          StepArgs<double> a = step_args<double>(c, u, v);
          a.src = src;
          a.src_off = c->src_off;
          a.flag = flag;
          a.cov = c->cov[ub];
          e = launch_plain<double>(a, exact, false, st);
        } else {
          StepArgs<float> a = step_args<float>(c, u, v);
          a.src = src;
          a.src_off = c->src_off;
          a.flag = flag;
          a.cov = c->cov[ub];
          e = launch_plain<float>(a, exact, c->bf16coef, st);
        }
        if (e != cudaSuccess) return fail(GIRIH_GPU_ECUDA, std::string("plain launch: ") + cudaGetErrorString(e));
        *launches += src ? 2 : 1;  // the sweep, and the source-point update
      }
    }
    return 0;
  }
  // fused: state S-1 in buffer iu1, state S in iu2; each pass writes the two
  // newest states into the two spare buffers
  const bool dfp = c->d.precision == GIRIH_FP64_DF;
  void *const *buf = dfp ? c->dfp : c->f;
  if (dfp && steps > 0) {
    // FP64 -> pairs: both states, the spares (whose halos the passes read), roc2
    int sp[2], n = 0;
    for (int b = 0; b < 4 && n < 2; b++)
      if (b != *iu1 && b != *iu2) sp[n++] = b;
    cudaError_t e = launch_df_split(c->g, static_cast<const double *>(c->f[*iu1]), c->dfp[*iu1], nullptr, nullptr,
                                    flag, st);
    if (e == cudaSuccess)
      e = launch_df_split(c->g, static_cast<const double *>(c->f[*iu2]), c->dfp[*iu2], c->dfp[sp[0]], c->dfp[sp[1]],
                          flag, st);
    if (e == cudaSuccess && c->g.to == 2)
      e = launch_df_split(c->g, static_cast<const double *>(c->roc2), c->dfr2, nullptr, nullptr, flag, st);
    if (e != cudaSuccess) return fail(GIRIH_GPU_ECUDA, std::string("double-float split: ") + cudaGetErrorString(e));
    *launches += c->g.to == 2 ? 3 : 2;
  }
  int left = steps;
  while (left > 0) {
    int T = std::min(left, c->fcfg.depth);
    int spare[2], n = 0;
    for (int b = 0; b < 4 && n < 2; b++)
      if (b != *iu1 && b != *iu2) spare[n++] = b;
    FusedLaunch L{};
    L.prev = buf[*iu1];
    L.cur = buf[*iu2];
    L.out_prev = buf[spare[0]];
    L.out_cur = buf[spare[1]];
    L.roc2 = dfp ? c->dfr2 : c->roc2;
    L.steps = T;
    // time order 1 never reads state t-1, so only the last pass writes it (U1)
    L.write_prev = (c->g.to == 2 || left == T) ? 1 : 0;
    L.range_flag = flag;
    L.cov_prev = c->cov[spare[0]];
    L.cov_cur = c->cov[spare[1]];
    c->run_expect[spare[1]]++;
    if (L.write_prev) c->run_expect[spare[0]]++;
    L.coef = c->coef;
    L.cscale = c->scale;
    if (c->d_src && c->src_n > 0) {
      L.src = c->d_src;
      L.src_off = (int)c->src_off;
      L.src_t0 = steps - left;
      L.src_n = c->src_n;
    }
    if (c->fcfg.box_w > 0) {  // TMA variant
      L.tma_prev = tensor_map(c, *iu1, buf[*iu1], true);
      L.tma_cur = tensor_map(c, *iu2, buf[*iu2], false);
      L.tma_roc2 = c->g.to == 2 ? tensor_map(c, 4, dfp ? c->dfr2 : c->roc2, true) : L.tma_cur;
      L.tma_box_w = c->fcfg.box_w;
      L.tma_box_h = c->fcfg.box_h;
      L.tma_box2_w = c->fcfg.box2_w > 0 ? c->fcfg.box2_w : c->fcfg.box_w;
      L.tma_box2_h = c->fcfg.box2_h > 0 ? c->fcfg.box2_h : c->fcfg.box_h;
      if (!L.tma_prev || !L.tma_cur || !L.tma_roc2)
        return fail(GIRIH_GPU_ECUDA, "TMA tensor map encoding failed");
    }
    for (int m = 0; m < 5; m++) L.cc[m] = c->cc[m];
    cudaError_t e = launch_fused(c->g, c->tsz, c->d.precision, c->fcfg, L, st);
    if (e != cudaSuccess) return fail(GIRIH_GPU_ECUDA, std::string("fused launch: ") + cudaGetErrorString(e));
    (*launches)++;
    *iu1 = spare[0];
    *iu2 = spare[1];
    left -= T;
  }
  if (dfp && steps > 0) {  // pairs -> FP64 (interior points; the halos keep their FP64 values)
    cudaError_t e = launch_df_join(c->g, c->dfp[*iu1], static_cast<double *>(c->f[*iu1]), st);
    if (e == cudaSuccess) e = launch_df_join(c->g, c->dfp[*iu2], static_cast<double *>(c->f[*iu2]), st);
    if (e != cudaSuccess) return fail(GIRIH_GPU_ECUDA, std::string("double-float join: ") + cudaGetErrorString(e));
    *launches += 2;
  }
  return 0;
}

int issue_steps(girih_gpu_ctx *c, int steps, int *launches, int *iu1, int *iu2) {
  return issue_steps_impl(c, steps, launches, iu1, iu2, c->st);
}

}  // namespace

namespace girih {
int issue_steps_on(girih_gpu_ctx *c, int steps, int *launches, int *iu1, int *iu2, cudaStream_t st) {
  return issue_steps_impl(c, steps, launches, iu1, iu2, st);
}
int ensure_fused_buffers_pub(girih_gpu_ctx *c) { return ensure_fused_buffers(c); }
}  // namespace girih

extern "C" {

int girih_gpu_abi_version(void) { return GIRIH_GPU_ABI_VERSION; }

const char *girih_gpu_strerror(int err) {
  switch (err) {
    case GIRIH_GPU_OK: return "success";
    case GIRIH_GPU_EINVAL: return "invalid argument";
    case GIRIH_GPU_EUNSUPPORTED: return "unsupported operator/precision/schedule combination";
    case GIRIH_GPU_ECUDA: return "CUDA runtime error";
    case GIRIH_GPU_ENOMEM: return "device out of memory";
    case GIRIH_GPU_ESTATE: return "call out of order";
    case GIRIH_GPU_ETIMEOUT: return "device-side wait timed out";
    case GIRIH_GPU_ENODEV: return "no usable CUDA device";
    case GIRIH_GPU_ERANGE: return "value outside the range of the selected precision";
    case GIRIH_GPU_EBOUNDS: return "bounds-checked build: a kernel index left its array or shared block";
    case GIRIH_GPU_ECOVERAGE: return "bounds-checked build: a point was not written exactly once per step";
  }
  return "unknown error";
}

const char *girih_gpu_last_error(void) { return g_last_error.c_str(); }

int girih_gpu_create(girih_gpu_ctx **out, const girih_gpu_desc *d) {
  if (!out || !d) return fail(GIRIH_GPU_EINVAL, "null argument");
  *out = nullptr;
  int r, to, nc, var;
  if (op_info(d->target_kernel, &r, &to, &nc, &var))
    return fail(GIRIH_GPU_EUNSUPPORTED, "operator id " + std::to_string(d->target_kernel) +
                                            " is not a star operator provided on the GPU");
  const int nx = d->stencil_shape[0], ny = d->stencil_shape[1], nz = d->stencil_shape[2];
  if (nx < 1 || ny < 1 || nz < 1) return fail(GIRIH_GPU_EINVAL, "interior extents must be >= 1");
  if (d->ldomain_shape[0] < nx + 2 * r || d->ldomain_shape[1] != ny + 2 * r || d->ldomain_shape[2] != nz + 2 * r)
    return fail(GIRIH_GPU_EINVAL, "ldomain_shape must be (>= nx+2r, ny+2r, nz+2r)");
  if (d->host_real_size != 4 && d->host_real_size != 8) return fail(GIRIH_GPU_EINVAL, "host_real_size must be 4 or 8");
  if (d->precision < GIRIH_FP64 || d->precision > GIRIH_FP64_DF) return fail(GIRIH_GPU_EINVAL, "bad precision");
  if (d->schedule < GIRIH_SCHED_PLAIN || d->schedule > GIRIH_SCHED_AUTO) return fail(GIRIH_GPU_EINVAL, "bad schedule");
  if ((int64_t)d->ldomain_shape[0] * d->ldomain_shape[1] > (int64_t)1 << 31)
    return fail(GIRIH_GPU_EINVAL, "x-y plane too large");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return fail(GIRIH_GPU_ENODEV, "no CUDA device");
  }
  if (d->device < 0 || d->device >= ndev) return fail(GIRIH_GPU_EINVAL, "device ordinal out of range");
  DeviceGuard dg(d->device);

  girih_gpu_ctx *c = new (std::nothrow) girih_gpu_ctx;
  if (!c) return fail(GIRIH_GPU_ENOMEM, "host allocation failed");
  c->d = *d;
  c->tsz = (d->precision == GIRIH_FP64 || d->precision == GIRIH_FP64_DF) ? 8 : 4;
  c->hsz = d->host_real_size;
  c->bf16coef = d->precision == GIRIH_MIXED && var;
  c->g = make_geom(d->target_kernel, nx, ny, nz, d->ldomain_shape[0], c->tsz);

  // schedule selection
  int sched = d->schedule;
  if (sched != GIRIH_SCHED_PLAIN) {
    bool ok = fused_supported(c->g, d->precision);
    if (sched == GIRIH_SCHED_FUSED && !ok) {
      delete c;
      return fail(GIRIH_GPU_EUNSUPPORTED, "no fused kernel for this operator/precision");
    }
    if (sched == GIRIH_SCHED_FUSED && d->exact) {
      delete c;
      return fail(GIRIH_GPU_EUNSUPPORTED, "exact rounding is provided by the plain schedule only");
    }
    sched = ok && !d->exact ? GIRIH_SCHED_FUSED : GIRIH_SCHED_PLAIN;
  }
  c->sched = sched;
  TuneChoice tc{};
  const bool untuned = d->fusion_depth == 0 && d->block_x == 0 && d->block_y == 0;
  if (sched != GIRIH_SCHED_PLAIN && untuned && cached_choice(c->g, d->precision, &tc)) {
    if (d->schedule == GIRIH_SCHED_AUTO) c->sched = sched = tc.sched;
    if (tc.sched == GIRIH_SCHED_FUSED) c->fcfg = make_fused_config(c->g, d->precision, tc.depth, tc.variant);
  } else if (d->schedule == GIRIH_SCHED_AUTO && !auto_prefers_fused(c->g, d->precision)) {
    c->sched = sched = GIRIH_SCHED_PLAIN;  // only a tuning run that measured otherwise selects fusion
  }
  if (sched == GIRIH_SCHED_FUSED && !c->fcfg.depth) {
    c->fcfg = choose_fused_config(c->g, d->precision, d->fusion_depth, d->block_x, d->block_y);
    if (!c->fcfg.depth) {
      delete c;
      return fail(GIRIH_GPU_EUNSUPPORTED, "requested fused tile/depth is not provided");
    }
  }

  int e = 0;
  auto bail = [&](int code) {
    girih_gpu_destroy(c);
    return code;
  };
  if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->e0) != cudaSuccess || cudaEventCreate(&c->e1) != cudaSuccess) {
    cudaGetLastError();
    return bail(fail(GIRIH_GPU_ECUDA, "stream/event creation failed"));
  }
  const size_t fb = (size_t)c->g.elems * c->tsz;
  if ((e = dev_alloc(c, &c->f[0], fb)) || (e = dev_alloc(c, &c->f[1], fb))) return bail(e);
  if (to == 2 && (e = dev_alloc(c, &c->roc2, fb))) return bail(e);
  if (var) {
    size_t cb = (size_t)c->g.elems * nc * (c->bf16coef ? 2 : c->tsz);
    if ((e = dev_alloc(c, &c->coef, cb))) return bail(e);
    if (c->bf16coef && (e = dev_alloc(c, (void **)&c->scale, 64 * sizeof(float)))) return bail(e);
  }
  if ((e = dev_alloc(c, (void **)&c->acc, 64))) return bail(e);
  if (GIRIH_CHECKED)  // write counters of the four state buffers
    for (int b = 0; b < 4; b++)
      if ((e = dev_alloc(c, (void **)&c->cov[b], (size_t)c->g.elems * sizeof(unsigned)))) return bail(e);
  if (sched == GIRIH_SCHED_FUSED && (e = ensure_fused_buffers(c))) return bail(e);
  if (cudaStreamSynchronize(c->st) != cudaSuccess) return bail(fail(GIRIH_GPU_ECUDA, "initial clear failed"));
  *out = c;
  return 0;
}

void girih_gpu_destroy(girih_gpu_ctx *c) {
  if (!c) return;
  DeviceGuard dg(c->d.device);
  if (c->st) cudaStreamSynchronize(c->st);
  drop_graph(c);
  for (void *p : c->f)
    if (p) cudaFree(p);
  for (void *p : c->dfp)
    if (p) cudaFree(p);
  if (c->dfr2) cudaFree(c->dfr2);
  if (c->d_src) cudaFree(c->d_src);
  if (c->roc2) cudaFree(c->roc2);
  if (c->coef) cudaFree(c->coef);
  if (c->scale) cudaFree(c->scale);
  if (c->staging) cudaFree(c->staging);
  if (c->acc) cudaFree(c->acc);
  for (unsigned *p : c->cov)
    if (p) cudaFree(p);
  if (c->e0) cudaEventDestroy(c->e0);
  if (c->e1) cudaEventDestroy(c->e1);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
}

int girih_gpu_upload(girih_gpu_ctx *c, const void *U1, const void *U2, const void *U3, const void *coef) {
  if (!c || !U1 || !U2) return fail(GIRIH_GPU_EINVAL, "null context or field array");
  const Geom &g = c->g;
  if (g.to == 2 && !U3) return fail(GIRIH_GPU_EINVAL, "time-order-2 operator needs U3 (roc2)");
  if (!coef) return fail(GIRIH_GPU_EINVAL, "null coefficient array");
  DeviceGuard dg(c->d.device);
  drop_graph(c);
  c->uploaded = false;
  int e;
  if ((e = upload_field(c, U1, c->f[0])) || (e = upload_field(c, U2, c->f[1]))) return e;
  if (g.to == 2 && (e = upload_field(c, U3, c->roc2))) return e;
  if (!g.var) {
    for (int m = 0; m < 5; m++)
      c->cc[m] = m < g.nc ? (c->hsz == 8 ? static_cast<const double *>(coef)[m]
                                         : (double)static_cast<const float *>(coef)[m])
                          : 0.0;
  } else {
    const size_t n = host_array_elems(c);
    for (int m = 0; m < g.nc; m++) {
      const char *src = static_cast<const char *>(coef) + (size_t)m * n * c->hsz;
      if (!c->bf16coef) {
        if ((e = upload_field(c, src, static_cast<char *>(c->coef) + (size_t)m * g.elems * c->tsz))) return e;
      } else {
        if ((e = ensure_staging(c, n * 8))) return e;
        CK(cudaMemcpyAsync(c->staging, src, n * c->hsz, cudaMemcpyHostToDevice, c->st));
        if ((e = c->hsz == 8 ? quantize_from_staging<double>(c, m) : quantize_from_staging<float>(c, m))) return e;
      }
    }
  }
  c->iu1 = 0;
  c->iu2 = 1;
  if ((e = check_halos(c))) return e;
  if (c->sched == GIRIH_SCHED_FUSED && !c->halos_equal && c->d.schedule == GIRIH_SCHED_AUTO)
    c->sched = GIRIH_SCHED_PLAIN;  // unequal halos: keep the exact ping-pong of the plain schedule
  if (c->sched == GIRIH_SCHED_FUSED && !c->halos_equal)
    return fail(GIRIH_GPU_EUNSUPPORTED,
                "fused schedule needs identical U1/U2 halos (the reference initialises them equal)");
  if (c->sched == GIRIH_SCHED_FUSED) {
    // every buffer carries the fixed halo
    for (int b = 2; b < 4; b++)
      CK(cudaMemcpyAsync(c->f[b], c->f[1], (size_t)g.elems * c->tsz, cudaMemcpyDeviceToDevice, c->st));
  }
  CK(cudaStreamSynchronize(c->st));
  c->uploaded = true;
  return 0;
}

int girih_gpu_fill_seeded(girih_gpu_ctx *c, uint64_t seed, const double ranges[6], const double *const_coefs,
                          int flags) {
  if (!c || !ranges) return fail(GIRIH_GPU_EINVAL, "null argument");
  const Geom &g = c->g;
  if (!g.var && !const_coefs) return fail(GIRIH_GPU_EINVAL, "constant operator needs const_coefs");
  DeviceGuard dg(c->d.device);
  drop_graph(c);
  c->uploaded = false;
  const int rf = (flags & GIRIH_SEED_F32_EXACT) ? 1 : 0;
  if (c->tsz == 8) {
    CK(launch_seeded<double>(g, seed, 0, ranges[0], ranges[1], rf, (double *)c->f[0], nullptr, c->st));
    if (g.to == 2) CK(launch_seeded<double>(g, seed, 1, ranges[2], ranges[3], rf, (double *)c->roc2, nullptr, c->st));
  } else {
    CK(launch_seeded<float>(g, seed, 0, ranges[0], ranges[1], rf, (float *)c->f[0], nullptr, c->st));
    if (g.to == 2) CK(launch_seeded<float>(g, seed, 1, ranges[2], ranges[3], rf, (float *)c->roc2, nullptr, c->st));
  }
  CK(cudaMemcpyAsync(c->f[1], c->f[0], (size_t)g.elems * c->tsz, cudaMemcpyDeviceToDevice, c->st));
  if (g.var) {
    for (int m = 0; m < g.nc; m++) {
      if (!c->bf16coef) {
        void *dst = static_cast<char *>(c->coef) + (size_t)m * g.elems * c->tsz;
        if (c->tsz == 8)
          CK(launch_seeded<double>(g, seed, 2 + m, ranges[4], ranges[5], rf, (double *)dst, nullptr, c->st));
        else
          CK(launch_seeded<float>(g, seed, 2 + m, ranges[4], ranges[5], rf, (float *)dst, nullptr, c->st));
      } else {
        int e = ensure_staging(c, host_array_elems(c) * 8);
        if (e) return e;
        CK(launch_seeded<float>(g, seed, 2 + m, ranges[4], ranges[5], rf, nullptr, (double *)c->staging, c->st));
        if ((e = quantize_from_staging<double>(c, m))) return e;
      }
    }
  } else {
    for (int m = 0; m < 5; m++) c->cc[m] = m < g.nc ? const_coefs[m] : 0.0;
  }
  c->iu1 = 0;
  c->iu2 = 1;
  c->halos_equal = true;
  if (c->sched == GIRIH_SCHED_FUSED)
    for (int b = 2; b < 4; b++)
      CK(cudaMemcpyAsync(c->f[b], c->f[1], (size_t)g.elems * c->tsz, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->uploaded = true;
  return 0;
}

int girih_gpu_run(girih_gpu_ctx *c, int nt, float *ms_out) {
  if (!c) return fail(GIRIH_GPU_EINVAL, "null context");
  if (!c->uploaded) return fail(GIRIH_GPU_ESTATE, "run before upload");
  if (nt < 0) return fail(GIRIH_GPU_EINVAL, "nt must be >= 0");
  DeviceGuard dg(c->d.device);
  const int steps = 2 * ((nt + 1) / 2);  // for(it=0; it<nt; it+=2): two sweeps each
  if (!c->gexec || c->g_steps != steps || c->g_iu1 != c->iu1 || c->g_iu2 != c->iu2) {
    drop_graph(c);
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeRelaxed));
    int launches = 0, a = c->iu1, b = c->iu2;
    int e = issue_steps(c, steps, &launches, &a, &b);
    cudaError_t ce = cudaStreamEndCapture(c->st, &graph);
    if (e) {
      if (graph) cudaGraphDestroy(graph);
      return e;
    }
    if (ce != cudaSuccess) return fail(GIRIH_GPU_ECUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
    ce = cudaGraphInstantiate(&c->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
      c->gexec = nullptr;
      return fail(GIRIH_GPU_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
    }
    c->g_steps = steps;
    c->g_iu1 = c->iu1;
    c->g_iu2 = c->iu2;
    c->g_launches = launches;
    c->g_new_iu1 = a;
    c->g_new_iu2 = b;
    for (int k = 0; k < 4; k++) c->g_expect[k] = c->run_expect[k];
  }
  // kernels that report through the flag word: the double-float split, the TMA
  // waits, and every kernel of the checked build
  const bool df = GIRIH_CHECKED ||
                  (c->sched == GIRIH_SCHED_FUSED && (c->d.precision == GIRIH_FP64_DF || c->fcfg.box_w > 0));
  unsigned *range_flag = reinterpret_cast<unsigned *>(c->acc + 6);
  if (df) CK(cudaMemsetAsync(range_flag, 0, sizeof(unsigned), c->st));
  if (GIRIH_CHECKED)  // write counters start from zero (autotuner trials and looped batch runs also count)
    for (int k = 0; k < 4; k++)
      if (c->cov[k]) CK(cudaMemsetAsync(c->cov[k], 0, (size_t)c->g.elems * sizeof(unsigned), c->st));
  CK(cudaEventRecord(c->e0, c->st));
  if (steps > 0) CK(cudaGraphLaunch(c->gexec, c->st));
  CK(cudaEventRecord(c->e1, c->st));
  CK(cudaEventSynchronize(c->e1));
  CK(cudaGetLastError());
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, c->e0, c->e1));
  if (ms_out) *ms_out = ms;
  if (GIRIH_CHECKED && steps > 0)
    for (int k = 0; k < 4; k++)
      if (c->cov[k]) CK(launch_coverage_check(c->g, c->cov[k], (unsigned)c->g_expect[k], range_flag, c->st));
  if (df) {
    unsigned bad = 0;
    CK(cudaMemcpyAsync(&bad, range_flag, sizeof(bad), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    if (bad) {
      c->iu1 = c->g_new_iu1;
      c->iu2 = c->g_new_iu2;
      if (bad & kFlagBounds) return fail(GIRIH_GPU_EBOUNDS, "a kernel index left its array or shared block");
      if (bad & kFlagCoverage)
        return fail(GIRIH_GPU_ECOVERAGE, "a point was not written exactly as often as the schedule writes it");
      if (bad & 2u) return fail(GIRIH_GPU_ETIMEOUT, "a TMA plane copy did not complete within the wait bound");
      return fail(GIRIH_GPU_ERANGE, "a field value left the FP32 exponent range of the double-float fused kernel; "
                                    "use GIRIH_FP64 for this grid");
    }
  }
  c->iu1 = c->g_new_iu1;
  c->iu2 = c->g_new_iu2;
  c->last_launches = steps > 0 ? c->g_launches : 0;
  c->last_steps = steps;
  return 0;
}

int girih_gpu_download(girih_gpu_ctx *c, void *U1, void *U2) {
  if (!c) return fail(GIRIH_GPU_EINVAL, "null context");
  if (!c->uploaded) return fail(GIRIH_GPU_ESTATE, "download before upload");
  DeviceGuard dg(c->d.device);
  int e;
  if (U1 && (e = download_field(c, c->f[c->iu1], U1))) return e;
  if (U1 && U2) CK(cudaStreamSynchronize(c->st));  // the staging buffer serves both arrays
  if (U2 && (e = download_field(c, c->f[c->iu2], U2))) return e;
  CK(cudaStreamSynchronize(c->st));
  return 0;
}

int girih_gpu_download_roc2(girih_gpu_ctx *c, void *U3) {
  if (!c || !U3) return fail(GIRIH_GPU_EINVAL, "null argument");
  if (c->g.to != 2) return fail(GIRIH_GPU_EINVAL, "operator has no roc2 array");
  if (!c->uploaded) return fail(GIRIH_GPU_ESTATE, "download before upload");
  DeviceGuard dg(c->d.device);
  int e = download_field(c, c->roc2, U3);
  if (e) return e;
  CK(cudaStreamSynchronize(c->st));
  return 0;
}

static int read_norms(girih_gpu_ctx *c, double out[4]) {
  double h[4];
  CK(cudaMemcpyAsync(h, c->acc, 32, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  for (int i = 0; i < 4; i++) out[i] = h[i];
  return 0;
}

int girih_gpu_error_norms(girih_gpu_ctx *c, const void *ref_U1, double out[4]) {
  if (!c || !ref_U1 || !out) return fail(GIRIH_GPU_EINVAL, "null argument");
  if (!c->uploaded) return fail(GIRIH_GPU_ESTATE, "norms before upload");
  DeviceGuard dg(c->d.device);
  size_t n = host_array_elems(c);
  int e = ensure_staging(c, n * 8);
  if (e) return e;
  CK(cudaMemcpyAsync(c->staging, ref_U1, n * c->hsz, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemsetAsync(c->acc, 0, 32, c->st));
  const void *a = c->f[c->iu1];
  if (c->tsz == 8 && c->hsz == 8)
    CK(launch_norms<double, double>(c->g, (const double *)a, (const double *)c->staging, c->g, nullptr, c->acc, c->st));
  else if (c->tsz == 8)
    CK(launch_norms<double, float>(c->g, (const double *)a, (const float *)c->staging, c->g, nullptr, c->acc, c->st));
  else if (c->hsz == 8)
    CK(launch_norms<float, double>(c->g, (const float *)a, (const double *)c->staging, c->g, nullptr, c->acc, c->st));
  else
    CK(launch_norms<float, float>(c->g, (const float *)a, (const float *)c->staging, c->g, nullptr, c->acc, c->st));
  return read_norms(c, out);
}

int girih_gpu_compare(girih_gpu_ctx *a, girih_gpu_ctx *b, double out[4]) {
  if (!a || !b || !out) return fail(GIRIH_GPU_EINVAL, "null argument");
  if (!a->uploaded || !b->uploaded) return fail(GIRIH_GPU_ESTATE, "compare before upload");
  if (a->d.device != b->d.device || a->g.op != b->g.op || a->g.nx != b->g.nx || a->g.ny != b->g.ny ||
      a->g.nz != b->g.nz)
    return fail(GIRIH_GPU_EINVAL, "contexts differ in device, operator or grid");
  DeviceGuard dg(a->d.device);
  CK(cudaStreamSynchronize(b->st));
  CK(cudaMemsetAsync(a->acc, 0, 32, a->st));
  const void *pa = a->f[a->iu1], *pb = b->f[b->iu1];
  if (a->tsz == 8 && b->tsz == 8)
    CK(launch_norms<double, double>(a->g, (const double *)pa, nullptr, b->g, (const double *)pb, a->acc, a->st));
  else if (a->tsz == 4 && b->tsz == 8)
    CK(launch_norms<float, double>(a->g, (const float *)pa, nullptr, b->g, (const double *)pb, a->acc, a->st));
  else if (a->tsz == 8)
    CK(launch_norms<double, float>(a->g, (const double *)pa, nullptr, b->g, (const float *)pb, a->acc, a->st));
  else
    CK(launch_norms<float, float>(a->g, (const float *)pa, nullptr, b->g, (const float *)pb, a->acc, a->st));
  return read_norms(a, out);
}

int girih_gpu_autotune(girih_gpu_ctx *c, int trial_steps, girih_gpu_info_t *chosen) {
  if (!c) return fail(GIRIH_GPU_EINVAL, "null context");
  if (!c->uploaded) return fail(GIRIH_GPU_ESTATE, "autotune before upload");
  DeviceGuard dg(c->d.device);
  const Geom &g = c->g;
  const int prec = c->d.precision;
  std::vector<TuneChoice> cands;
  const bool explicit_cfg = c->d.fusion_depth != 0 || c->d.block_x != 0 || c->d.block_y != 0;
  if (c->d.schedule == GIRIH_SCHED_AUTO || (c->d.schedule == GIRIH_SCHED_PLAIN))
    cands.push_back({GIRIH_SCHED_PLAIN, 0, 1});
  if (c->d.schedule != GIRIH_SCHED_PLAIN && !c->d.exact && fused_supported(g, prec) && c->halos_equal) {
    for (int v = 0; v < FV_COUNT; v++)
      for (int t = 1; t <= fused_max_depth(g, prec); t++) {
        FusedConfig fc = make_fused_config(g, prec, t, v);
        if (!fc.depth) continue;
        if (explicit_cfg && ((c->d.fusion_depth && t != c->d.fusion_depth) || (c->d.block_x && fc.bx != c->d.block_x) ||
                             (c->d.block_y && fc.by != c->d.block_y)))
          continue;
        cands.push_back({GIRIH_SCHED_FUSED, v, t});
      }
  }
  if (cands.empty()) return girih_gpu_info(c, chosen);
  int e = 0;
  if (cands.size() > 1 || cands[0].sched == GIRIH_SCHED_FUSED) {
    if ((e = ensure_fused_buffers(c))) return e;
    for (int b = 2; b < 4; b++)  // spare buffers carry the fixed halo
      CK(cudaMemcpyAsync(c->f[b], c->f[c->iu2], (size_t)g.elems * c->tsz, cudaMemcpyDeviceToDevice, c->st));
  }
  // back up the state so that tuning leaves the grid unchanged; the backup is
  // freed on every return, early error returns included
  const size_t fb = (size_t)g.elems * c->tsz;
  struct Backup {
    girih_gpu_ctx *c;
    size_t fb;
    void *p[2];
    ~Backup() {
      for (void *q : p)
        if (q) {
          cudaFree(q);
          c->dev_bytes -= (double)fb;
        }
    }
  } backup{c, fb, {nullptr, nullptr}};
  void **bk = backup.p;
  if ((e = dev_alloc(c, &bk[0], fb)) || (e = dev_alloc(c, &bk[1], fb))) return e;
  CK(cudaMemcpyAsync(bk[0], c->f[c->iu1], fb, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(bk[1], c->f[c->iu2], fb, cudaMemcpyDeviceToDevice, c->st));
  const int steps = trial_steps > 0 ? 2 * ((trial_steps + 1) / 2) : (g.r == 4 ? 8 : 24);
  double best = 1e300;
  TuneChoice best_c = cands[0];
  drop_graph(c);
  for (const TuneChoice &tc : cands) {
    c->sched = tc.sched;
    c->fcfg = tc.sched == GIRIH_SCHED_FUSED ? make_fused_config(g, prec, tc.depth, tc.variant) : FusedConfig{};
    float ms_min = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
      int a = c->iu1, b = c->iu2, launches = 0;
      CK(cudaEventRecord(c->e0, c->st));
      if ((e = issue_steps(c, steps, &launches, &a, &b))) return e;
      CK(cudaEventRecord(c->e1, c->st));
      CK(cudaEventSynchronize(c->e1));
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, c->e0, c->e1));
      if (rep > 0) ms_min = std::min(ms_min, ms);  // first repetition warms up
      c->iu1 = a;
      c->iu2 = b;
    }
    if (ms_min < best) {
      best = ms_min;
      best_c = tc;
    }
  }
  // restore the state into the first two buffers
  CK(cudaMemcpyAsync(c->f[0], bk[0], fb, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(c->f[1], bk[1], fb, cudaMemcpyDeviceToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->iu1 = 0;
  c->iu2 = 1;
  c->sched = best_c.sched;
  c->fcfg = best_c.sched == GIRIH_SCHED_FUSED ? make_fused_config(g, prec, best_c.depth, best_c.variant) : FusedConfig{};
  if (!explicit_cfg) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache[std::make_tuple(g.op, prec, size_class(g))] = best_c;
  }
  return girih_gpu_info(c, chosen);
}

int girih_gpu_set_source(girih_gpu_ctx *c, const int pt[3], const double *source, int n) {
  if (!c) return fail(GIRIH_GPU_EINVAL, "null context");
  if (n < 0) return fail(GIRIH_GPU_EINVAL, "negative source count");
  DeviceGuard dg(c->d.device);
  drop_graph(c);  // the captured launches carry the source arguments
  if (!source || n == 0) {
    c->src_n = 0;
    c->src_off = -1;
    return 0;
  }
  if (!pt) return fail(GIRIH_GPU_EINVAL, "null source point");
  const Geom &g = c->g;
  const int n3[3] = {g.nx, g.ny, g.nz};
  for (int a = 0; a < 3; a++)
    if (pt[a] < g.r || pt[a] >= n3[a] + g.r) return fail(GIRIH_GPU_EINVAL, "source point outside the interior");
  if (n > c->d_src_cap) {
    if (c->d_src) {
      cudaFree(c->d_src);
      c->dev_bytes -= 8.0 * c->d_src_cap;
      c->d_src = nullptr;
      c->d_src_cap = 0;
    }
    int e = dev_alloc(c, (void **)&c->d_src, (size_t)n * sizeof(double));
    if (e) return e;
    c->d_src_cap = n;
  }
  CK(cudaMemcpyAsync(c->d_src, source, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->src_off = g.at(pt[0], pt[1], pt[2]);  // array indices include the halo
  c->src_n = n;
  return 0;
}

int girih_gpu_info(girih_gpu_ctx *c, girih_gpu_info_t *info) {
  if (!c || !info) return fail(GIRIH_GPU_EINVAL, "null argument");
  std::memset(info, 0, sizeof(*info));
  const Geom &g = c->g;
  info->precision = c->d.precision;
  info->schedule = c->sched;
  info->fusion_depth = c->sched == GIRIH_SCHED_FUSED ? c->fcfg.depth : 1;
  info->block_x = c->sched == GIRIH_SCHED_FUSED ? c->fcfg.bx : 0;
  info->block_y = c->sched == GIRIH_SCHED_FUSED ? c->fcfg.by : 0;
  info->launches_last_run = c->last_launches;
  info->steps_last_run = c->last_steps;
  // compulsory traffic of one step: read v (+ u, roc2 for time order 2, + coefficient
  // arrays), write u
  double fb = c->tsz, cb = c->bf16coef ? 2.0 : c->tsz;
  double bytes = 2 * fb;
  if (g.to == 2) bytes += 2 * fb;
  if (g.var) bytes += g.nc * cb;
  info->bytes_per_lup = bytes;
  info->device_bytes = c->dev_bytes;
  std::snprintf(info->kernel_name, sizeof(info->kernel_name), "%s",
                c->sched == GIRIH_SCHED_FUSED ? fused_kernel_name(g.op, c->d.precision, c->fcfg) : plain_kernel_name(g.op));
  return 0;
}

}  // extern "C"
