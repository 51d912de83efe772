// Time-fused stepping for callers that cannot allocate device memory.
//
// girih_gpu_run() keeps two spare state buffers per context, allocated with
// cudaMalloc when the context is created.  Some callers cannot do that: a host
// application that owns the device's memory through its own pool (a cudaMalloc
// behind its back escapes its accounting, or fails under its memory cap), or a
// code path that must not take the implicit device synchronisation that
// cudaMalloc/cudaFree can cause.  girih_gpu_fused_run_noalloc() serves them: the
// caller passes its own device arrays, and the two spare buffers live in the
// file-scope array below instead.
//
// The array is GIRIH_NOALLOC_SCRATCH_BYTES (64 MiB) of static device memory;
// every GPU that loads this library holds it until the process exits.  All
// calls share it and it keeps the last call's contents, so calls whose work
// overlaps on the GPU (different streams, different host threads) race on it:
// serialise them.  Each call re-initialises what it reads (the halo flag is
// cleared and both spare buffers are overwritten from U2 before the first
// pass).  The first call in a device context looks up the array's device
// address (set-up); later calls in the same context reuse it.
#include <mutex>
#include <string>

#include "fused.cuh"
#include "internal.cuh"

namespace girih {
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[GIRIH_NOALLOC_SCRATCH_BYTES];

constexpr size_t kFlagBytes = 256;  // halo-equality flag, then the two spare buffers
constexpr int kMaxDevices = 64;

std::mutex g_setup_mutex;
struct ScratchSlot {
  void *addr;
  unsigned long long ctx_id;  // device context the address belongs to
};
ScratchSlot g_scratch[kMaxDevices] = {};

// Unique id of the calling thread's current device context (driver API
// cuCtxGetCurrent / cuCtxGetId through the runtime's entry-point query, so the
// library needs no link against libcuda); 0 where unavailable.
unsigned long long current_context_id() {
  using GetCurrent = int (*)(void **);
  using GetId = int (*)(void *, unsigned long long *);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(p);
  });
  void *ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == 0 && ctx && get_id(ctx, &id) == 0) return id;
  return 0;
}

// Device address of the scratch array on the current device (which must be
// `dev`).  In host code the array's name is only a host-side stand-in, so the
// address comes from cudaGetSymbolAddress, looked up once per device context:
// again after a cudaDeviceReset(), which reloads the module and may move the
// array, and on every call where the context id cannot be read.
int scratch_address(int dev, unsigned char **out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  // (a context not yet bound reads as id 0: the lookup below binds it, and the
  // next call records its id)
  const unsigned long long ctx = current_context_id();
  ScratchSlot &slot = g_scratch[dev];
  if (!slot.addr || ctx == 0 || slot.ctx_id != ctx) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      slot.addr = nullptr;
      set_error(std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
      return GIRIH_GPU_ECUDA;
    }
    slot.addr = p;
    slot.ctx_id = ctx;
  }
  *out = static_cast<unsigned char *>(slot.addr);
  return 0;
}

// Geometry of arrays kept in the reference layout itself (x pitch ldomain_shape[0]).
Geom reference_layout_geom(const girih_gpu_desc *d) {
  Geom g{};
  op_info(d->target_kernel, &g.r, &g.to, &g.nc, &g.var);
  g.op = d->target_kernel;
  g.nx = d->stencil_shape[0];
  g.ny = d->stencil_shape[1];
  g.nz = d->stencil_shape[2];
  g.nnx = g.nx + 2 * g.r;
  g.nny = g.ny + 2 * g.r;
  g.nnz = g.nz + 2 * g.r;
  g.hpx = d->ldomain_shape[0];
  g.ox = 0;
  g.px = d->ldomain_shape[0];
  g.plane = (int64_t)g.px * g.nny;
  g.elems = g.plane * g.nnz;
  return g;
}

int fail_na(int code, const std::string &msg) {
  set_error(msg);
  return code;
}

#define NA_CK(...)                                                            \
  do {                                                                        \
    cudaError_t e_ = (__VA_ARGS__);                                           \
    if (e_ != cudaSuccess) {                                                  \
      set_error(std::string(#__VA_ARGS__) + ": " + cudaGetErrorString(e_));   \
      return GIRIH_GPU_ECUDA;                                                 \
    }                                                                         \
  } while (0)

}  // namespace
}  // namespace girih

using namespace girih;

extern "C" int girih_gpu_fused_run_noalloc(const girih_gpu_desc *d, void *U1, void *U2, const void *U3,
                                           const double *coefs, int nt, void *stream) {
  if (!d || !U1 || !U2 || !coefs) return fail_na(GIRIH_GPU_EINVAL, "null argument");
  int r, to, nc, var;
  if (op_info(d->target_kernel, &r, &to, &nc, &var) || var ||
      (d->target_kernel != 0 && d->target_kernel != 1 && d->target_kernel != 8))
    return fail_na(GIRIH_GPU_EUNSUPPORTED,
                   "the no-allocation entry point runs operators 0, 1 and 8, not " + std::to_string(d->target_kernel));
  const int nx = d->stencil_shape[0], ny = d->stencil_shape[1], nz = d->stencil_shape[2];
  if (nx < 1 || ny < 1 || nz < 1 || d->ldomain_shape[0] < nx + 2 * r || d->ldomain_shape[1] != ny + 2 * r ||
      d->ldomain_shape[2] != nz + 2 * r)
    return fail_na(GIRIH_GPU_EINVAL, "ldomain_shape must be (>= nx+2r, ny+2r, nz+2r)");
  if (d->precision < GIRIH_FP64 || d->precision > GIRIH_MIXED) return fail_na(GIRIH_GPU_EINVAL, "bad precision");
  if (to == 2 && !U3) return fail_na(GIRIH_GPU_EINVAL, "time-order-2 operator needs U3 (roc2)");
  if (nt < 0) return fail_na(GIRIH_GPU_EINVAL, "nt must be >= 0");
  if (d->device < 0 || d->device >= kMaxDevices) return fail_na(GIRIH_GPU_EINVAL, "device ordinal out of range");

  const int tsz = d->precision == GIRIH_FP64 ? 8 : 4;
  // the radius-1 fused kernels move x pairs as one vector: rows must start on
  // a pair boundary and the arrays on a 16-byte boundary
  if (d->ldomain_shape[0] % 2 != 0)
    return fail_na(GIRIH_GPU_EINVAL, "ldomain_shape[0] (x pitch) must be even for the no-allocation entry point");
  for (const void *ptr : {(const void *)U1, (const void *)U2, U3})
    if (ptr && (reinterpret_cast<uintptr_t>(ptr) & 15u))
      return fail_na(GIRIH_GPU_EINVAL, "device arrays must be 16-byte aligned");
  const Geom g = reference_layout_geom(d);
  const size_t state_bytes = (size_t)g.elems * tsz;
  const size_t spare_bytes = (state_bytes + 255) / 256 * 256;
  if (kFlagBytes + 2 * spare_bytes > (size_t)GIRIH_NOALLOC_SCRATCH_BYTES)
    return fail_na(GIRIH_GPU_EINVAL,
                   "grid too large for the no-allocation entry point: two state arrays of " +
                       std::to_string(state_bytes) + " bytes exceed its " +
                       std::to_string((unsigned long long)GIRIH_NOALLOC_SCRATCH_BYTES) + "-byte scratch");
  FusedConfig cfg = choose_fused_config(g, d->precision, d->fusion_depth, d->block_x, d->block_y);
  if (!cfg.depth) return fail_na(GIRIH_GPU_EUNSUPPORTED, "requested fused tile/depth is not provided");
  if (cfg.box_w)  // TMA tiles read through tensor maps that a context encodes and keeps per array
    return fail_na(GIRIH_GPU_EUNSUPPORTED,
                   "the requested tile is a TMA-staged variant, which only the context entry points run");

  int prev_dev = -1;
  cudaGetDevice(&prev_dev);
  if (prev_dev != d->device) NA_CK(cudaSetDevice(d->device));
  struct Restore {
    int dev;
    ~Restore() {
      int cur = -1;
      cudaGetDevice(&cur);
      if (dev >= 0 && cur != dev) cudaSetDevice(dev);
    }
  } restore{prev_dev};

  unsigned char *scratch = nullptr;
  int e = scratch_address(d->device, &scratch);
  if (e) return e;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned int *flag = reinterpret_cast<unsigned int *>(scratch);
  void *spare0 = scratch + kFlagBytes;
  void *spare1 = scratch + kFlagBytes + spare_bytes;

  // the fused schedule needs U1 and U2 to carry the same fixed halo
  NA_CK(cudaMemsetAsync(flag, 0, sizeof(unsigned int), st));
  NA_CK(launch_halo_equal(g, U1, U2, tsz, flag, st));
  unsigned int h = 1;
  NA_CK(cudaMemcpyAsync(&h, flag, sizeof(h), cudaMemcpyDeviceToHost, st));
  NA_CK(cudaStreamSynchronize(st));
  if (h != 0) return fail_na(GIRIH_GPU_EUNSUPPORTED, "U1 and U2 halos differ; the fused schedule needs them equal");

  // spare buffers start as copies of U2 so that their halos hold the fixed values
  NA_CK(cudaMemcpyAsync(spare0, U2, state_bytes, cudaMemcpyDeviceToDevice, st));
  NA_CK(cudaMemcpyAsync(spare1, U2, state_bytes, cudaMemcpyDeviceToDevice, st));

  void *buf[4] = {U1, U2, spare0, spare1};
  int iu1 = 0, iu2 = 1;
  const int steps = 2 * ((nt + 1) / 2);
  int left = steps;
  while (left > 0) {
    const int T = left < cfg.depth ? left : cfg.depth;
    int spare[2], n = 0;
    for (int b = 0; b < 4 && n < 2; b++)
      if (b != iu1 && b != iu2) spare[n++] = b;
    FusedLaunch L{};
    L.prev = buf[iu1];
    L.cur = buf[iu2];
    L.out_prev = buf[spare[0]];
    L.out_cur = buf[spare[1]];
    L.roc2 = U3;
    L.steps = T;
    L.write_prev = (to == 2 || left == T) ? 1 : 0;
    for (int m = 0; m < 5; m++) L.cc[m] = m <= r ? coefs[m] : 0.0;
    NA_CK(launch_fused(g, tsz, d->precision, cfg, L, st));
    iu1 = spare[0];
    iu2 = spare[1];
    left -= T;
  }
  // The passes alternate between the buffer pairs (0, 1) and (2, 3), so the
  // final states (U1 = state steps-1, U2 = state steps) are either already in
  // the caller's arrays (even pass count) or in the two spare buffers (odd).
  // In the latter case copy them back row by row: nnx columns per row, so the
  // caller's x padding [nnx, ldomain_shape[0]) keeps its own values (the
  // spares' padding came from U2).
  if (iu1 != 0) {
    const size_t row = (size_t)g.nnx * tsz, pitch = (size_t)g.hpx * tsz, rows = (size_t)g.nny * g.nnz;
    NA_CK(cudaMemcpy2DAsync(U1, pitch, buf[iu1], pitch, row, rows, cudaMemcpyDeviceToDevice, st));
    NA_CK(cudaMemcpy2DAsync(U2, pitch, buf[iu2], pitch, row, rows, cudaMemcpyDeviceToDevice, st));
  }
  NA_CK(cudaStreamSynchronize(st));
  NA_CK(cudaGetLastError());
  return 0;
}
