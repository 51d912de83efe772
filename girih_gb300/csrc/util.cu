// Data movement and reduction kernels: layout conversion between the
// reference's host layout and the device layout, BF16 quantisation, seeded
// initialisation and the FP64 error norms used by verification.
#include "check.cuh"
#include "df64.cuh"
#include "internal.cuh"

namespace girih {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// Same value as go_seeded_value() in the CPU oracle: every operation rounded on
// its own, so host and device agree bit for bit.
__device__ __forceinline__ double seeded_value(uint64_t key, uint64_t idx, double lo, double hi) {
  uint64_t h = splitmix64(key + idx);
  double u = __dmul_rn(__ull2double_rn(h >> 11), 0x1.0p-53);
  double d = __dsub_rn(hi, lo);
  return __dadd_rn(lo, __dmul_rn(d, u));
}

uint64_t host_splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

int grid_for(int64_t n) {
  int64_t b = (n + kThreads - 1) / kThreads;
  return (int)(b < 152 * 32 ? (b < 1 ? 1 : b) : 152 * 32);
}

// Layout conversion, one (k, j) row per CTA iteration: the row's nnx elements
// are contiguous on both sides, so reads and writes coalesce (also when one
// side is pinned host memory that the kernel reads or writes directly).
template <class Tin, class Tout>
__global__ void to_device_layout(Geom g, const Tin *__restrict__ src, Tout *__restrict__ dst) {
  const int64_t rows = (int64_t)g.nny * g.nnz;
  for (int64_t row = blockIdx.x; row < rows; row += gridDim.x) {
    const Tin *s = src + row * g.hpx;
    Tout *d = dst + row * g.px + g.ox;
    for (int i = threadIdx.x; i < g.nnx; i += blockDim.x) d[i] = static_cast<Tout>(s[i]);
  }
}

template <class Tin, class Tout>
__global__ void to_host_layout(Geom g, const Tin *__restrict__ src, Tout *__restrict__ dst) {
  const int64_t rows = (int64_t)g.nny * g.nnz;
  for (int64_t row = blockIdx.x; row < rows; row += gridDim.x) {
    const Tin *s = src + row * g.px + g.ox;
    Tout *d = dst + row * g.hpx;
    for (int i = threadIdx.x; i < g.nnx; i += blockDim.x) d[i] = static_cast<Tout>(s[i]);
  }
}

int rows_grid(const Geom &g) {
  const int64_t rows = (int64_t)g.nny * g.nnz;
  return (int)(rows < 152 * 16 ? rows : 152 * 16);
}

__device__ __forceinline__ double nan_max(double a, double b) { return (a > b || a != a) ? a : b; }

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long *acc, double v) {
  atomicMax(acc, (unsigned long long)__double_as_longlong(v));
}

template <class Tin>
__global__ void maxabs_kernel(Geom g, const Tin *__restrict__ src, unsigned long long *acc) {
  const int64_t n = (int64_t)g.nnx * g.nny * g.nnz;
  double m = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(t % g.nnx);
    int64_t row = t / g.nnx;
    m = nan_max(m, fabs((double)src[row * g.hpx + i]));
  }
  for (int o = 16; o > 0; o >>= 1) m = nan_max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomic_max_nonneg(acc, m);
}

template <class Tin>
__global__ void quantize_kernel(Geom g, const Tin *__restrict__ src, __nv_bfloat16 *dst,
                                const float *scale) {
  const int64_t n = (int64_t)g.nnx * g.nny * g.nnz;
  const double s = (double)scale[0];
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(t % g.nnx);
    int64_t row = t / g.nnx;
    dst[row * g.px + g.ox + i] = __double2bfloat16((double)src[row * g.hpx + i] / s);
  }
}

// acc = {max|a-b| (as bits), max|b| (as bits), sum (a-b)^2, sum b^2} over the interior.
template <class Ta, class Tb>
__global__ void norms_kernel(Geom g, const Ta *__restrict__ a, const Tb *__restrict__ bh,
                             Geom gb, const Tb *__restrict__ bd, double *acc) {
  const int r = g.r;
  const int64_t n = (int64_t)g.nx * g.ny * g.nz;
  double me = 0, mb = 0, se = 0, sb = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(t % g.nx) + r;
    int64_t rest = t / g.nx;
    int j = (int)(rest % g.ny) + r;
    int k = (int)(rest / g.ny) + r;
    double av = (double)a[g.at(i, j, k)];
    double bv = bh ? (double)bh[((int64_t)k * g.nny + j) * g.hpx + i] : (double)bd[gb.at(i, j, k)];
    double e = fabs(av - bv), bb = fabs(bv);
    me = nan_max(me, e);
    mb = nan_max(mb, bb);
    se += e * e;
    sb += bb * bb;
  }
  for (int o = 16; o > 0; o >>= 1) {
    me = nan_max(me, __shfl_xor_sync(0xffffffffu, me, o));
    mb = nan_max(mb, __shfl_xor_sync(0xffffffffu, mb, o));
    se += __shfl_xor_sync(0xffffffffu, se, o);
    sb += __shfl_xor_sync(0xffffffffu, sb, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomic_max_nonneg(reinterpret_cast<unsigned long long *>(acc + 0), me);
    atomic_max_nonneg(reinterpret_cast<unsigned long long *>(acc + 1), mb);
    atomicAdd(acc + 2, se);
    atomicAdd(acc + 3, sb);
  }
}

template <class T>
__global__ void seeded_kernel(Geom g, uint64_t key, double lo, double hi, int round_f32, T *dd,
                              double *dh) {
  const int64_t n = (int64_t)g.nnx * g.nny * g.nnz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(t % g.nnx);
    int64_t row = t / g.nnx;
    double v = seeded_value(key, (uint64_t)t, lo, hi);
    if (round_f32) v = (double)__double2float_rn(v);
    if (dd) dd[row * g.px + g.ox + i] = static_cast<T>(v);
    if (dh) dh[row * g.hpx + i] = v;
  }
}

template <class W>
__global__ void halo_equal_kernel(Geom g, const W *__restrict__ a, const W *__restrict__ b,
                                  unsigned int *flag) {
  const int64_t n = (int64_t)g.nnx * g.nny * g.nnz;
  const int r = g.r;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(t % g.nnx);
    int64_t rest = t / g.nnx;
    int j = (int)(rest % g.nny);
    int k = (int)(rest / g.nny);
    bool halo = i < r || i >= g.nnx - r || j < r || j >= g.nny - r || k < r || k >= g.nnz - r;
    if (halo) {
      int64_t c = g.at(i, j, k);
      if (a[c] != b[c]) atomicOr(flag, 1u);
    }
  }
}


// FP64 -> pairs, two elements per thread (the element count of a device field
// is even: the row pitch is a multiple of 16 doubles).
__global__ void df_split_kernel(int64_t n2, const double2 *__restrict__ in, float4 *o0, float4 *o1, float4 *o2,
                                unsigned *flag) {
  unsigned bad = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n2; t += (int64_t)gridDim.x * blockDim.x) {
    const double2 d = in[t];
    const Df64 a = df_split(d.x, bad), b = df_split(d.y, bad);
    const float4 v = make_float4(a.hi, a.lo, b.hi, b.lo);
    o0[t] = v;
    if (o1) o1[t] = v;
    if (o2) o2[t] = v;
  }
  if (bad) atomicOr(flag, 1u);
}

// pairs -> FP64 at the interior points (x fastest; one row segment per thread group)
__global__ void df_join_kernel(Geom g, const Df64 *__restrict__ in, double *__restrict__ out) {
  const int64_t n = (int64_t)g.nx * g.ny * g.nz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.nx);
    const int64_t row = t / g.nx;
    const int j = (int)(row % g.ny), k = (int)(row / g.ny);
    const int64_t at = g.at(g.r + i, g.r + j, g.r + k);
    const float2 v = __ldg(reinterpret_cast<const float2 *>(in + at));
    out[at] = df_to_double(Df64(v.x, v.y));
  }
}
// Checked build: every interior point written `expect` times, nothing else
// written at all; the counters are cleared.
__global__ void coverage_check_kernel(Geom g, unsigned *cov, unsigned expect, unsigned *flag) {
  const int64_t n = g.elems;
  unsigned bad = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = t / g.plane, rem = t - k * g.plane;
    const int64_t j = rem / g.px, i = rem - j * g.px - g.ox;  // i: index along x with the halo at 0..r-1
    const bool interior = i >= g.r && i < g.nnx - g.r && j >= g.r && j < g.nny - g.r && k >= g.r && k < g.nnz - g.r;
    if (cov[t] != (interior ? expect : 0u)) bad = 1;
    cov[t] = 0;
  }
  if (bad) atomicOr(flag, kFlagCoverage);
}
}  // namespace

cudaError_t launch_coverage_check(const Geom &g, unsigned *cov, unsigned expect, unsigned *flag, cudaStream_t s) {
  coverage_check_kernel<<<grid_for(g.elems), kThreads, 0, s>>>(g, cov, expect, flag);
  return cudaGetLastError();
}

template <class Tin, class Tout>
cudaError_t launch_to_device_layout(const Geom &g, const Tin *src, Tout *dst, cudaStream_t s) {
  to_device_layout<Tin, Tout><<<rows_grid(g), kThreads, 0, s>>>(g, src, dst);
  return cudaGetLastError();
}
template <class Tin, class Tout>
cudaError_t launch_to_host_layout(const Geom &g, const Tin *src, Tout *dst, cudaStream_t s) {
  to_host_layout<Tin, Tout><<<rows_grid(g), kThreads, 0, s>>>(g, src, dst);
  return cudaGetLastError();
}
template <class Tin>
cudaError_t launch_maxabs(const Geom &g, const Tin *src, unsigned long long *acc, cudaStream_t s) {
  maxabs_kernel<Tin><<<grid_for((int64_t)g.nnx * g.nny * g.nnz), kThreads, 0, s>>>(g, src, acc);
  return cudaGetLastError();
}
template <class Tin>
cudaError_t launch_quantize_bf16(const Geom &g, const Tin *src, __nv_bfloat16 *dst,
                                 const float *scale, cudaStream_t s) {
  quantize_kernel<Tin><<<grid_for((int64_t)g.nnx * g.nny * g.nnz), kThreads, 0, s>>>(g, src, dst, scale);
  return cudaGetLastError();
}
template <class Ta, class Tb>
cudaError_t launch_norms(const Geom &g, const Ta *a, const Tb *bh, const Geom &gb, const Tb *bd,
                         double *acc, cudaStream_t s) {
  norms_kernel<Ta, Tb><<<grid_for((int64_t)g.nx * g.ny * g.nz), kThreads, 0, s>>>(g, a, bh, gb, bd, acc);
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_seeded(const Geom &g, uint64_t seed, uint32_t stream, double lo, double hi,
                          int round_f32, T *dd, double *dh, cudaStream_t s) {
  uint64_t key = host_splitmix64(seed ^ ((uint64_t)stream * 0xD1B54A32D192ED03ULL));
  seeded_kernel<T><<<grid_for((int64_t)g.nnx * g.nny * g.nnz), kThreads, 0, s>>>(g, key, lo, hi, round_f32,
                                                                                 dd, dh);
  return cudaGetLastError();
}
cudaError_t launch_halo_equal(const Geom &g, const void *a, const void *b, int tsz,
                              unsigned int *flag, cudaStream_t s) {
  int grid = grid_for((int64_t)g.nnx * g.nny * g.nnz);
  if (tsz == 8)
    halo_equal_kernel<unsigned long long><<<grid, kThreads, 0, s>>>(
        g, static_cast<const unsigned long long *>(a), static_cast<const unsigned long long *>(b), flag);
  else
    halo_equal_kernel<unsigned int><<<grid, kThreads, 0, s>>>(
        g, static_cast<const unsigned int *>(a), static_cast<const unsigned int *>(b), flag);
  return cudaGetLastError();
}

template cudaError_t launch_to_device_layout<double, double>(const Geom &, const double *, double *, cudaStream_t);
template cudaError_t launch_to_device_layout<double, float>(const Geom &, const double *, float *, cudaStream_t);
template cudaError_t launch_to_device_layout<float, float>(const Geom &, const float *, float *, cudaStream_t);
template cudaError_t launch_to_device_layout<float, double>(const Geom &, const float *, double *, cudaStream_t);
template cudaError_t launch_to_host_layout<double, double>(const Geom &, const double *, double *, cudaStream_t);
template cudaError_t launch_to_host_layout<float, double>(const Geom &, const float *, double *, cudaStream_t);
template cudaError_t launch_to_host_layout<float, float>(const Geom &, const float *, float *, cudaStream_t);
template cudaError_t launch_to_host_layout<double, float>(const Geom &, const double *, float *, cudaStream_t);
template cudaError_t launch_norms<double, double>(const Geom &, const double *, const double *, const Geom &, const double *, double *, cudaStream_t);
template cudaError_t launch_norms<float, double>(const Geom &, const float *, const double *, const Geom &, const double *, double *, cudaStream_t);
template cudaError_t launch_norms<double, float>(const Geom &, const double *, const float *, const Geom &, const float *, double *, cudaStream_t);
template cudaError_t launch_norms<float, float>(const Geom &, const float *, const float *, const Geom &, const float *, double *, cudaStream_t);
template cudaError_t launch_maxabs<double>(const Geom &, const double *, unsigned long long *, cudaStream_t);
template cudaError_t launch_maxabs<float>(const Geom &, const float *, unsigned long long *, cudaStream_t);
template cudaError_t launch_quantize_bf16<double>(const Geom &, const double *, __nv_bfloat16 *, const float *, cudaStream_t);
template cudaError_t launch_quantize_bf16<float>(const Geom &, const float *, __nv_bfloat16 *, const float *, cudaStream_t);
template cudaError_t launch_seeded<double>(const Geom &, uint64_t, uint32_t, double, double, int, double *, double *, cudaStream_t);
template cudaError_t launch_seeded<float>(const Geom &, uint64_t, uint32_t, double, double, int, float *, double *, cudaStream_t);

cudaError_t launch_df_split(const Geom &g, const double *in, void *out0, void *out1, void *out2, unsigned *flag,
                            cudaStream_t s) {
  const int64_t n2 = g.elems / 2;
  df_split_kernel<<<grid_for(n2), kThreads, 0, s>>>(n2, reinterpret_cast<const double2 *>(in),
                                                    static_cast<float4 *>(out0), static_cast<float4 *>(out1),
                                                    static_cast<float4 *>(out2), flag);
  return cudaGetLastError();
}

cudaError_t launch_df_join(const Geom &g, const void *in, double *out, cudaStream_t s) {
  df_join_kernel<<<grid_for((int64_t)g.nx * g.ny * g.nz), kThreads, 0, s>>>(g, static_cast<const Df64 *>(in), out);
  return cudaGetLastError();
}

}  // namespace girih
