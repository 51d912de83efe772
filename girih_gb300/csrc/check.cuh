// Bounds and write-coverage checks of the checked build.
//
// Compiled with GIRIH_CHECK (girih_gb300/build.py --checked, which links
// libgirih_gpu_check.so), every kernel tests each global-memory access range
// against the extent of the array it addresses and each shared-memory block it
// reads or writes against the CTA's shared allocation; an access outside is
// skipped (a load yields zero) and sets kFlagBounds in the run's error word,
// which girih_gpu_run() returns as GIRIH_GPU_EBOUNDS.  Every store of a new
// state value also counts one write of that point into a per-buffer counter
// array, which the run checks afterwards: each interior point of a buffer must
// have been written exactly as many times as the schedule wrote the buffer, and
// no halo or padding point at all (GIRIH_GPU_ECOVERAGE otherwise).
// Without GIRIH_CHECK every test is a compile-time `true` and costs nothing.
#pragma once
#include <cstdint>

#ifdef GIRIH_CHECK
#define GIRIH_CHECKED 1
#else
#define GIRIH_CHECKED 0
#endif

namespace girih {

constexpr unsigned kFlagBounds = 4u;    // an index left its array or shared block
constexpr unsigned kFlagCoverage = 8u;  // a point was written other than once per step

// [off, off + n) inside [0, extent) elements of one array
__device__ __forceinline__ bool in_array(int64_t off, int64_t n, int64_t extent, unsigned *flag) {
#if GIRIH_CHECKED
  if (off >= 0 && off + n <= extent) return true;
  if (flag) atomicOr(flag, kFlagBounds);
  return false;
#else
  (void)off, (void)n, (void)extent, (void)flag;
  return true;
#endif
}

// [p, p + bytes) inside the shared allocation [base, base + extent)
__device__ __forceinline__ bool in_shared(const void *p, int64_t bytes, const void *base, int64_t extent,
                                          unsigned *flag) {
#if GIRIH_CHECKED
  const char *q = static_cast<const char *>(p), *b = static_cast<const char *>(base);
  if (q >= b && q + bytes <= b + extent) return true;
  if (flag) atomicOr(flag, kFlagBounds);
  return false;
#else
  (void)p, (void)bytes, (void)base, (void)extent, (void)flag;
  return true;
#endif
}

// one write of points [off, off + n) of a state buffer
__device__ __forceinline__ void count_writes(unsigned *cov, int64_t off, int64_t n) {
#if GIRIH_CHECKED
  if (cov)
    for (int64_t k = 0; k < n; k++) atomicAdd(cov + off + k, 1u);
#else
  (void)cov, (void)off, (void)n;
#endif
}

}  // namespace girih
