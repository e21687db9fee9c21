// Internal helpers shared by the host translation units.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <string>

#include "dym_core.h"
#include "engine.h"

namespace dym {

// NVTX range over an entry point, for timeline profilers (header-only NVTX 3:
// a no-op unless a tool injects itself).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

inline int cuda_fail(cudaError_t e, const char* what) {
  return fail(DYM_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T>
inline cudaError_t dmalloc(T** p, size_t n) {
  return cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T));
}

// Copy that is complete when it returns and ordered after earlier work on `s`.
// The engine's streams are non-blocking, so a plain cudaMemcpy (legacy default
// stream) is not ordered with them, and a host-to-device cudaMemcpy from
// pageable memory may return before its data has reached the device: a kernel
// launched next on a non-blocking stream could read the old contents.
inline cudaError_t copy_sync(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s) {
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e;
}

// Fixed-point scale 2^S of the class values for the mixed-precision kernels:
// the largest S <= 24 for which a difference of two sums of NR = 6(D-1)
// rectangle terms, each at most |c| 2^S + 1/2, stays inside int32.
inline int fix_shift(const Group& g, int D) { return dym_fix_shift(g.max_abs_retr, D); }

// Rounding error of one fixed-point class value: half a unit plus the spread
// of ReTr inside a class.
inline double fix_q(const Group& g, int S) { return std::ldexp(1.0, -(S + 1)) + g.cls_spread; }

// dym_mixed_margin for a Metropolis sweep at couplings (b0, b1, b2), rounded up
// to FP32.  With DYM_RECHECK_ALL=1 in the environment (a validation mode, read
// when a sweep or batch is set up) the bound is infinite, so every hit of the
// mixed kernels takes the FP64 re-evaluation path.
inline float mixed_margin(const Group& g, int D, int S, double b0, double b1, double b2) {
  const char* all = std::getenv("DYM_RECHECK_ALL");
  if (all && all[0] == '1') return INFINITY;
  const double m = dym_mixed_margin(b0, b1, 2.0 * (D - 1), b2, 6.0 * (D - 1), fix_q(g, S), g.max_abs_retr);
  return std::nextafter((float)m, INFINITY);
}

}  // namespace dym

#define DYM_CUDA(call, what)                                      \
  do {                                                            \
    cudaError_t _e = (call);                                      \
    if (_e != cudaSuccess) return ::dym::cuda_fail(_e, what);     \
  } while (0)
