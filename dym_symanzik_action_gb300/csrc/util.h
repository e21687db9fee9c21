// Internal helpers shared by the host translation units.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "engine.h"

namespace dym {

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

}  // namespace dym

#define DYM_CUDA(call, what)                                      \
  do {                                                            \
    cudaError_t _e = (call);                                      \
    if (_e != cudaSuccess) return ::dym::cuda_fail(_e, what);     \
  } while (0)
