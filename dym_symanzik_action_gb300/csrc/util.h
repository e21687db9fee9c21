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

}  // namespace dym

#define DYM_CUDA(call, what)                                      \
  do {                                                            \
    cudaError_t _e = (call);                                      \
    if (_e != cudaSuccess) return ::dym::cuda_fail(_e, what);     \
  } while (0)
