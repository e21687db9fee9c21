// L2 random-gather probe: the peak against which the sweep kernels' table
// gathers are reported.  Every thread issues independent 2-byte loads at
// hashed positions of an L2-resident table, cached at L2 only (as a gather
// from a multi-megabyte table effectively is), so the rate measured is the
// random 32-byte-sector throughput of the L2.
#include <cuda_runtime.h>

#include "chain.h"

namespace dym {

namespace {

__device__ __forceinline__ uint32_t mix(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

constexpr int kChains = 16;

__global__ void __launch_bounds__(256) k_probe(const uint16_t* __restrict__ tab, uint32_t n, int iters,
                                               uint32_t* sink) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t h[kChains];
#pragma unroll
  for (int j = 0; j < kChains; ++j) h[j] = mix(tid * kChains + j + 1);
  uint32_t acc = 0;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int j = 0; j < kChains; ++j) {
      const uint32_t idx = (uint32_t)(((uint64_t)h[j] * n) >> 32);
      acc += __ldcg(tab + idx);
      h[j] = h[j] * 1664525u + 1013904223u + acc;  // next position depends on the load
    }
  }
  if (acc == 0xFFFFFFFFu) sink[0] = acc;
}

}  // namespace

cudaError_t probe_l2_gather(uint32_t table_bytes, double* sectors_per_s) {
  const uint32_t n = table_bytes / 2;
  uint16_t* tab = nullptr;
  uint32_t* sink = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t err = cudaMalloc(&tab, (size_t)n * 2);
  if (err == cudaSuccess) err = cudaMalloc(&sink, 4);
  if (err == cudaSuccess) err = cudaMemset(tab, 0x11, (size_t)n * 2);
  if (err == cudaSuccess) err = cudaEventCreate(&e0);
  if (err == cudaSuccess) err = cudaEventCreate(&e1);
  int sms = 0, dev = 0;
  if (err == cudaSuccess) err = cudaGetDevice(&dev);
  if (err == cudaSuccess) err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256, iters = 256;
  float best = 1e30f;
  for (int rep = 0; err == cudaSuccess && rep < 4; ++rep) {
    cudaEventRecord(e0);
    k_probe<<<blocks, threads>>>(tab, n, iters, sink);
    cudaEventRecord(e1);
    err = cudaEventSynchronize(e1);
    float ms = 0;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;  // first launch is warm-up
  }
  if (err == cudaSuccess)
    *sectors_per_s = (double)blocks * threads * iters * kChains / (best * 1e-3);
  cudaFree(tab);
  cudaFree(sink);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  return err;
}

}  // namespace dym
