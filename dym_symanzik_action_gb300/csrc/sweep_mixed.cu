// Mixed-precision sweep kernel (packed sub-table of element and class; the
// visit is visit.cuh visit_mixed) and its per-phase launcher.
#include <cuda_runtime.h>

#include <algorithm>

#include "chain.h"
#include "dym_core.h"
#include "staples.cuh"
#include "sweep_launch.cuh"
#include "visit.cuh"

namespace dym {

namespace {

// Shared memory: ReTr (FP64) | class values (int32 fixed point) | inverses |
// packed sub-table (entries of type E, starting at mixed_psub_offset) |
// element classes.
template <int D, int DIR, class E, int HU>
__global__ void __launch_bounds__(kMixedMaxThreads, 1) k_sweep_mixed(SweepArgs a, const E* __restrict__ psub) {
  extern __shared__ __align__(16) unsigned char smem[];
  double* s_retr = reinterpret_cast<double*>(smem);
  int32_t* s_cfix = reinterpret_cast<int32_t*>(s_retr + a.P);
  uint16_t* s_inv = reinterpret_cast<uint16_t*>(s_cfix + kMixedMaxCls);
  E* s_psub = reinterpret_cast<E*>(smem + mixed_psub_offset(a.P, sizeof(E)));
  uint8_t* s_cls = reinterpret_cast<uint8_t*>(s_psub + (size_t)a.npool * a.P);
  // The staging copies npool * P entries as halfwords.
  stage_sub_tables(a.retr, a.inv, reinterpret_cast<const uint16_t*>(psub), a.P, a.npool * (uint32_t)(sizeof(E) / 2),
                   s_retr, s_inv, reinterpret_cast<uint16_t*>(s_psub));
  for (uint32_t t = threadIdx.x; t < a.P; t += blockDim.x) s_cls[t] = a.cls8[t];
  if (threadIdx.x < kMixedMaxCls) s_cfix[threadIdx.x] = a.cfix[threadIdx.x];
  uint32_t lo, hi;
  phase_range(a.n, lo, hi);
  uint32_t t = lo + threadIdx.x;
  uint32_t i_next = 0, xyz_next = 0;  // constant site list: fetched before the wait
  if (t < hi) {
    i_next = a.sites[t];
    xyz_next = a.xyz[t];
  }
  pdl_launch_dependents();
  pdl_wait_prior();
  cp_async_wait_all();
  __syncthreads();
  if (sweep_skipped(a)) return;

  unsigned hits = 0, accs = 0, rechecks = 0;
  float max_err = 0.0f;
  for (; t < hi; t += blockDim.x) {
    const uint32_t i = i_next, xyz = xyz_next;
    if (t + blockDim.x < hi) {
      i_next = a.sites[t + blockDim.x];
      xyz_next = a.xyz[t + blockDim.x];
    }
    visit_mixed<D, DIR, E, HU, true>(a, i, xyz, a.sweep, s_retr, s_inv, s_psub, s_cls, s_cfix, hits, accs, rechecks,
                               max_err);
  }
  flush_counters(a.counters, hits, accs, rechecks);
  flush_max_err(a.counters + 3, max_err);
}

template <int D, class E>
cudaError_t mixed_dispatch(int dir, const SweepArgs& a, const E* psub, cudaStream_t s) {
  const size_t smem = mixed_smem_bytes(a.P, a.npool, sizeof(E));
  void (*fn)(SweepArgs, const E*) = nullptr;
  switch (hit_unroll_index(a.hit_unroll) * 4 + dir) {
#define DYM_MIXED_CASE(q, hu, d) \
    case 4 * q + d: if (D > d) fn = k_sweep_mixed<D, (D > d ? d : 0), E, hu>; break;
#define DYM_MIXED_HU(q, hu) DYM_MIXED_CASE(q, hu, 0) DYM_MIXED_CASE(q, hu, 1) DYM_MIXED_CASE(q, hu, 2) \
    DYM_MIXED_CASE(q, hu, 3)
    DYM_MIXED_HU(0, 1) DYM_MIXED_HU(1, 2) DYM_MIXED_HU(2, 5) DYM_MIXED_HU(3, 10)
#undef DYM_MIXED_HU
#undef DYM_MIXED_CASE
  }
  if (!fn) return cudaErrorInvalidValue;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  if (a.n == 0) return cudaSuccess;
  // One block per SM at most (the shared tables allow no more), each on a
  // contiguous chunk of the phase, walked in turn when larger than a block.
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const PhaseShape sh = phase_shape(a.n, sms, kMixedMaxThreads);
  return launch_phase(fn, sh.grid, sh.threads, smem, s, a, psub);
}

}  // namespace

cudaError_t launch_sweep_mixed(int D, int dir, const SweepArgs& a, const uint16_t* psub, cudaStream_t s) {
  if (D == 4) return mixed_dispatch<4, uint16_t>(dir, a, psub, s);  // four dimensions only, as launch_sweep_sub
  return cudaErrorInvalidValue;
}

cudaError_t launch_sweep_mixed_wide(int D, int dir, const SweepArgs& a, const uint32_t* psub, cudaStream_t s) {
  if (D == 4) return mixed_dispatch<4, uint32_t>(dir, a, psub, s);
  return cudaErrorInvalidValue;
}

}  // namespace dym
