// Value-table sweep kernel (shared table of fixed-point values; the visit is
// visit.cuh vt_prepare/vt_hits) and its per-phase launcher.
#include <cuda_runtime.h>

#include <algorithm>

#include "chain.h"
#include "dym_core.h"
#include "staples.cuh"
#include "sweep_launch.cuh"
#include "visit.cuh"

namespace dym {

namespace {

// Value-table form of k_sweep_mixed (visit.cuh vt_prepare/vt_hits).  Shared
// memory: value table (element-major, padded to 16 bytes) | ReTr (FP64) |
// inverses | element values | pool.  The value table is copied with cp.async
// and the small tables with plain loads; none of them is written by the
// previous colour phase, so the staging runs before the programmatic wait and
// overlaps the previous launch's tail when launched with PDL.  (Waiting for
// the value table only after the first staple phase, which needs the small
// tables alone, was measured 3% slower: the staging's transfers then queue
// with the staple gathers.)
template <int D, int DIR, int HU>
__global__ void __launch_bounds__(kMixedMaxThreads, 1) k_sweep_vt(SweepArgs a, const int16_t* __restrict__ vsub) {
  extern __shared__ __align__(16) unsigned char smem[];
  const size_t vbytes = vt_table_bytes(a.P, a.npool);
  int16_t* s_vsub = reinterpret_cast<int16_t*>(smem);
  double* s_retr = reinterpret_cast<double*>(smem + vbytes);
  uint16_t* s_inv = reinterpret_cast<uint16_t*>(s_retr + a.P);
  int16_t* s_val = reinterpret_cast<int16_t*>(s_inv + a.P);
  uint16_t* s_pool = reinterpret_cast<uint16_t*>(s_val + a.P);
  cp_async_stage(s_vsub, vsub, vbytes);
  for (uint32_t t = threadIdx.x; t < a.P; t += blockDim.x) {
    s_retr[t] = a.retr[t];
    s_inv[t] = a.inv[t];
    s_val[t] = a.val16[t];
  }
  for (uint32_t t = threadIdx.x; t < a.npool; t += blockDim.x) s_pool[t] = a.pool[t];
  // The site list and coordinates are constant: fetch this thread's first
  // entry before the wait as well.
  uint32_t lo, hi;
  phase_range(a.n, lo, hi);
  uint32_t t = lo + threadIdx.x;
  uint32_t i_next = 0, xyz_next = 0;
  if (t < hi) {
    i_next = a.sites[t];
    xyz_next = a.xyz[t];
  }
  pdl_launch_dependents();
  pdl_wait_prior();  // the previous phase's links are final from here on
  cp_async_wait_all();
  __syncthreads();
  if (sweep_skipped(a)) return;
  constexpr int NT = 8 * (D - 1);
  unsigned hits = 0, accs = 0, rechecks = 0;
  float max_err = 0.0f;
  for (; t < hi; t += blockDim.x) {
    uint32_t u[NT], b;
    int32_t R, M;
    const uint32_t i = i_next, xyz = xyz_next;
    if (t + blockDim.x < hi) {
      i_next = a.sites[t + blockDim.x];
      xyz_next = a.xyz[t + blockDim.x];
    }
    vt_prepare<D, DIR>(a, i, xyz, s_inv, s_val, u, b, R, M);
    vt_hits<D, DIR, HU>(a, i, a.sweep, s_retr, s_inv, s_vsub, s_pool, u, b, R, M, hits, accs, rechecks, max_err);
  }
  flush_counters(a.counters, hits, accs, rechecks);
  flush_max_err(a.counters + 3, max_err);
}

// k_sweep_vt with two lanes per link (visit.cuh vt2_prepare/vt2_hits): twice
// the warps on a phase, so that the staple gathers and the hits' shared loads
// of a 65,536-link phase (431 links an SM) have 27 warps an SM to overlap
// instead of 13.  Same shared memory as k_sweep_vt.
template <int D, int DIR>
__global__ void __launch_bounds__(kVt2MaxThreads, 1) k_sweep_vt2(SweepArgs a, const int16_t* __restrict__ vsub) {
  extern __shared__ __align__(16) unsigned char smem[];
  const size_t vbytes = vt_table_bytes(a.P, a.npool);
  int16_t* s_vsub = reinterpret_cast<int16_t*>(smem);
  double* s_retr = reinterpret_cast<double*>(smem + vbytes);
  uint16_t* s_inv = reinterpret_cast<uint16_t*>(s_retr + a.P);
  int16_t* s_val = reinterpret_cast<int16_t*>(s_inv + a.P);
  uint16_t* s_pool = reinterpret_cast<uint16_t*>(s_val + a.P);
  cp_async_stage(s_vsub, vsub, vbytes);
  for (uint32_t t = threadIdx.x; t < a.P; t += blockDim.x) {
    s_retr[t] = a.retr[t];
    s_inv[t] = a.inv[t];
    s_val[t] = a.val16[t];
  }
  for (uint32_t t = threadIdx.x; t < a.npool; t += blockDim.x) s_pool[t] = a.pool[t];
  const bool back = (threadIdx.x & 1u) != 0;  // the pair: lanes 2m, 2m+1 of a warp
  const unsigned pm = pair_mask();
  const uint32_t stride = blockDim.x >> 1;
  uint32_t lo, hi;
  phase_range(a.n, lo, hi);
  uint32_t t = lo + (threadIdx.x >> 1);
  uint32_t i_next = 0, xyz_next = 0;
  if (t < hi) {
    i_next = a.sites[t];
    xyz_next = a.xyz[t];
  }
  pdl_launch_dependents();
  pdl_wait_prior();  // the previous phase's links are final from here on
  cp_async_wait_all();
  __syncthreads();
  if (sweep_skipped(a)) return;
  constexpr int NP = D - 1, NQ = 3 * (D - 1);
  unsigned hits = 0, accs = 0, rechecks = 0;
  float max_err = 0.0f;
  for (; t < hi; t += stride) {  // the same trip count for both lanes of a pair
    uint32_t up[NP], ur[NQ], b;
    int32_t R, M;
    const uint32_t i = i_next, xyz = xyz_next;
    if (t + stride < hi) {
      i_next = a.sites[t + stride];
      xyz_next = a.xyz[t + stride];
    }
    vt2_prepare<D, DIR>(a, i, xyz, back, pm, s_inv, s_val, up, ur, b, R, M);
    vt2_hits<D, DIR>(a, i, a.sweep, back, pm, s_retr, s_inv, s_vsub, s_pool, up, ur, b, R, M, hits, accs, rechecks,
                     max_err);
  }
  flush_counters(a.counters, hits, accs, rechecks);
  flush_max_err(a.counters + 3, max_err);
}

template <int D>
cudaError_t vt2_dispatch(int dir, const SweepArgs& a, const int16_t* vsub, cudaStream_t s) {
  const size_t smem = vt_smem_bytes(a.P, a.npool);
  void (*fn)(SweepArgs, const int16_t*) = nullptr;
  switch (dir) {
    case 0: fn = k_sweep_vt2<D, 0>; break;
    case 1: fn = k_sweep_vt2<D, 1>; break;
    case 2: if (D > 2) fn = k_sweep_vt2<D, (D > 2 ? 2 : 0)>; break;
    case 3: if (D > 3) fn = k_sweep_vt2<D, (D > 3 ? 3 : 0)>; break;
  }
  if (!fn) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (a.n == 0) return cudaSuccess;
  int dev = 0, sms = 0;
  e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  // Two threads a link: chunks as k_sweep_vt, twice the threads.
  const PhaseShape sh = phase_shape(a.n, sms, kVt2MaxThreads / 2, 64);
  return launch_phase(fn, sh.grid, 2 * sh.threads, smem, s, a, vsub);
}

template <int D>
cudaError_t vt_dispatch(int dir, const SweepArgs& a, const int16_t* vsub, cudaStream_t s) {
  const size_t smem = vt_smem_bytes(a.P, a.npool);
  void (*fn)(SweepArgs, const int16_t*) = nullptr;
  switch (hit_unroll_index(a.hit_unroll) * 4 + dir) {
#define DYM_VT_CASE(q, hu, d) \
    case 4 * q + d: if (D > d) fn = k_sweep_vt<D, (D > d ? d : 0), hu>; break;
#define DYM_VT_HU(q, hu) DYM_VT_CASE(q, hu, 0) DYM_VT_CASE(q, hu, 1) DYM_VT_CASE(q, hu, 2) DYM_VT_CASE(q, hu, 3)
    DYM_VT_HU(0, 1) DYM_VT_HU(1, 2) DYM_VT_HU(2, 5) DYM_VT_HU(3, 10)
#undef DYM_VT_HU
#undef DYM_VT_CASE
  }
  if (!fn) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (a.n == 0) return cudaSuccess;
  int dev = 0, sms = 0;
  e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const PhaseShape sh = phase_shape(a.n, sms, kMixedMaxThreads);  // one wave of chunks, as k_sweep_mixed
  return launch_phase(fn, sh.grid, sh.threads, smem, s, a, vsub);
}

}  // namespace

cudaError_t launch_sweep_vt(int D, int dir, const SweepArgs& a, const int16_t* vsub, cudaStream_t s) {
  if (D == 4) return a.lanes_per_link == 2 ? vt2_dispatch<4>(dir, a, vsub, s) : vt_dispatch<4>(dir, a, vsub, s);
  return cudaErrorInvalidValue;
}

}  // namespace dym
