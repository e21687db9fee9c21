// Metropolis sweep kernels: one thread per link of one colour phase.
//
// Two kernels implement the hit loop of dym-mod-metro.cpp:161-192 with the
// reference's FP64 arithmetic and order:
//
//  * k_sweep_direct -- any table, any proposal pool: every hit gathers
//    mult[bnew][staple] for all 8(D-1) staples from the L2-resident Cayley
//    table (358 gathers per link visit at 10 hits in 4D).
//
//  * k_sweep_sub    -- class-constant tables, nearest-element pool: with
//    u_j = s_j * b (staple times current link), Tr(bnew s_j) = Tr(b g s_j) =
//    Tr(g s_j b) = Tr(u_j g), so a proposal's terms depend only on (g, u_j).
//    The products u * g for the pool elements fit in shared memory as
//    sub[k][u] = u * g_k (155 KB for S(1080)'s 72-element pool): a hit is
//    8(D-1) shared-memory loads instead of L2 gathers, and an accepted hit
//    advances u_j <- u_j * g_k from the same entries.  108 L2 gathers per
//    link visit remain (staples and u_j).
//
//  * k_sweep_mixed  -- the same decisions with exact integer sums of
//    fixed-point class values and an FP32 threshold test; FP64 only for the
//    hits within a proven bound of the threshold (visit_mixed), re-evaluated
//    on the reference's own elements b s_j, so the configurations are the
//    FP64 path's bit for bit on any table (also one whose ReTr carries
//    rounding noise inside a class, as the reference's shipped files do).
//
//  * k_sweep_vt     -- k_sweep_mixed with the shared table holding fixed-point
//    values instead of elements (fastest while accepted moves are rare).//
// This file holds the FP64 kernels, the lattice set-up kernels and their
// launchers; the mixed-precision kernels are in sweep_mixed.cu and
// sweep_vt.cu.
#include <cuda_runtime.h>

#include <algorithm>

#include "chain.h"
#include "dym_core.h"
#include "staples.cuh"
#include "sweep_launch.cuh"
#include "visit.cuh"

namespace dym {

namespace {

template <int D, int DIR>
__global__ void __launch_bounds__(256) k_sweep_direct(SweepArgs a) {
  constexpr int NS = 2 * (D - 1), NR = 6 * (D - 1);
  extern __shared__ __align__(16) unsigned char smem[];
  double* s_retr = reinterpret_cast<double*>(smem);
  uint16_t* s_inv = reinterpret_cast<uint16_t*>(s_retr + a.P);
  uint16_t* s_pool = s_inv + a.P;
  for (uint32_t t = threadIdx.x; t < a.P; t += blockDim.x) {
    s_retr[t] = a.retr[t];
    s_inv[t] = a.inv[t];
  }
  for (uint32_t t = threadIdx.x; t < a.npool; t += blockDim.x) s_pool[t] = a.pool[t];
  pdl_launch_dependents();
  pdl_wait_prior();
  __syncthreads();
  if (sweep_skipped(a)) return;

  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned hits = 0, accs = 0;
  if (tid < a.n) {
    const uint32_t i = a.sites[tid];
    SiteGeo<D> geo;
    site_geo<D>(i, a.Nt, a.Nx, geo);
    GlobalTab T{a.mult, s_inv, a.P};
    const uint16_t* L = a.links;
    const uint32_t V = a.V;
    auto ld = [L, V](uint32_t s, int d) -> uint32_t { return __ldg(L + (size_t)d * V + s); };
    uint32_t st[NS], re[NR];
    build_staples<D, DIR>(i, geo, T, ld, st, re);

    uint16_t* own = a.links + (size_t)DIR * V + i;
    uint32_t b = *own;
    const uint32_t b0 = b;
    double r1 = 0, m1 = 0;
#pragma unroll
    for (int j = 0; j < NS; ++j) r1 = DYM_ADD(r1, s_retr[T.mul(b, st[j])]);
#pragma unroll
    for (int k = 0; k < NR; ++k) m1 = DYM_ADD(m1, s_retr[T.mul(b, re[k])]);
    // The plain draw: with the per-link Philox state (dym_metro_hit) this
    // kernel used 64 registers instead of 80 (a fourth block per SM) and
    // measured 26% slower.
    for (int h = 0; h < a.nhit; ++h) {
      const dym_u32x4 r = dym_hit_random(a.seed, a.sweep, i, DIR, (uint32_t)h, DYM_TAG_METRO);
      const uint32_t g = s_pool[dym_pick(r.v[0], a.npool)];
      const uint32_t bnew = T.mul(b, g);
      double r1n = 0, m1n = 0;
#pragma unroll
      for (int j = 0; j < NS; ++j) r1n = DYM_ADD(r1n, s_retr[T.mul(bnew, st[j])]);
#pragma unroll
      for (int k = 0; k < NR; ++k) m1n = DYM_ADD(m1n, s_retr[T.mul(bnew, re[k])]);
      const double oldact = dym_action(a.beta0, a.beta1, a.beta2, r1, m1);
      const double newact = dym_action(a.beta0, a.beta1, a.beta2, r1n, m1n);
      ++hits;
      if (dym_accept(oldact, newact, dym_u53(r.v[1], r.v[2]))) {
        b = bnew;
        r1 = r1n;
        m1 = m1n;
        ++accs;
      }
    }
    finish_link<D>(a, DIR, i, b, b0);
  }
  flush_counters(a.counters, hits, accs, 0);
}

// ---------------------------------------------------------------------------
// Shared sub-table kernel (FP64, class-constant tables).  A minimal change of
// k_sweep_direct: same launch shape, counters and FP64 arithmetic; only the
// per-hit products come from sub[k][u] = u * g_k in shared memory instead of
// mult[bnew][s_j] in L2.  With u_j = s_j * b, the element u_j * g_k =
// s_j b g_k is conjugate to bnew s_j = b g_k s_j, so for a table whose ReTr
// is the same double on every conjugacy class ReTr[u_j g_k] is bit-identical
// to the reference's ReTr[mult[bnew][s_j]], summed in the same order.
// ---------------------------------------------------------------------------
template <int D, int DIR>
__global__ void __launch_bounds__(256) k_sweep_sub(SweepArgs a, const uint16_t* __restrict__ sub) {
  extern __shared__ __align__(16) unsigned char smem[];
  double* s_retr = reinterpret_cast<double*>(smem);
  uint16_t* s_inv = reinterpret_cast<uint16_t*>(s_retr + a.P);
  uint16_t* s_sub = s_inv + a.P;
  stage_sub_tables(a.retr, a.inv, sub, a.P, a.npool, s_retr, s_inv, s_sub);
  pdl_launch_dependents();
  pdl_wait_prior();
  __syncthreads();
  if (sweep_skipped(a)) return;

  unsigned hits = 0, accs = 0;
  // One wave of blocks, each staging the table once and visiting several links.
  for (uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x; tid < a.n; tid += gridDim.x * blockDim.x)
    visit_sub<D, DIR, true>(a, a.sites[tid], a.sweep, s_retr, s_inv, s_sub, hits, accs);
  flush_counters(a.counters, hits, accs, 0);
}

__global__ void k_hot_start(uint16_t* links, uint32_t V, int D, uint32_t P, uint64_t seed) {
  const size_t n = (size_t)V * D;
  for (size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
    const uint32_t dir = (uint32_t)(l / V), site = (uint32_t)(l % V);
    dym_u32x4 c;
    c.v[0] = site;
    c.v[1] = 0;
    c.v[2] = dir;
    c.v[3] = DYM_TAG_HOT;
    const dym_u32x4 r = dym_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    links[l] = (uint16_t)dym_pick(r.v[0], P);
  }
}

// dym_links_set on the device: the complement of the smallest index whose id
// is >= P into *first (0 beforehand; the smallest index has the largest
// complement), then the stage copied into the links only if there is none.
__device__ __forceinline__ void note_bad(unsigned long long* first, size_t k) {
  atomicMax(first, ~(unsigned long long)k);
}

__global__ void k_ids_first_bad(const uint16_t* __restrict__ ids, size_t n, uint32_t P, unsigned long long* first) {
  pdl_launch_dependents();  // the commit may be scheduled; it waits for this grid
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    if (ids[k] >= P) note_bad(first, k);
}

// The same check reading the ids straight from page-locked host memory (the
// caller's buffer, through its device mapping) and writing them to the stage:
// one pass over the host link instead of a copy-engine transfer and a pass.
// Host reads are 16 bytes wide (eight ids) when the host buffer starts on 16
// bytes; `nv` is the number of such groups (0 otherwise), the ids after them
// go one by one.
__global__ void k_ids_from_host(uint16_t* __restrict__ stage, const uint16_t* __restrict__ host, size_t n, size_t nv,
                                uint32_t P, unsigned long long* first) {
  pdl_launch_dependents();  // the commit may be scheduled; it waits for this grid
  const size_t t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x, dt = (size_t)gridDim.x * blockDim.x;
  for (size_t q = t0; q < nv; q += dt) {
    const uint4 w = reinterpret_cast<const uint4*>(host)[q];
    reinterpret_cast<uint4*>(stage)[q] = w;
    const uint32_t x[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int h = 0; h < 8; ++h) {
      const uint32_t v = (x[h >> 1] >> (16 * (h & 1))) & 0xFFFFu;
      if (v >= P) note_bad(first, 8 * q + h);
    }
  }
  for (size_t k = 8 * nv + t0; k < n; k += dt) {
    const uint16_t v = host[k];
    stage[k] = v;
    if (v >= P) note_bad(first, k);
  }
}

// Launched with programmatic serialization behind the check: waits for it
// (its result in *first) before reading anything.
__global__ void k_ids_commit(uint16_t* __restrict__ links, const uint16_t* __restrict__ stage, size_t n,
                             const unsigned long long* first) {
  pdl_wait_prior();
  pdl_launch_dependents();  // the first sweep may stage its tables
  if (*first != 0) return;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    links[k] = stage[k];
}

// dym_sweep_refarray's upload: the reference's a[i*D + d] (int32) read in
// order, checked (ids outside [0, P), the smallest index into *first) and
// written to the stage direction-major.
__global__ void k_ids_from_ref(uint16_t* __restrict__ stage, const int32_t* __restrict__ ref, uint32_t V, int D,
                               uint32_t P, unsigned long long* first) {
  pdl_launch_dependents();  // the commit may be scheduled; it waits for this grid
  const size_t n = (size_t)V * D;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const int32_t v = ref[k];
    const uint32_t i = (uint32_t)(k / (uint32_t)D), d = (uint32_t)(k % (uint32_t)D);
    if (v < 0 || (uint32_t)v >= P) note_bad(first, k);
    stage[(size_t)d * V + i] = (uint16_t)v;
  }
}

// dym_sweep_refarray's read-back into a page-locked array: ref[i*D + d] =
// links[d*V + i] in the array's order, so that the writes through the
// device mapping are coalesced; skipped entirely after a refused upload.
__global__ void k_links_to_ref(int32_t* __restrict__ ref, const uint16_t* __restrict__ links, uint32_t V, int D,
                               const unsigned long long* skip) {
  pdl_wait_prior();
  if (*skip != 0) return;
  const size_t n = (size_t)V * D;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const uint32_t i = (uint32_t)(k / (uint32_t)D), d = (uint32_t)(k % (uint32_t)D);
    ref[k] = links[(size_t)d * V + i];
  }
}

__global__ void k_counters_out(unsigned long long* dev, unsigned long long* host, int n) {
  pdl_wait_prior();
  const int t = threadIdx.x;
  if (t < n) {
    host[t] = dev[t];
    dev[t] = 0;
  }
  __threadfence_system();
}

__global__ void k_fill(uint16_t* p, size_t n, uint16_t v) {
  for (size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) p[l] = v;
}

template <int D, int DIR>
__global__ void k_staples(SweepArgs a, const uint32_t* sites, uint32_t n, uint16_t* out) {
  constexpr int NS = 2 * (D - 1), NR = 6 * (D - 1);
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= n) return;
  const uint32_t i = sites[tid];
  SiteGeo<D> geo;
  site_geo<D>(i, a.Nt, a.Nx, geo);
  GlobalTab T{a.mult, a.inv, a.P};
  const uint16_t* L = a.links;
  const uint32_t V = a.V;
  auto ld = [L, V](uint32_t s, int d) -> uint32_t { return L[(size_t)d * V + s]; };
  uint32_t st[NS], re[NR];
  build_staples<D, DIR>(i, geo, T, ld, st, re);
  for (int j = 0; j < NS; ++j) out[(size_t)tid * (NS + NR) + j] = (uint16_t)st[j];
  for (int j = 0; j < NR; ++j) out[(size_t)tid * (NS + NR) + NS + j] = (uint16_t)re[j];
}

template <int D>
cudaError_t direct_dispatch(int dir, const SweepArgs& a, cudaStream_t s) {
  const size_t smem = (size_t)a.P * 8 + (size_t)a.P * 2 + (size_t)a.npool * 2 + 16;
  const unsigned grid = (a.n + 255) / 256;
  void (*fn)(SweepArgs) = nullptr;
  switch (dir) {
    case 0: fn = k_sweep_direct<D, 0>; break;
    case 1: fn = k_sweep_direct<D, 1>; break;
    case 2: if (D > 2) fn = k_sweep_direct<D, (D > 2 ? 2 : 0)>; break;
    case 3: if (D > 3) fn = k_sweep_direct<D, (D > 3 ? 3 : 0)>; break;
  }
  if (!fn) return cudaErrorInvalidValue;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  if (grid == 0) return cudaSuccess;
  return launch_phase(fn, grid, 256, smem, s, a);
}

template <int D>
cudaError_t sub_dispatch(int dir, const SweepArgs& a, const uint16_t* sub, cudaStream_t s) {
  const size_t smem = sub_smem_bytes(a.P, a.npool);
  void (*fn)(SweepArgs, const uint16_t*) = nullptr;
  switch (dir) {
    case 0: fn = k_sweep_sub<D, 0>; break;
    case 1: fn = k_sweep_sub<D, 1>; break;
    case 2: if (D > 2) fn = k_sweep_sub<D, (D > 2 ? 2 : 0)>; break;
    case 3: if (D > 3) fn = k_sweep_sub<D, (D > 3 ? 3 : 0)>; break;
  }
  if (!fn) return cudaErrorInvalidValue;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const unsigned need = (a.n + 255) / 256;
  if (need == 0) return cudaSuccess;
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, smem);
  if (e != cudaSuccess) return e;
  const unsigned grid = std::min<unsigned>(need, (unsigned)std::max(1, sms * std::max(per_sm, 1)));
  return launch_phase(fn, grid, 256, smem, s, a, sub);
}

template <int D>
cudaError_t staples_dispatch(int dir, const SweepArgs& a, const uint32_t* sites, uint32_t n, uint16_t* out,
                             cudaStream_t s) {
  void (*fn)(SweepArgs, const uint32_t*, uint32_t, uint16_t*) = nullptr;
  switch (dir) {
    case 0: fn = k_staples<D, 0>; break;
    case 1: fn = k_staples<D, 1>; break;
    case 2: if (D > 2) fn = k_staples<D, (D > 2 ? 2 : 0)>; break;
    case 3: if (D > 3) fn = k_staples<D, (D > 3 ? 3 : 0)>; break;
  }
  if (!fn) return cudaErrorInvalidValue;
  if (n == 0) return cudaSuccess;
  fn<<<(n + 127) / 128, 128, 0, s>>>(a, sites, n, out);
  return cudaGetLastError();
}

}  // namespace

size_t sub_smem_bytes(uint32_t P, uint32_t npool) {
  return (size_t)P * 8 + (size_t)P * 2 + (size_t)npool * P * 2 + 16;
}

size_t mixed_smem_bytes(uint32_t P, uint32_t npool, size_t entry) {
  return mixed_psub_offset(P, entry) + (size_t)npool * P * entry + (size_t)P + 16;
}

size_t vt_smem_bytes(uint32_t P, uint32_t npool) {
  return vt_table_bytes(P, npool) + (size_t)P * 8 + (size_t)P * 2 + (size_t)P * 2 + (size_t)npool * 2 + 16;
}

cudaError_t launch_sweep_direct(int D, int dir, const SweepArgs& a, cudaStream_t s) {
  switch (D) {
    case 2: return direct_dispatch<2>(dir, a, s);
    case 3: return direct_dispatch<3>(dir, a, s);
    case 4: return direct_dispatch<4>(dir, a, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_sweep_sub(int D, int dir, const SweepArgs& a, const uint16_t* sub, cudaStream_t s) {
  // Four dimensions only: the D = 2 and D = 3 instantiations of the shared
  // sub-table kernels faulted on the GPU without a cause found in the source
  // (see sub_eligible in capi.cu); those lattices use k_sweep_direct.
  if (D == 4) return sub_dispatch<4>(dir, a, sub, s);
  return cudaErrorInvalidValue;
}

cudaError_t launch_staples(int D, int dir, const SweepArgs& a, const uint32_t* sites, uint32_t n, uint16_t* out,
                           cudaStream_t s) {
  switch (D) {
    case 2: return staples_dispatch<2>(dir, a, sites, n, out, s);
    case 3: return staples_dispatch<3>(dir, a, sites, n, out, s);
    case 4: return staples_dispatch<4>(dir, a, sites, n, out, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_hot_start(uint16_t* links, uint32_t V, int D, uint32_t P, uint64_t seed, cudaStream_t s) {
  const size_t n = (size_t)V * D;
  unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 16);
  if (grid == 0) return cudaSuccess;
  k_hot_start<<<grid, 256, 0, s>>>(links, V, D, P, seed);
  return cudaGetLastError();
}

cudaError_t launch_links_commit(uint16_t* links, const uint16_t* stage, size_t n, uint32_t P,
                                unsigned long long* first, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 8);
  k_ids_first_bad<<<grid, 256, 0, s>>>(stage, n, P, first);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return launch_phase(k_ids_commit, grid, 256, 0, s, links, (const uint16_t*)stage, n,
                      (const unsigned long long*)first);
}

cudaError_t launch_links_from_host(uint16_t* links, uint16_t* stage, const uint16_t* host_mapped, size_t n,
                                   uint32_t P, unsigned long long* first, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const size_t nv = (reinterpret_cast<uintptr_t>(host_mapped) & 15u) ? 0 : n / 8;
  const unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 8);
  k_ids_from_host<<<grid, 256, 0, s>>>(stage, host_mapped, n, nv, P, first);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return launch_phase(k_ids_commit, grid, 256, 0, s, links, (const uint16_t*)stage, n,
                      (const unsigned long long*)first);
}

cudaError_t launch_links_from_ref(uint16_t* links, uint16_t* stage, const int32_t* ref, uint32_t V, int D, uint32_t P,
                                  unsigned long long* first, cudaStream_t s) {
  const size_t n = (size_t)V * D;
  if (n == 0) return cudaSuccess;
  const unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 8);
  k_ids_from_ref<<<grid, 256, 0, s>>>(stage, ref, V, D, P, first);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return launch_phase(k_ids_commit, grid, 256, 0, s, links, (const uint16_t*)stage, n,
                      (const unsigned long long*)first);
}

cudaError_t launch_links_to_ref(int32_t* ref, const uint16_t* links, uint32_t V, int D,
                                const unsigned long long* skip, cudaStream_t s) {
  const size_t n = (size_t)V * D;
  if (n == 0) return cudaSuccess;
  const unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 8);
  return launch_phase(k_links_to_ref, grid, 256, 0, s, ref, links, V, D, skip);
}

cudaError_t launch_counters_out(unsigned long long* dev, unsigned long long* host_mapped, int n, cudaStream_t s) {
  return launch_phase(k_counters_out, 1, 32, 0, s, dev, host_mapped, n);
}

cudaError_t launch_fill(uint16_t* links, size_t n, uint16_t v, cudaStream_t s) {
  unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 16);
  if (grid == 0) return cudaSuccess;
  k_fill<<<grid, 256, 0, s>>>(links, n, v);
  return cudaGetLastError();
}

}  // namespace dym
