// Batched ensemble: many independent chains of uneven lattice size (and of
// up to four groups) updated by one kernel per colour-phase slot.
//
// Slot k holds the k-th colour phase of every chain that has one; a chain's
// phases run in order, so every chain follows exactly the sequence of its
// single-chain sweep and gives bit-identical configurations.  A slot's work is
// a list of tiles (chain, first site of the phase list, count, direction);
// the blocks of one wave stage the shared tables of every group once and then
// take tiles in turn.  Sweep counters (the Philox key component) live in
// device memory and are advanced by a last kernel, so one sweep is a fixed
// sequence of launches that is captured once into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "batch.h"
#include "chain.h"
#include "visit.cuh"

namespace dym {

namespace {

template <int D>
__global__ void __launch_bounds__(256) k_batch_sub(const BatchTile* __restrict__ tiles, uint32_t ntiles,
                                                   const BatchChainDev* __restrict__ chains, const __grid_constant__ BatchGroups groups,
                                                   const uint32_t* __restrict__ sweeps, int nhit) {
  extern __shared__ __align__(16) unsigned char smem[];
  for (int g = 0; g < groups.n; ++g) {
    const BatchGroupDev& G = groups.g[g];
    stage_sub_tables(G.retr, G.inv, G.sub, G.P, G.npool, reinterpret_cast<double*>(smem + G.off_retr),
                     reinterpret_cast<uint16_t*>(smem + G.off_inv), reinterpret_cast<uint16_t*>(smem + G.off_sub));
  }
  __syncthreads();
  for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const BatchTile tl = tiles[t];
    const BatchChainDev c = chains[tl.chain];
    if ((unsigned)c.group >= (unsigned)groups.n) continue;  // checked on the host as well
    const BatchGroupDev& G = groups.g[c.group];
    SweepArgs a{};
    a.links = c.links;
    a.V = c.V;
    a.Nt = c.Nt;
    a.Nx = c.Nx;
    a.mult = G.mult;
    a.P = G.P;
    a.npool = G.npool;
    a.beta0 = c.beta0;
    a.beta1 = c.beta1;
    a.beta2 = c.beta2;
    a.seed = c.seed;
    a.nhit = nhit;
    const uint32_t sweep = sweeps[tl.chain];
    const double* s_retr = reinterpret_cast<const double*>(smem + G.off_retr);
    const uint16_t* s_inv = reinterpret_cast<const uint16_t*>(smem + G.off_inv);
    const uint16_t* s_sub = reinterpret_cast<const uint16_t*>(smem + G.off_sub);
    unsigned hits = 0, accs = 0;
    for (uint32_t k = threadIdx.x; k < tl.count; k += blockDim.x) {
      const uint32_t i = c.sites[tl.begin + k];
      switch (tl.dir) {
        case 0: visit_sub<D, 0>(a, i, sweep, s_retr, s_inv, s_sub, hits, accs); break;
        case 1: visit_sub<D, 1>(a, i, sweep, s_retr, s_inv, s_sub, hits, accs); break;
        case 2: if (D > 2) visit_sub<D, (D > 2 ? 2 : 0)>(a, i, sweep, s_retr, s_inv, s_sub, hits, accs); break;
        case 3: if (D > 3) visit_sub<D, (D > 3 ? 3 : 0)>(a, i, sweep, s_retr, s_inv, s_sub, hits, accs); break;
      }
    }
    flush_counters(c.ctr, hits, accs, 0);
  }
}

// The same work list with the mixed-precision visit (visit_mixed): every group
// of the batch stages ReTr, inverses, packed sub-table, element classes and
// fixed-point class values.
template <int D, int HU>
__global__ void __launch_bounds__(kMixedMaxThreads, 1) k_batch_mixed(const BatchTile* __restrict__ tiles, uint32_t ntiles,
                                                     const BatchChainDev* __restrict__ chains, const __grid_constant__ BatchGroups groups,
                                                     const uint32_t* __restrict__ sweeps, int nhit) {
  extern __shared__ __align__(16) unsigned char smem[];
  for (int g = 0; g < groups.n; ++g) {
    const BatchGroupDev& G = groups.g[g];
    stage_sub_tables(G.retr, G.inv, G.sub, G.P, G.npool, reinterpret_cast<double*>(smem + G.off_retr),
                     reinterpret_cast<uint16_t*>(smem + G.off_inv), reinterpret_cast<uint16_t*>(smem + G.off_sub));
    uint8_t* s_cls = smem + G.off_cls8;
    for (uint32_t t = threadIdx.x; t < G.P; t += blockDim.x) s_cls[t] = G.cls8[t];
    if (threadIdx.x < kMixedMaxCls) reinterpret_cast<int32_t*>(smem + G.off_cfix)[threadIdx.x] = G.cfix[threadIdx.x];
  }
  __syncthreads();
  for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const BatchTile tl = tiles[t];
    const BatchChainDev c = chains[tl.chain];
    if ((unsigned)c.group >= (unsigned)groups.n) continue;  // checked on the host as well
    const BatchGroupDev& G = groups.g[c.group];
    SweepArgs a{};
    a.links = c.links;
    a.V = c.V;
    a.Nt = c.Nt;
    a.Nx = c.Nx;
    a.mult = G.mult;
    a.P = G.P;
    a.npool = G.npool;
    a.beta0 = c.beta0;
    a.beta1 = c.beta1;
    a.beta2 = c.beta2;
    a.seed = c.seed;
    a.nhit = nhit;
    a.b1f = c.b1f;
    a.b2f = c.b2f;
    a.dscale = G.dscale;
    a.dmargin = c.dmargin;
    dym_philox_round_keys(c.seed, a.rk);  // block-uniform: the tile's chain
    const uint32_t sweep = sweeps[tl.chain];
    const double* s_retr = reinterpret_cast<const double*>(smem + G.off_retr);
    const uint16_t* s_inv = reinterpret_cast<const uint16_t*>(smem + G.off_inv);
    const uint16_t* s_psub = reinterpret_cast<const uint16_t*>(smem + G.off_sub);
    const uint8_t* s_cls = smem + G.off_cls8;
    const int32_t* s_cfix = reinterpret_cast<const int32_t*>(smem + G.off_cfix);
    unsigned hits = 0, accs = 0, rechecks = 0;
    float max_err = 0.0f;
    for (uint32_t k = threadIdx.x; k < tl.count; k += blockDim.x) {
      const uint32_t i = c.sites[tl.begin + k];
      const uint32_t xyz = c.xyz[tl.begin + k];
      switch (tl.dir) {
        case 0: visit_mixed<D, 0, uint16_t, HU, true>(a, i, xyz, sweep, s_retr, s_inv, s_psub, s_cls, s_cfix, hits, accs, rechecks, max_err); break;
        case 1: visit_mixed<D, 1, uint16_t, HU, true>(a, i, xyz, sweep, s_retr, s_inv, s_psub, s_cls, s_cfix, hits, accs, rechecks, max_err); break;
        case 2: visit_mixed<D, 2, uint16_t, HU, true>(a, i, xyz, sweep, s_retr, s_inv, s_psub, s_cls, s_cfix, hits, accs, rechecks, max_err); break;
        case 3: visit_mixed<D, 3, uint16_t, HU, true>(a, i, xyz, sweep, s_retr, s_inv, s_psub, s_cls, s_cfix, hits, accs, rechecks, max_err); break;
      }
    }
    flush_counters(c.ctr, hits, accs, rechecks);
    flush_max_err(c.ctr + 3, max_err);
  }
}

__global__ void k_batch_advance(uint32_t* sweeps, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) sweeps[i] += 1;
}

template <int D>
void* batch_kernel() {
  return (void*)k_batch_sub<D>;
}

// The mixed kernel for a hit-unroll factor (1, 2, 5, 10: HitDraws groups).
using BatchMixedFn = void (*)(const BatchTile*, uint32_t, const BatchChainDev*, const BatchGroups, const uint32_t*,
                              int);

template <int D>
BatchMixedFn batch_mixed_for(int hu) {
  switch (hu >= 10 ? 10 : hu >= 5 ? 5 : hu >= 2 ? 2 : 1) {
    case 2: return k_batch_mixed<D, 2>;
    case 5: return k_batch_mixed<D, 5>;
    case 10: return k_batch_mixed<D, 10>;
    default: return k_batch_mixed<D, 1>;
  }
}

}  // namespace

void* batch_kernel_for(int D, bool mixed, int hit_unroll) {
  if (D != 4) return nullptr;
  return mixed ? (void*)batch_mixed_for<4>(hit_unroll) : batch_kernel<4>();
}



cudaError_t launch_batch_slot(int D, bool mixed, int hit_unroll, const BatchTile* tiles, uint32_t ntiles,
                              const BatchChainDev* chains, const BatchGroups& groups, const uint32_t* sweeps, int nhit,
                              unsigned grid, unsigned threads, size_t smem, cudaStream_t s) {
  if (ntiles == 0) return cudaSuccess;
  if (D != 4) return cudaErrorInvalidValue;  // four dimensions only (see launch_sweep_sub)
  if (mixed) {
    const BatchMixedFn fn = batch_mixed_for<4>(hit_unroll);
    fn<<<grid, threads, smem, s>>>(tiles, ntiles, chains, groups, sweeps, nhit);
  } else
    k_batch_sub<4><<<grid, threads, smem, s>>>(tiles, ntiles, chains, groups, sweeps, nhit);
  return cudaGetLastError();
}

cudaError_t launch_batch_advance(uint32_t* sweeps, uint32_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_batch_advance<<<(n + 255) / 256, 256, 0, s>>>(sweeps, n);
  return cudaGetLastError();
}

}  // namespace dym
