// Launch helpers shared by the sweep kernels' translation units (sweep.cu,
// sweep_mixed.cu, sweep_vt.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

namespace dym {

// Launch one colour phase with programmatic stream serialization: the next
// phase's blocks may start, and stage their tables, as this phase's blocks
// retire; every sweep kernel waits for the whole previous grid (pdl_wait_prior)
// before it reads a site list entry or a link.
template <class... K, class... A>
inline cudaError_t launch_phase(void (*fn)(K...), unsigned grid, unsigned threads, size_t smem, cudaStream_t s,
                         A... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, fn, args...);
}

// Hit-unroll factors the mixed kernels are built for (hits whose draws are
// computed ahead as a group, visit.cuh HitDraws): 1, 2, 5, 10.
inline int hit_unroll_index(int hu) { return hu >= 10 ? 3 : hu >= 5 ? 2 : hu >= 2 ? 1 : 0; }

// Launch shape of a one-wave shared-table sweep: block b takes the chunk
// [b c, (b + 1) c) of the phase's site list with c = ceil(n / grid) (phase_range),
// a compact slab of the lattice, so that the staple loads of neighbouring links
// share L1 lines.  c is ceil(n / SMs), so that every SM gets links, but at least
// min_chunk (a tiny phase uses fewer blocks rather than staging the tables on
// every SM for a few links); the block has c threads rounded up to warps, at
// most max_threads, and walks a larger chunk in turn.
struct PhaseShape {
  unsigned grid, threads;
};

inline PhaseShape phase_shape(uint32_t n, int sms, unsigned max_threads, uint32_t min_chunk = 128) {
  uint32_t c = (n + (uint32_t)sms - 1) / (uint32_t)sms;
  if (c < min_chunk) c = min_chunk;
  PhaseShape sh;
  sh.grid = (unsigned)((n + c - 1) / c);
  sh.threads = std::min<unsigned>(max_threads, std::max<unsigned>(128, (c + 31) / 32 * 32));
  return sh;
}

// The block's chunk of a phase of n links (phase_shape).
__device__ __forceinline__ void phase_range(uint32_t n, uint32_t& lo, uint32_t& hi) {
  const uint32_t c = (n + gridDim.x - 1) / gridDim.x;
  lo = blockIdx.x * c;
  hi = min(n, lo + c);
}

}  // namespace dym
