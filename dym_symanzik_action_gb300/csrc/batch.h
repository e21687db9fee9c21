// Device descriptors of the batched ensemble (internal).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace dym {

struct BatchChainDev {
  uint16_t* links;
  const uint32_t* sites;
  uint32_t V;
  int Nt, Nx;
  int group;
  double beta0, beta1, beta2;
  uint64_t seed;
  unsigned long long* ctr;  // [hits, accepts] of this chain
};

struct BatchGroupDev {
  const uint16_t* mult;
  const uint16_t* inv;
  const double* retr;
  const uint16_t* sub;  // sub[k][u] = u * pool[k]
  uint32_t P, npool;
  uint32_t off_retr, off_inv, off_sub;  // byte offsets of the staged copies in shared memory
};

constexpr int kBatchMaxGroups = 4;
struct BatchGroups {
  BatchGroupDev g[kBatchMaxGroups];
  int n;
};

struct BatchTile {
  uint32_t chain, begin, count, dir;
};

void* batch_kernel_for(int D);
cudaError_t launch_batch_slot(int D, const BatchTile* tiles, uint32_t ntiles, const BatchChainDev* chains,
                              const BatchGroups& groups, const uint32_t* sweeps, int nhit, unsigned grid,
                              unsigned threads, size_t smem, cudaStream_t s);
cudaError_t launch_batch_advance(uint32_t* sweeps, uint32_t n, cudaStream_t s);

}  // namespace dym
