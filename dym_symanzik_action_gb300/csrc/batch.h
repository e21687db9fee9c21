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
  unsigned long long* ctr;  // [hits, accepts, rechecks, max |dS error| bits] of this chain
  float b1f, b2f, dmargin;  // mixed-precision kernel: FP32 betas, error bound at these betas
  const uint32_t* xyz;      // mixed-precision kernel: packed coordinates of sites[k]
};

struct BatchGroupDev {
  const uint16_t* mult;
  const uint16_t* inv;
  const double* retr;
  const uint16_t* sub;  // sub[k][u] = u * pool[k]
  const uint16_t* cls16;  // ReTr class of each element (LLR only)
  const int32_t* ev;      // LLR: each class's ReTr times 2^evshift, rounded (dym_fix_shift); kLlrMaxCls
  int evshift;
  int wide;               // LLR: sub holds 32-bit entries element | class << 16 (P > 2048), else 16-bit
                          // element | class << 11
  uint32_t P, npool;
  uint32_t off_retr, off_inv, off_sub, off_cls;  // byte offsets of the staged copies in shared memory
  uint32_t off_ev;                               // LLR: staged class values (off_retr is unused there)
  // Mixed-precision kernel: sub holds packed entries (element | class << 11),
  // cls8 the class of each element, cfix the fixed-point class values.
  const uint8_t* cls8;
  const int32_t* cfix;
  float dscale;
  uint32_t off_cls8, off_cfix;
};

constexpr int kBatchMaxGroups = 4;
struct BatchGroups {
  BatchGroupDev g[kBatchMaxGroups];
  int n;
};

struct BatchTile {
  uint32_t chain, begin, count, dir;
};

// LLR work lists (llr.cu): per-chain descriptors, tiles of one colour-phase
// slot, and the chains whose phase the slot's commit closes.
struct LlrState;
struct LlrLinkRec;
struct LlrBlockRec;
struct LlrChainDev {
  uint16_t* links;
  const uint32_t* sites;
  uint32_t V;
  int Nt, Nx;
  uint64_t seed;
  LlrState* st;
  LlrLinkRec* rec;    // one per link of the largest phase
  LlrBlockRec* brec;  // one per block of scan links
  uint8_t* bref;      // per block: refused by the scan of this slot
  int group;
};
struct LlrTile {
  uint32_t chain, begin, count, dir, pos;  // pos: offset of the tile inside its phase
};
struct LlrCommit {
  uint32_t chain, last;  // last: this slot holds the chain's last phase of a sweep
  uint32_t count, dir;   // the phase's links and direction
};
void* llr_propose_kernel_for(int D);
cudaError_t launch_llr_slot(int D, const LlrTile* tiles, uint32_t ntiles, const LlrCommit* commits, uint32_t ncommit,
                            const LlrChainDev* chains, const BatchGroups& groups, int nhit, unsigned grid,
                            size_t smem, cudaStream_t s);

void* batch_kernel_for(int D, bool mixed, int hit_unroll);
cudaError_t launch_batch_slot(int D, bool mixed, int hit_unroll, const BatchTile* tiles, uint32_t ntiles,
                              const BatchChainDev* chains, const BatchGroups& groups, const uint32_t* sweeps, int nhit,
                              unsigned grid, unsigned threads, size_t smem, cudaStream_t s);
cudaError_t launch_batch_advance(uint32_t* sweeps, uint32_t n, cudaStream_t s);

}  // namespace dym
