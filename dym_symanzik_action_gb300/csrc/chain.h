// Device-resident chain state and kernel launchers (internal).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.h"

struct dym_group {
  dym::Group* g;
};

namespace dym {

// Everything a sweep kernel needs, passed by value.
struct SweepArgs {
  uint16_t* links;          // D*V
  const uint32_t* sites;    // phase site list (already offset)
  uint32_t n;               // links in this phase
  uint32_t V;
  int Nt, Nx;
  const uint16_t* mult;     // P*P
  const uint16_t* inv;      // P
  const double* retr;       // P
  const uint16_t* pool;     // npool
  uint32_t P, npool, id;
  double beta0, beta1, beta2;
  uint64_t seed;
  uint32_t sweep;
  int nhit;
  unsigned long long* counters;  // [0] hits, [1] accepts, [2] rechecks
};

// Shared-memory sub-table path (pool of nearest elements).
struct FastTables {
  uint16_t* sub;            // npool*P entries: (u*g_k) | (cls(u*g_k) << shift)
  uint8_t* cls;             // P: ReTr class of each element
  float* cls_val32;         // ncls
  double* cls_val64;        // ncls
  int ncls;
  int shift;                // bits of the product field
  int exact;                // 1: ReTr constant on classes (bitwise)
  double eps;               // bound on |dS_fp32 - dS_fp64|, set per launch
};

struct ChainDev {
  int D, Nt, Nx;
  uint32_t V;
  uint16_t* links = nullptr;
  uint32_t* sites = nullptr;
  uint16_t* pool = nullptr;    // proposal pool actually used
  uint32_t npool = 0;
  unsigned long long* counters = nullptr;
  double* maxerr = nullptr;    // mixed precision: max |dS err| (bits as u64 atomics)
  FastTables fast{};
  bool fast_ok = false;
};

// Launch one colour phase of the FP64 direct sweep.
cudaError_t launch_sweep_direct(int D, int dir, const SweepArgs& a, cudaStream_t s);
// Launch one colour phase of the mixed-precision shared sub-table sweep.
cudaError_t launch_sweep_fast(int D, int dir, const SweepArgs& a, const FastTables& ft, double* maxerr,
                              cudaStream_t s);
size_t fast_smem_bytes(uint32_t P, uint32_t npool, int ncls);
cudaError_t launch_hot_start(uint16_t* links, uint32_t V, int D, uint32_t P, uint64_t seed, cudaStream_t s);
cudaError_t launch_fill(uint16_t* links, size_t n, uint16_t v, cudaStream_t s);
cudaError_t launch_staples(int D, int dir, const SweepArgs& a, const uint32_t* sites, uint32_t n, uint16_t* out,
                           cudaStream_t s);

// Observables.
struct MeasArgs {
  const uint16_t* links;
  uint32_t V;
  int D, Nt, Nx;
  const uint16_t* mult;
  const uint16_t* inv;
  uint32_t P, id;
};
cudaError_t launch_measure(const MeasArgs& m, int wl_nx, int wl_nt, bool assoc, unsigned long long* hist,
                           uint16_t* scratch, cudaStream_t s);
size_t measure_scratch_elems(const MeasArgs& m, int wl_nx, int wl_nt, bool assoc);
cudaError_t probe_l2_gather(uint32_t table_bytes, double* sectors_per_s);

}  // namespace dym

struct dym_chain {
  dym_group* grp;
  dym_chain_params p;
  dym::Schedule sched;
  dym::ChainDev dev;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // device timing of sweeps
  uint32_t sweep = 0;
  unsigned long long* h_counters = nullptr;  // pinned
  // Measurement buffers (allocated on first use, sized for the largest grid).
  unsigned long long* d_hist = nullptr;
  size_t hist_elems = 0;
  uint16_t* d_meas_scratch = nullptr;
  size_t meas_scratch_elems = 0;
  unsigned long long* h_hist = nullptr;
  size_t h_hist_elems = 0;
};
