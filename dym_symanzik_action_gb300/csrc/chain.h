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
  unsigned long long* counters;  // [0] hits, [1] accepts, [2] rechecks, [3] low word: max |dS error| (FP32 bits)
  unsigned long long* status;    // self-checking build only: first bad index
  // Mixed-precision kernel (k_sweep_mixed): class of each element, class
  // values in fixed point (ReTr * 2^fix_shift, rounded), FP32 betas, 2^-fix_shift
  // and the bound on |dS_fast - dS_fp64| within which a decision is re-evaluated.
  const uint8_t* cls8;
  const int32_t* cfix;
  float b1f, b2f, dscale, dmargin;
  const uint32_t* xyz;  // coordinates of sites[k], 8 bits per axis (already offset)
  const int16_t* val16;  // value-table kernel: fixed-point ReTr of every element
  int hit_unroll;        // mixed kernels: hits per group of draws computed ahead (1, 2, 5 or 10)
  int lanes_per_link;    // value-table kernel: threads sharing a link visit (1 or 2)
  // dym_sweep_host, dym_sweep_refarray: the upload check's word (0 when every
  // id was valid, else the complement of the first bad index); a sweep launch
  // after a refused upload does nothing.  Null for the other calls.
  const unsigned long long* skip;
  // The final sweep of a host-resident call also writes the value of every
  // link it visits into the caller's buffer: `out` direction-major
  // (out[dir*V + site], dym_sweep_host's page-locked host_out through its
  // device mapping), `out_ref` the reference's layout (out_ref[site*D + dir],
  // int32: dym_sweep_refarray's device copy of a pageable array; a
  // page-locked one is written by a coalesced pass instead, since these
  // scattered 4-byte writes are slow over the host link).  Every link is
  // visited once a sweep, so no copy of the configuration follows the sweeps.
  // Null otherwise.
  uint16_t* out;
  int32_t* out_ref;
  // Philox round keys of `seed` (dym_philox_round_keys): the single-chain
  // kernels' hit draws read them as kernel parameters (dym_metro_hit).
  uint32_t rk[20];
};

struct ChainDev {
  int D, Nt, Nx;
  uint32_t V;
  uint16_t* links = nullptr;
  uint32_t* sites = nullptr;
  uint16_t* pool = nullptr;    // proposal pool actually used
  uint32_t npool = 0;
  // [0..4] the sweep counters (SweepArgs::counters), [5] the upload check of
  // dym_links_set / dym_sweep_host / dym_sweep_refarray: 0 when every id was
  // valid, else the complement of the smallest bad index (atomicMax), so one
  // memset clears all six words and one copy reads them back.
  unsigned long long* counters = nullptr;
  uint16_t* sub = nullptr;     // sub[k*P + u] = u * pool[k] (shared sub-table kernel)
  bool sub_ok = false;
  // Mixed-precision kernel: psub[k*P + u] = (u * pool[k]) | class << 11 for
  // P <= 2048; otherwise psub32[k*P + u] = (u * pool[k]) | class << 16.
  uint16_t* psub = nullptr;
  uint32_t* psub32 = nullptr;
  bool mixed_wide = false;
  uint8_t* cls8 = nullptr;
  int32_t* cfix = nullptr;
  int fix_shift = 0;
  bool mixed_ok = false;
  uint32_t* xyz = nullptr;     // packed coordinates of sites[k] (mixed kernel)
  int16_t* vsub = nullptr;     // value-table kernel: vsub[u*npool + k] = ReTr(u * pool[k]) * 2^vt_shift
  int16_t* val16 = nullptr;    // ReTr(u) * 2^vt_shift
  int vt_shift = 0;
  bool vt_ok = false;
  double last_acc = 1.0;       // acceptance of the chain's previous dym_sweep call (kernel choice)
};

// Launch one colour phase of the FP64 direct sweep.
cudaError_t launch_sweep_direct(int D, int dir, const SweepArgs& a, cudaStream_t s);
// Launch one colour phase of the shared sub-table sweep.
cudaError_t launch_sweep_sub(int D, int dir, const SweepArgs& a, const uint16_t* sub, cudaStream_t s);
size_t sub_smem_bytes(uint32_t P, uint32_t npool);
// Launch one colour phase of the mixed-precision shared sub-table sweep.
cudaError_t launch_sweep_mixed(int D, int dir, const SweepArgs& a, const uint16_t* psub, cudaStream_t s);
cudaError_t launch_sweep_mixed_wide(int D, int dir, const SweepArgs& a, const uint32_t* psub, cudaStream_t s);
size_t mixed_smem_bytes(uint32_t P, uint32_t npool, size_t entry = 2);
cudaError_t launch_sweep_vt(int D, int dir, const SweepArgs& a, const int16_t* vsub, cudaStream_t s);
size_t vt_smem_bytes(uint32_t P, uint32_t npool);
// Bytes of the value table vsub[u * npool + k], padded with zeros to a
// multiple of 16 (the unit of its cp.async staging).
__host__ __device__ inline size_t vt_table_bytes(uint32_t P, uint32_t npool) {
  return ((size_t)P * npool * 2 + 15) / 16 * 16;
}
constexpr int kMixedMaxCls = 32;    // classes addressable by the 5 high bits of a psub entry
constexpr uint32_t kMixedMaxP = 2048;  // 16-bit packed entries: element ids in the 11 low bits
constexpr int kMixedMaxExtent = 256;   // coordinates packed 8 bits per axis
constexpr int kMixedMaxThreads = 512;
constexpr int kDefaultHitUnroll = 1;        // element-table kernel (k_sweep_mixed)
constexpr int kDefaultHitUnrollValues = 2;  // value-table kernel (k_sweep_vt): speculative pairs
constexpr int kDefaultLanesPerLink = 1;
// Threads per block of the two-lanes-per-link value-table kernel at most
// (two lanes for each of 448 links; 72 registers a thread).
constexpr int kVt2MaxThreads = 896;
constexpr double kDefaultVtMaxAccept = 0.01;
// Copy n counter words into page-locked host memory (its device mapping) and
// clear them for the next call, behind the previous kernel (programmatic
// serialization): one kernel instead of a copy-engine read-back and a memset.
cudaError_t launch_counters_out(unsigned long long* dev, unsigned long long* host_mapped, int n, cudaStream_t s);
cudaError_t launch_hot_start(uint16_t* links, uint32_t V, int D, uint32_t P, uint64_t seed, cudaStream_t s);
cudaError_t launch_fill(uint16_t* links, size_t n, uint16_t v, cudaStream_t s);
// Check n uploaded ids against P on the device and copy the stage into the
// links only if all are in range.  *first is the check word: 0 beforehand
// (the caller clears it), afterwards the complement of the smallest bad index
// if there is one.
cudaError_t launch_links_commit(uint16_t* links, const uint16_t* stage, size_t n, uint32_t P,
                                unsigned long long* first, cudaStream_t s);
// The same reading the ids from page-locked host memory through its device
// mapping (no copy-engine transfer).
cudaError_t launch_links_from_host(uint16_t* links, uint16_t* stage, const uint16_t* host_mapped, size_t n,
                                   uint32_t P, unsigned long long* first, cudaStream_t s);
// The reference's link array a[i*D + d] (int32 ids, site-major; device
// memory or the device mapping of page-locked host memory): its ids checked
// against P (negative ones too) and narrowed into the stage, direction-major
// (stage[d*V + i]), then committed into the links as launch_links_commit.
cudaError_t launch_links_from_ref(uint16_t* links, uint16_t* stage, const int32_t* ref, uint32_t V, int D, uint32_t P,
                                  unsigned long long* first, cudaStream_t s);
// The links written back into the reference's layout, ref[i*D + d] =
// links[d*V + i] (coalesced writes, for page-locked host arrays); nothing is
// written when the upload check word *skip is set.
cudaError_t launch_links_to_ref(int32_t* ref, const uint16_t* links, uint32_t V, int D,
                                const unsigned long long* skip, cudaStream_t s);
cudaError_t launch_staples(int D, int dir, const SweepArgs& a, const uint32_t* sites, uint32_t n, uint16_t* out,
                           cudaStream_t s);
// Shared memory of k_sweep_mixed: ReTr (FP64) | class values | inverses | packed
// sub-table (entries of `entry` bytes; 32-bit entries start on 16 bytes) | classes.
__host__ __device__ inline size_t mixed_psub_offset(uint32_t P, size_t entry) {
  const size_t o = (size_t)P * 8 + kMixedMaxCls * 4 + (size_t)P * 2;
  return entry == 2 ? o : (o + 15) / 16 * 16;
}

// LLR (interval-restricted sweeps with Robbins-Monro updates): per-chain
// state in device memory, updated by the commit kernel after every colour
// phase.  Energies are exact 64-bit fixed-point sums of the plaquette (Ef[0])
// and rectangle (Ef[1]) class values, each value times 2^kLlrFixShift rounded
// (vf); E holds the same sums as FP64.  The window tests compare fixed-point
// values: wlo/whi/wmid[0] bound the windowed energy (S1 for axis 1, S2 for
// axis 2; S1 of a two-dimensional cell), [1] the S2 window of a cell.
constexpr int kLlrMaxCls = 32;
constexpr int kLlrFixShift = 32;
// The LLR propose kernel runs 512-thread blocks whose warps take 32-link tiles
// independently.
constexpr int kLlrWarps = 16;
constexpr int kLlrTile = 32;
struct LlrState {
  double a, bg, elo, ehi, emid, ewin, w2;
  double E[2];
  double sumE;
  long long Ef[2];
  long long vf[kLlrMaxCls];
  long long wlo[2], whi[2], wmid[2];
  double wsc[2];  // 2^-kLlrFixShift / half-width per axis (two-dimensional drive-in)
  int blk;        // links per block of the scan (dym_llr_block_links)
  int restore;    // set by the commit: some block of the phase was refused, restore its links
  double a_hist[DYM_LLR_MAX_NRM];
  int axis, mode, k, m, K, NRM, drive_sweeps, drive_cap, sweeps;
  uint32_t phase, sweep;  // colour phases committed, Philox sweep counter
  unsigned long long phase_acc, phase_rej, hits, accepts;  // phase_acc/rej: links kept/refused by the scan
  // Two-dimensional cells (dims == 2, llr2d.cpp:178-259): S1 in [elo, ehi] and
  // S2 in [elo2, ehi2] (axis is 1); a is a1 and bg is a2, both updated by
  // Robbins-Monro; ihw are the reciprocal half-widths of the normalised
  // distance to the cell centre used by the drive-in hits.
  int dims;
  double elo2, ehi2, emid2, ewin2, w2b, sumE2;
  double ihw[2];
  double a2_hist[DYM_LLR_MAX_NRM];
};

// What the propose kernel leaves for the scan of the commit kernel: per link
// of the phase (in site-list order) its site, its value before the hits and
// whether they changed it; per block of LlrState::blk consecutive links the
// exact fixed-point sums of the links' changes of S1 and S2 and the number of
// changed links.
struct LlrLinkRec {
  uint32_t site;
  uint16_t old;
  uint16_t changed;
};

struct LlrBlockRec {
  long long s[2];
  uint32_t nchg;
  uint32_t pad;
};

// Drive-in parameters as the propose kernel passes them to visit_llr: the
// phase-start fixed-point energies, the window centre (the windowed axis's in
// index 0; a cell's S2 centre in index 1) and, for a two-dimensional cell,
// 2^-kLlrFixShift over each half-width.
struct LlrDrive {
  int dims, axis;
  long long E[2], mid[2];
  double sc[2];
};

// Observables.
struct MeasArgs {
  const uint16_t* links;
  uint32_t V;
  int D, Nt, Nx;
  const uint16_t* mult;
  const uint16_t* inv;
  uint32_t P, id;
};
// Fresh start configuration and Philox key for an existing chain (capi.cu).
int chain_reset(dym_chain* c, uint64_t seed, int start);

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
  unsigned long long* h_counters_dev = nullptr;  // its device mapping (k_counters_out writes it)
  // Whether the device counter words may be non-zero on entry to a call: a
  // call ends by reading them out and clearing them in one kernel; one that
  // returned before that leaves this set, and the next call clears them first.
  bool counters_dirty = true;
  // Measurement buffers (allocated on first use, sized for the largest grid).
  unsigned long long* d_hist = nullptr;
  size_t hist_elems = 0;
  uint16_t* d_meas_scratch = nullptr;
  size_t meas_scratch_elems = 0;
  unsigned long long* h_hist = nullptr;
  size_t h_hist_elems = 0;
  // LLR state (allocated on first use).
  dym::LlrState* d_llr = nullptr;
  dym::LlrLinkRec* d_llr_rec = nullptr;   // per link of the largest colour phase (rounded up to 32)
  dym::LlrBlockRec* d_llr_blk = nullptr;  // per block of it (as many)
  uint8_t* d_llr_bref = nullptr;          // per block: refused by the last scan
  uint16_t* d_stage = nullptr;  // dym_links_set: upload buffer, copied into the links once checked
  int32_t* d_ref32 = nullptr;   // dym_sweep_refarray: the reference-layout array in device memory (pageable callers)
  bool l2_window = false;  // dym_chain_set_l2_window: the stream pins the Cayley table in L2
};
