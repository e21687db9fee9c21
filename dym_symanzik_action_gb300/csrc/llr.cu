// Interval-restricted (LLR) Metropolis sweeps with the Robbins-Monro update,
// on the device, for any number of chains at once.
//
// The reference (llr.cpp:178-250) updates links one at a time and tests the
// window on the global energy after every hit.  Here a colour class moves in
// three kernels per colour-phase slot over a work list of chains:
//  1. k_llr_propose: every link of the class runs nhit Metropolis hits with
//     weight exp(-a dE_w - bg dE_bg) (llr.cpp:211) and no window test; outside
//     the window (drive-in) a hit is kept iff it moves the link's running
//     energy towards the window centre (llr.cpp:208-209).  Links of one colour
//     share no plaquette or rectangle, so each link's energy change is its own:
//     the kernel records each link's old value and, per block of st->blk
//     consecutive links, the exact fixed-point sum of their changes.  A warp
//     takes a tile of 32 links, so a short work list still reaches every SM
//     (the FP64 pipe bounds this kernel).
//  2. k_llr_commit: one warp per chain scans the phase's blocks in site-list
//     order and keeps a block's moves iff the running energy plus their change
//     stays in the window (outside it: iff it comes closer to the centre),
//     then advances the drive-in / Robbins-Monro state machine at the end of
//     a sweep (a += 12/(W^2 (m+1)) (<E> - Ewin), llr.cpp:244).
//  3. k_llr_restore: the changed links of refused blocks get their old values.
// A link's nhit identical single-hit Metropolis kernels compose into a
// reversible kernel, so keeping a block's moves iff the energy stays in the
// window is an exact Metropolis-Hastings step for the window-restricted
// distribution, and the scan is a composition of such steps.  A block's
// largest possible change is a quarter of the window width
// (dym_llr_block_links), so a block can always move away from a wall; on
// narrow windows a block is one link.  Energies are exact 64-bit fixed-point
// sums of the class values, so the tracked energy never drifts.  Every
// chain's state (Philox sweep counter, energies) lives in its own LlrState,
// so a chain gives the same result alone or in any mix.
#include <cuda_runtime.h>

#include <climits>

#include "batch.h"
#include "chain.h"
#include "dym_core.h"
#include "staples.cuh"
#include "visit.cuh"

namespace dym {

namespace {

// Fixed-point window tests of the scan (chain.h LlrState).
__device__ __forceinline__ bool llr_in(const LlrState* st, long long e1, long long e2) {
  if (st->dims == 2) return e1 >= st->wlo[0] && e1 <= st->whi[0] && e2 >= st->wlo[1] && e2 <= st->whi[1];
  const long long e = st->axis == 1 ? e1 : e2;
  return e >= st->wlo[0] && e <= st->whi[0];
}

__device__ __forceinline__ double llr_nsq(const LlrState* st, long long e1, long long e2) {
  const double x = DYM_MUL((double)(e1 - st->wmid[0]), st->wsc[0]);
  const double y = DYM_MUL((double)(e2 - st->wmid[1]), st->wsc[1]);
  return DYM_ADD(DYM_MUL(x, x), DYM_MUL(y, y));
}

__device__ __forceinline__ bool llr_closer(const LlrState* st, long long e1, long long e2, long long p1, long long p2) {
  if (st->dims == 2) return llr_nsq(st, e1, e2) < llr_nsq(st, p1, p2);
  const long long e = st->axis == 1 ? e1 : e2, p = st->axis == 1 ? p1 : p2;
  return llabs(e - st->wmid[0]) < llabs(p - st->wmid[0]);
}

// Inclusive prefix sum within aligned segments of `seg` lanes (a power of
// two up to 32; exact: 64-bit integers).
__device__ __forceinline__ long long seg_prefix(long long x, uint32_t lane, uint32_t seg) {
#pragma unroll
  for (uint32_t o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (o < seg && (lane & (seg - 1)) >= o) x += y;
  }
  return x;
}

template <int D>
__global__ void __launch_bounds__(kLlrWarps * 32) k_llr_propose(const LlrTile* __restrict__ tiles, uint32_t ntiles,
                                                                const LlrChainDev* __restrict__ chains,
                                                                const __grid_constant__ BatchGroups groups, int nhit) {
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (int g = 0; g < groups.n; ++g) {  // packed sub-table by cp.async (16-byte aligned on both sides)
    const BatchGroupDev& G = groups.g[g];
    const uint32_t nsub = G.npool * G.P * (G.wide ? 2u : 1u), nb16 = (nsub * 2u) & ~15u;  // halfwords
    uint16_t* s_sub = reinterpret_cast<uint16_t*>(smem + G.off_sub);
    cp_async_stage(s_sub, G.sub, nb16);
    for (uint32_t t = nb16 / 2 + threadIdx.x; t < nsub; t += blockDim.x) s_sub[t] = G.sub[t];
    int32_t* s_cv = reinterpret_cast<int32_t*>(smem + G.off_ev);
    if (threadIdx.x < kLlrMaxCls) s_cv[threadIdx.x] = G.ev[threadIdx.x];
    uint16_t* s_inv = reinterpret_cast<uint16_t*>(smem + G.off_inv);
    uint16_t* s_cls = reinterpret_cast<uint16_t*>(smem + G.off_cls);
    for (uint32_t t = threadIdx.x; t < G.P; t += blockDim.x) {
      s_inv[t] = G.inv[t];
      s_cls[t] = G.cls16[t];
    }
  }
  // The tables are constant: they were staged while the previous kernel of the
  // stream (the last slot's restore) ran; its links and chain states are read
  // from here on.
  pdl_launch_dependents();
  pdl_wait_prior();
  cp_async_wait_all();
  __syncthreads();
  // Tile t goes to warp t / gridDim.x of block t % gridDim.x: a short list
  // spreads over the SMs (one warp each) before any SM takes a second tile.
  const uint32_t stride = (blockDim.x >> 5) * gridDim.x;
  for (uint32_t t = warp * gridDim.x + blockIdx.x; t < ntiles; t += stride) {
    const LlrTile tl = tiles[t];
    const LlrChainDev c = chains[tl.chain];
    LlrState* st = c.st;
    const int mode = st->mode;
    if (mode >= DYM_LLR_DONE) continue;  // the same for every lane of the warp
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
    a.seed = c.seed;
    a.nhit = nhit;
    const int32_t* s_cv = reinterpret_cast<const int32_t*>(smem + G.off_ev);
    const uint16_t* s_inv = reinterpret_cast<const uint16_t*>(smem + G.off_inv);
    const unsigned char* s_sub = smem + G.off_sub;
    const uint16_t* s_cls = reinterpret_cast<const uint16_t*>(smem + G.off_cls);
    const int axis = st->axis;
    const double aa = st->a, bg = st->bg;
    const bool drive = (mode == DYM_LLR_DRIVE);
    LlrDrive dr;
    dr.dims = st->dims;
    dr.axis = axis;
    if (drive) {
      dr.E[0] = st->Ef[0];
      dr.E[1] = st->Ef[1];
      dr.mid[0] = st->wmid[0];
      dr.mid[1] = st->wmid[1];
      dr.sc[0] = st->wsc[0];
      dr.sc[1] = st->wsc[1];
    }
    const uint32_t sweep = st->sweep;
    unsigned hits = 0, accs = 0;
    long long de1 = 0, de2 = 0;
    bool changed = false;
    if (lane < tl.count) {
      const uint32_t i = c.sites[tl.begin + lane];
      uint32_t b0 = 0;
      // The packed entries' width is the group's (uniform across the warp).
#define DYM_LLR_VISIT(DD, E)                                                                                   \
  visit_llr<D, DD, E>(a, i, sweep, s_cv, G.evshift, s_inv, reinterpret_cast<const E*>(s_sub), s_cls, st->vf, \
                      axis, aa, bg, dr, drive, de1, de2, hits, accs)
      switch (tl.dir) {
        case 0: b0 = G.wide ? DYM_LLR_VISIT(0, uint32_t) : DYM_LLR_VISIT(0, uint16_t); break;
        case 1: b0 = G.wide ? DYM_LLR_VISIT(1, uint32_t) : DYM_LLR_VISIT(1, uint16_t); break;
        case 2:
          if (D > 2) b0 = G.wide ? DYM_LLR_VISIT((D > 2 ? 2 : 0), uint32_t) : DYM_LLR_VISIT((D > 2 ? 2 : 0), uint16_t);
          break;
        case 3:
          if (D > 3) b0 = G.wide ? DYM_LLR_VISIT((D > 3 ? 3 : 0), uint32_t) : DYM_LLR_VISIT((D > 3 ? 3 : 0), uint16_t);
          break;
      }
#undef DYM_LLR_VISIT
      changed = c.links[(size_t)tl.dir * c.V + i] != (uint16_t)b0;
      LlrLinkRec r;
      r.site = i;
      r.old = (uint16_t)b0;
      r.changed = changed;
      c.rec[tl.pos + lane] = r;
    }
    // Block records: tiles start at multiples of 32 and blocks of st->blk
    // (a power of two up to 32) links never straddle them; lanes past the
    // phase's end add nothing.
    {
      const uint32_t blk = (uint32_t)st->blk;
      const long long p1 = seg_prefix(de1, lane, blk), p2 = seg_prefix(de2, lane, blk);
      const uint32_t chg = __ballot_sync(0xffffffffu, changed);
      if ((lane & (blk - 1)) == blk - 1 && (lane & ~(blk - 1)) < tl.count) {
        const uint32_t segmask = (blk == 32 ? 0xffffffffu : ((1u << blk) - 1u)) << (lane & ~(blk - 1));
        LlrBlockRec b;
        b.s[0] = p1;
        b.s[1] = p2;
        b.nchg = __popc(chg & segmask);
        b.pad = 0;
        c.brec[(tl.pos + lane) / blk] = b;
      }
    }
    hits = __reduce_add_sync(0xffffffffu, hits);
    accs = __reduce_add_sync(0xffffffffu, accs);
    if (lane == 0) {
      if (hits) atomicAdd(&st->hits, (unsigned long long)hits);
      if (accs) atomicAdd(&st->accepts, (unsigned long long)accs);
    }
  }
}

// One warp per chain whose phase the slot closes: the scan of the phase's
// blocks in site-list order, 32 block records per load (the next 32 loading
// meanwhile).  A block with changed links is kept iff the running energy plus
// its change stays in the window (in the drive-in: iff it comes closer to the
// centre); refused blocks are flagged for k_llr_restore.  Lane 0 then
// advances the chain's state machine.
__global__ void k_llr_commit(const LlrCommit* __restrict__ commits, uint32_t n,
                             const LlrChainDev* __restrict__ chains) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t idx = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (idx >= n) return;  // the same for every lane of the warp
  const LlrCommit cm = commits[idx];  // constant: read before the propose kernel has finished
  const LlrChainDev c = chains[cm.chain];
  pdl_launch_dependents();
  pdl_wait_prior();
  LlrState* st = c.st;
  int mode = st->mode;
  if (mode >= DYM_LLR_DONE) {
    if (lane == 0) st->restore = 0;
    return;
  }
  const bool drive = (mode == DYM_LLR_DRIVE);
  const bool box = st->dims == 2;
  const int w = st->axis - 1;
  const long long lo0 = st->wlo[0], hi0 = st->whi[0], mid0 = st->wmid[0];
  const long long lo1 = st->wlo[1], hi1 = st->whi[1], mid1 = st->wmid[1];
  const double sc0 = st->wsc[0], sc1 = st->wsc[1];
  // The scan's tests (llr_in, llr_closer) on register copies of the window.
  auto in_win = [&](long long e1, long long e2) -> bool {
    if (box) return e1 >= lo0 && e1 <= hi0 && e2 >= lo1 && e2 <= hi1;
    const long long e = w ? e2 : e1;
    return e >= lo0 && e <= hi0;
  };
  auto closer = [&](long long e1, long long e2, long long q1, long long q2) -> bool {
    if (box) {
      const double x = DYM_MUL((double)(e1 - mid0), sc0), y = DYM_MUL((double)(e2 - mid1), sc1);
      const double u = DYM_MUL((double)(q1 - mid0), sc0), v = DYM_MUL((double)(q2 - mid1), sc1);
      return DYM_ADD(DYM_MUL(x, x), DYM_MUL(y, y)) < DYM_ADD(DYM_MUL(u, u), DYM_MUL(v, v));
    }
    const long long e = w ? e2 : e1, q = w ? q2 : q1;
    return llabs(e - mid0) < llabs(q - mid0);
  };
  const uint32_t blk = (uint32_t)st->blk, lb = (uint32_t)(__ffs((int)blk) - 1);
  const uint32_t nblocks = (cm.count + blk - 1) >> lb;
  long long R1 = st->Ef[0], R2 = st->Ef[1];
  unsigned kept = 0, refused = 0;
  LlrBlockRec br{};
  if (lane < nblocks) br = c.brec[lane];
  for (uint32_t wave = 0; wave < nblocks; wave += 32) {
    LlrBlockRec next{};  // the next 32 block records, in flight meanwhile
    if (wave + 32 + lane < nblocks) next = c.brec[wave + 32 + lane];
    const uint32_t nj = nblocks - wave < 32 ? nblocks - wave : 32;
    uint32_t refused_blocks = 0;
    if (!drive) {
      // All 32 kept when every running energy, every block kept, stays in the
      // window (then the serial walk keeps each one in turn).
      const long long p1 = seg_prefix(br.s[0], lane, 32), p2 = seg_prefix(br.s[1], lane, 32);
      if (__all_sync(0xffffffffu, br.nchg == 0 || in_win(R1 + p1, R2 + p2))) {
        kept += __reduce_add_sync(0xffffffffu, br.nchg);
        R1 += __shfl_sync(0xffffffffu, p1, 31);
        R2 += __shfl_sync(0xffffffffu, p2, 31);
        if (lane < nj) c.bref[wave + lane] = 0;
        br = next;
        continue;
      }
    }
    if (!drive) {
      // In the window: the same walk without branches (the keep bit selects).
      const long long lo2 = box ? lo1 : LLONG_MIN, hi2 = box ? hi1 : LLONG_MAX;
      const long long loA = (box || !w) ? lo0 : LLONG_MIN, hiA = (box || !w) ? hi0 : LLONG_MAX;
      const long long loB = box ? lo2 : (w ? lo0 : LLONG_MIN), hiB = box ? hi2 : (w ? hi0 : LLONG_MAX);
#pragma unroll 8
      for (uint32_t j = 0; j < 32; ++j) {
        const uint32_t nch = j < nj ? __shfl_sync(0xffffffffu, br.nchg, j) : 0u;
        const long long s1 = __shfl_sync(0xffffffffu, br.s[0], j), s2 = __shfl_sync(0xffffffffu, br.s[1], j);
        const long long e1 = R1 + s1, e2 = R2 + s2;
        const bool ok = e1 >= loA && e1 <= hiA && e2 >= loB && e2 <= hiB;
        const bool keep = nch != 0u && ok, drop = nch != 0u && !ok;
        R1 = keep ? e1 : R1;
        R2 = keep ? e2 : R2;
        kept += keep ? nch : 0u;
        refused += drop ? nch : 0u;
        refused_blocks |= drop ? (1u << j) : 0u;
      }
    } else {
#pragma unroll 8
      for (uint32_t j = 0; j < 32; ++j) {
        const uint32_t nch = __shfl_sync(0xffffffffu, br.nchg, j);
        const long long s1 = __shfl_sync(0xffffffffu, br.s[0], j), s2 = __shfl_sync(0xffffffffu, br.s[1], j);
        if (j < nj && nch) {  // the same for every lane
          const long long e1 = R1 + s1, e2 = R2 + s2;
          if (closer(e1, e2, R1, R2)) {
            R1 = e1;
            R2 = e2;
            kept += nch;
          } else {
            refused += nch;
            refused_blocks |= 1u << j;
          }
        }
      }
    }
    if (lane < nj) c.bref[wave + lane] = (uint8_t)((refused_blocks >> lane) & 1u);
    br = next;
  }
  if (lane != 0) return;
  st->restore = refused ? 1 : 0;
  st->Ef[0] = R1;
  st->Ef[1] = R2;
  st->E[0] = DYM_MUL((double)R1, 0x1p-32);
  st->E[1] = DYM_MUL((double)R2, 0x1p-32);
  st->phase_acc += kept;
  st->phase_rej += refused;
  st->phase++;
  if (mode == DYM_LLR_DRIVE && llr_in(st, R1, R2)) mode = DYM_LLR_SETTLE;
  if (cm.last) {
    st->sweeps++;
    st->sweep++;
    if (mode == DYM_LLR_DRIVE) {
      if (++st->drive_sweeps >= st->drive_cap) mode = DYM_LLR_UNREACHED;
    } else if (mode == DYM_LLR_SETTLE) {
      mode = st->NRM > 0 ? DYM_LLR_RM : DYM_LLR_DONE;  // NRM = 0: drive-in only (seed_cell)
      st->k = 0;
      st->m = 0;
      st->sumE = 0;
      st->sumE2 = 0;
    } else if (mode == DYM_LLR_RM) {
      st->sumE = DYM_ADD(st->sumE, st->E[w]);
      if (st->dims == 2) st->sumE2 = DYM_ADD(st->sumE2, st->E[1]);
      if (++st->k == st->K) {
        const double g = DYM_SUB(st->sumE / (double)st->K, st->ewin);
        const double step = 12.0 / DYM_MUL(st->w2, (double)(st->m + 1));
        st->a = DYM_ADD(st->a, DYM_MUL(step, g));
        st->a_hist[st->m] = st->a;
        if (st->dims == 2) {  // llr2d.cpp:252-253
          const double g2 = DYM_SUB(st->sumE2 / (double)st->K, st->ewin2);
          const double step2 = 12.0 / DYM_MUL(st->w2b, (double)(st->m + 1));
          st->bg = DYM_ADD(st->bg, DYM_MUL(step2, g2));
          st->a2_hist[st->m] = st->bg;
        }
        st->m++;
        st->k = 0;
        st->sumE = 0;
        st->sumE2 = 0;
        if (st->m >= st->NRM) mode = DYM_LLR_DONE;
      }
    }
  }
  st->mode = mode;
}

// After the commit: the changed links of refused blocks get their old values
// (a warp per propose tile, so every SM takes part).
__global__ void k_llr_restore(const LlrTile* __restrict__ tiles, uint32_t ntiles,
                              const LlrChainDev* __restrict__ chains) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t stride = (gridDim.x * blockDim.x) >> 5;
  pdl_launch_dependents();
  pdl_wait_prior();  // the commit's flags and states
  for (uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < ntiles; t += stride) {
    const LlrTile tl = tiles[t];
    const LlrChainDev c = chains[tl.chain];
    if (!c.st->restore || lane >= tl.count) continue;
    const uint32_t pos = tl.pos + lane;
    const uint32_t lb = (uint32_t)(__ffs(c.st->blk) - 1);
    if (!c.bref[pos >> lb]) continue;
    const LlrLinkRec r = c.rec[pos];
    if (r.changed) c.links[(size_t)tl.dir * c.V + r.site] = r.old;
  }
}

// Launch, with programmatic stream serialization when `pdl`: each of a slot's
// kernels may then start its constant prologue (the propose kernel: table
// staging) while the previous kernel drains, and waits for it (pdl_wait_prior)
// before it reads links or chain states.  Without the attribute the waits are
// no-ops and the stream orders the kernels.
template <class... K, class... A>
cudaError_t launch_pdl(bool pdl, void (*fn)(K...), unsigned grid, unsigned threads, size_t smem, cudaStream_t s,
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
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, fn, args...);
}

}  // namespace

void* llr_propose_kernel_for(int D) { return D == 4 ? (void*)k_llr_propose<4> : nullptr; }

cudaError_t launch_llr_slot(int D, const LlrTile* tiles, uint32_t ntiles, const LlrCommit* commits, uint32_t ncommit,
                            const LlrChainDev* chains, const BatchGroups& groups, int nhit, unsigned grid,
                            size_t smem, cudaStream_t s) {
  if (D != 4) return cudaErrorInvalidValue;  // four dimensions only (see launch_sweep_sub)
  // Overlap the launches only when a slot is short (at most one tile per warp
  // of the propose grid): then the gaps between its three kernels are a large
  // part of it; on a loaded work list the early propose blocks cost more than
  // they hide (measured on the served stream).
  const bool pdl = ntiles <= (size_t)grid * kLlrWarps;
  cudaError_t e = cudaSuccess;
  if (ntiles) {
    const unsigned g = grid < ntiles ? grid : ntiles;
    e = launch_pdl(pdl, k_llr_propose<4>, g, kLlrWarps * 32, smem, s, tiles, ntiles, chains, groups, nhit);
  }
  if (e == cudaSuccess && ncommit)
    e = launch_pdl(pdl, k_llr_commit, (ncommit + 3) / 4, 128, 0, s, commits, ncommit, chains);
  if (e == cudaSuccess && ntiles) e = launch_pdl(pdl, k_llr_restore, (ntiles + 7) / 8, 256, 0, s, tiles, ntiles, chains);
  return e;
}

}  // namespace dym
