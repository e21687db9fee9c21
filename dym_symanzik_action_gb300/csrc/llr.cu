// Interval-restricted (LLR) Metropolis sweeps with the Robbins-Monro update,
// on the device, for any number of chains at once.
//
// The reference (llr.cpp:178-250) updates links one at a time because the
// window constraint is on the global energy.  Here a colour class moves at
// once, in three kernels per colour-phase slot over a work list of chains:
//  1. k_llr_propose: every link of the class runs nhit Metropolis hits with
//     weight exp(-a dE_w - bg dE_bg) (llr.cpp:211) and no window test; links of
//     one colour share no plaquette or rectangle, so their energy changes add.
//     Outside the window (drive-in) a hit is kept iff it moves the link's
//     running energy towards the window centre (llr.cpp:208-209), and only a
//     deterministic fraction q of the links takes part; after each phase q is
//     set so that the expected move covers the remaining distance.  Each
//     link's change of plaquette and rectangle classes is added to the chain's
//     integer histogram delta.  A warp takes a tile of 32 links, so a short
//     work list still reaches every SM (the FP64 pipe bounds this kernel).
//  2. k_llr_commit: one warp per chain forms the energies after the class
//     move from the histograms plus the delta and keeps the move iff the new
//     windowed energy lies in [Elo, Ehi] (outside the window: iff it is closer
//     to the centre); it folds a kept delta into the histograms, adapts q, and
//     at the end of a sweep advances the drive-in / Robbins-Monro state
//     machine (a += 12/(W^2 (m+1)) (<E> - Ewin), llr.cpp:244).
//  3. k_llr_restore: the links of a refused class move get their old values.
// NHIT identical single-hit Metropolis kernels compose into a reversible
// kernel, so accepting the class move iff it stays in the window is an exact
// Metropolis-Hastings step for the window-restricted distribution.  Every
// chain's state (Philox sweep counter, delta parity, energies) lives in its
// own LlrState, so a chain gives the same result alone or in any mix.
#include <cuda_runtime.h>

#include "batch.h"
#include "chain.h"
#include "dym_core.h"
#include "staples.cuh"
#include "visit.cuh"

namespace dym {

namespace {

// Squared normalised distance of (e1, e2) to a two-dimensional cell's centre
// (the reference compares hypot() of the same terms, llr2d.cpp:207-209).
__device__ __forceinline__ double norm_sq(const LlrState* st, double e1, double e2) {
  const double x = DYM_MUL(DYM_SUB(e1, st->emid), st->ihw[0]);
  const double y = DYM_MUL(DYM_SUB(e2, st->emid2), st->ihw[1]);
  return DYM_ADD(DYM_MUL(x, x), DYM_MUL(y, y));
}

__device__ __forceinline__ bool in_box(const LlrState* st, double e1, double e2) {
  return e1 >= st->elo && e1 <= st->ehi && e2 >= st->elo2 && e2 <= st->ehi2;
}

__device__ __forceinline__ uint32_t q_threshold(double q) {
  const double t = DYM_MUL(q, 4294967296.0);
  return t >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)t;
}

template <int D>
__global__ void __launch_bounds__(kLlrWarps * 32) k_llr_propose(const LlrTile* __restrict__ tiles, uint32_t ntiles,
                                                                const LlrChainDev* __restrict__ chains,
                                                                BatchGroups groups, int nhit) {
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  int* s_delta = reinterpret_cast<int*>(smem) + warp * 2 * kLlrMaxCls;  // this warp's class deltas
  for (uint32_t x = lane; x < 2 * kLlrMaxCls; x += 32) s_delta[x] = 0;
  for (int g = 0; g < groups.n; ++g) {
    const BatchGroupDev& G = groups.g[g];
    stage_sub_tables(G.retr, G.inv, G.sub, G.P, G.npool, reinterpret_cast<double*>(smem + G.off_retr),
                     reinterpret_cast<uint16_t*>(smem + G.off_inv), reinterpret_cast<uint16_t*>(smem + G.off_sub));
    uint16_t* s_cls = reinterpret_cast<uint16_t*>(smem + G.off_cls);
    for (uint32_t t = threadIdx.x; t < G.P; t += blockDim.x) s_cls[t] = G.cls16[t];
  }
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
    const double* s_retr = reinterpret_cast<const double*>(smem + G.off_retr);
    const uint16_t* s_inv = reinterpret_cast<const uint16_t*>(smem + G.off_inv);
    const uint16_t* s_sub = reinterpret_cast<const uint16_t*>(smem + G.off_sub);
    const uint16_t* s_cls = reinterpret_cast<const uint16_t*>(smem + G.off_cls);
    const int axis = st->axis;
    const double aa = st->a, bg = st->bg, emid = st->emid, E0 = st->E[axis - 1];
    const LlrDrive2 d2{st->dims, st->E[1], st->emid2, st->ihw[0], st->ihw[1]};
    const bool drive = (mode == DYM_LLR_DRIVE);
    const uint32_t qthr = drive ? q_threshold(st->qp[st->phase % (uint32_t)st->nphase]) : 0u;
    const uint32_t sweep = st->sweep;
    unsigned hits = 0, accs = 0;
    if (lane < tl.count) {
      const uint32_t i = c.sites[tl.begin + lane];
      uint32_t b0 = 0;
      switch (tl.dir) {
        case 0: b0 = visit_llr<D, 0>(a, i, sweep, s_retr, s_inv, s_sub, s_cls, axis, aa, bg, E0, emid, d2, drive, qthr,
                                     s_delta, hits, accs); break;
        case 1: b0 = visit_llr<D, 1>(a, i, sweep, s_retr, s_inv, s_sub, s_cls, axis, aa, bg, E0, emid, d2, drive, qthr,
                                     s_delta, hits, accs); break;
        case 2: if (D > 2) b0 = visit_llr<D, (D > 2 ? 2 : 0)>(a, i, sweep, s_retr, s_inv, s_sub, s_cls, axis, aa,
                                                               bg, E0, emid, d2, drive, qthr, s_delta, hits, accs);
          break;
        case 3: if (D > 3) b0 = visit_llr<D, (D > 3 ? 3 : 0)>(a, i, sweep, s_retr, s_inv, s_sub, s_cls, axis, aa,
                                                               bg, E0, emid, d2, drive, qthr, s_delta, hits, accs);
          break;
      }
      c.oldv[tl.pos + lane] = (uint16_t)b0;
    }
    hits = __reduce_add_sync(0xffffffffu, hits);
    accs = __reduce_add_sync(0xffffffffu, accs);
    if (lane == 0) {
      if (hits) atomicAdd(&st->hits, (unsigned long long)hits);
      if (accs) atomicAdd(&st->accepts, (unsigned long long)accs);
    }
    __syncwarp();  // every lane's shared-memory deltas are in
    const uint32_t buf = st->phase & 1u;
    for (uint32_t x = lane; x < 2 * kLlrMaxCls; x += 32) {
      const int v = s_delta[x];
      if (v) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&st->d[buf][x / kLlrMaxCls][x % kLlrMaxCls]),
                  (unsigned long long)(long long)v);
        s_delta[x] = 0;
      }
    }
    __syncwarp();
  }
}

// After the commit: the links of a refused class move get their old values.
__global__ void k_llr_restore(const LlrTile* __restrict__ tiles, uint32_t ntiles,
                              const LlrChainDev* __restrict__ chains) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t stride = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < ntiles; t += stride) {
    const LlrTile tl = tiles[t];
    const LlrChainDev c = chains[tl.chain];
    if (!c.st->restore || lane >= tl.count) continue;
    const uint32_t i = c.sites[tl.begin + lane];
    uint16_t* own = c.links + (size_t)tl.dir * c.V + i;
    const uint16_t old = c.oldv[tl.pos + lane];
    if (*own != old) *own = old;
  }
}

// One warp per chain whose phase the slot closes.  The lanes form the class
// products (h + d) v of both histograms at once; lane 0 sums them in class
// order, which gives the oracle's class sums bit for bit, decides the class
// move from them, and runs the chain's state machine.
__global__ void k_llr_commit(const LlrCommit* __restrict__ commits, uint32_t n,
                             const LlrChainDev* __restrict__ chains) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t idx = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (idx >= n) return;  // the same for every lane of the warp
  const LlrCommit cm = commits[idx];
  LlrState* st = chains[cm.chain].st;
  int mode = st->mode;
  if (mode >= DYM_LLR_DONE) {
    if (lane == 0) st->restore = 0;
    return;
  }
  const uint32_t buf = st->phase & 1u;
  const int ncls = st->ncls;
  double p1 = 0, p2 = 0;
  long long n1 = 0, n2 = 0;
  if ((int)lane < ncls) {
    n1 = st->h[0][lane] + st->d[buf][0][lane];
    n2 = st->h[1][lane] + st->d[buf][1][lane];
    p1 = DYM_MUL((double)n1, st->v[lane]);
    p2 = DYM_MUL((double)n2, st->v[lane]);
  }
  double En1 = 0, En2 = 0;  // the energies after the class move
  for (int c = 0; c < ncls; ++c) {
    En1 = DYM_ADD(En1, __shfl_sync(0xffffffffu, p1, c));
    En2 = DYM_ADD(En2, __shfl_sync(0xffffffffu, p2, c));
  }
  const int w = st->axis - 1;
  const double Eo1 = st->E[0], Eo2 = st->E[1];
  const double Enw = w ? En2 : En1, Eow = w ? Eo2 : Eo1;
  bool ok;
  if (st->dims == 2) {
    ok = mode == DYM_LLR_DRIVE ? norm_sq(st, En1, En2) < norm_sq(st, Eo1, Eo2) : in_box(st, En1, En2);
  } else {
    ok = mode == DYM_LLR_DRIVE ? fabs(DYM_SUB(Enw, st->emid)) < fabs(DYM_SUB(Eow, st->emid))
                               : (Enw >= st->elo && Enw <= st->ehi);
  }
  if (ok && (int)lane < ncls) {
    st->h[0][lane] = n1;
    st->h[1][lane] = n2;
  }
  for (uint32_t x = lane; x < (uint32_t)kLlrMaxCls; x += 32) {
    st->d[buf][0][x] = 0;
    st->d[buf][1][x] = 0;
  }
  if (lane != 0) return;
  const double dE = DYM_SUB(Enw, Eow), dE2 = DYM_SUB(En2, Eo2);
  st->restore = ok ? 0 : 1;
  if (ok) {
    st->E[0] = En1;
    st->E[1] = En2;
    st->phase_acc++;
  } else {
    st->phase_rej++;
  }
  const uint32_t pidx = st->phase % (uint32_t)st->nphase;
  st->phase++;
  if (mode == DYM_LLR_DRIVE) {
    // Aim this phase's next expected move at the remaining distance (in a
    // two-dimensional cell: normalised distance and normalised move).
    double dist, move;
    if (st->dims == 2) {
      dist = sqrt(norm_sq(st, st->E[0], st->E[1]));
      const double x = DYM_MUL(dE, st->ihw[0]), y = DYM_MUL(dE2, st->ihw[1]);
      move = sqrt(DYM_ADD(DYM_MUL(x, x), DYM_MUL(y, y)));
    } else {
      dist = fabs(DYM_SUB(st->emid, st->E[w]));
      move = fabs(dE);
    }
    const double qo = st->qp[pidx];
    const double q = move > 0 ? DYM_MUL(qo, dist / move) : DYM_MUL(qo, 2.0);
    st->qp[pidx] = fmin(1.0, fmax(q, 0x1.0p-32));
    const bool in = st->dims == 2 ? in_box(st, st->E[0], st->E[1]) : (st->E[w] >= st->elo && st->E[w] <= st->ehi);
    if (in) mode = DYM_LLR_SETTLE;
  }
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

}  // namespace

void* llr_propose_kernel_for(int D) { return D == 4 ? (void*)k_llr_propose<4> : nullptr; }

cudaError_t launch_llr_slot(int D, const LlrTile* tiles, uint32_t ntiles, const LlrCommit* commits, uint32_t ncommit,
                            const LlrChainDev* chains, const BatchGroups& groups, int nhit, unsigned grid,
                            size_t smem, cudaStream_t s) {
  if (D != 4) return cudaErrorInvalidValue;  // four dimensions only (see launch_sweep_sub)
  if (ntiles) {
    const unsigned g = grid < ntiles ? grid : ntiles;
    k_llr_propose<4><<<g, kLlrWarps * 32, smem, s>>>(tiles, ntiles, chains, groups, nhit);
  }
  if (ncommit) k_llr_commit<<<(ncommit + 3) / 4, 128, 0, s>>>(commits, ncommit, chains);
  if (ntiles) k_llr_restore<<<(ntiles + 7) / 8, 256, 0, s>>>(tiles, ntiles, chains);
  return cudaGetLastError();
}

}  // namespace dym
