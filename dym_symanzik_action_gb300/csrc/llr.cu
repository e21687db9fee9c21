// Interval-restricted (LLR) Metropolis sweeps with the Robbins-Monro update,
// on the device.
//
// The reference (llr.cpp:178-250) updates links one at a time because the
// window constraint is on the global energy.  Here a colour class moves at
// once:
//  1. k_llr_propose: every link of the class runs nhit Metropolis hits with
//     weight exp(-a dE_w - bg dE_bg) (llr.cpp:211) and no window test; links of
//     one colour share no plaquette or rectangle, so their energy changes add.
//     Outside the window (drive-in) a hit is kept iff it moves the link's
//     running energy towards the window centre (llr.cpp:208-209), and only a
//     deterministic fraction q of the links takes part; after each phase q is
//     set so that the expected move covers the remaining distance.  Each link's change of
//     plaquette and rectangle classes is added to an integer histogram delta.
//  2. k_llr_decide: the class move is kept iff the new windowed energy lies in
//     [Elo, Ehi] (outside the window: iff it is closer to the centre);
//     otherwise every link of the class is restored.
//  3. k_llr_commit: one thread folds the delta into the chain's histograms,
//     recomputes the exact energies, adapts q, and at the end of a sweep
//     advances the drive-in / Robbins-Monro state machine
//     (a += 12/(W^2 (m+1)) (<E> - Ewin), llr.cpp:244).
// NHIT identical single-hit Metropolis kernels compose into a reversible
// kernel, so accepting the class move iff it stays in the window is an exact
// Metropolis-Hastings step for the window-restricted distribution.
#include <cuda_runtime.h>

#include "chain.h"
#include "dym_core.h"
#include "staples.cuh"

namespace dym {

namespace {

__device__ __forceinline__ double class_sum(const long long* h, const long long* d, const double* v, int ncls) {
  double s = 0;
  for (int c = 0; c < ncls; ++c) s = DYM_ADD(s, DYM_MUL((double)(h[c] + (d ? d[c] : 0)), v[c]));
  return s;
}

// Whether the class move of the phase with parity `buf` is kept.
__device__ __forceinline__ bool phase_ok(const LlrState* st, int buf) {
  const int w = st->axis - 1;
  const double En = class_sum(st->h[w], st->d[buf][w], st->v, st->ncls);
  if (st->mode == DYM_LLR_DRIVE) return fabs(DYM_SUB(En, st->emid)) < fabs(DYM_SUB(st->E[w], st->emid));
  return En >= st->elo && En <= st->ehi;
}

__device__ __forceinline__ uint32_t q_threshold(double q) {
  const double t = DYM_MUL(q, 4294967296.0);
  return t >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)t;
}

__device__ __forceinline__ void flush_hits(unsigned long long* ctr, unsigned hits, unsigned accs) {
  hits = __reduce_add_sync(0xffffffffu, hits);
  accs = __reduce_add_sync(0xffffffffu, accs);
  if ((threadIdx.x & 31) == 0) {
    if (hits) atomicAdd(ctr + 0, (unsigned long long)hits);
    if (accs) atomicAdd(ctr + 1, (unsigned long long)accs);
  }
}

template <int D, int DIR>
__global__ void __launch_bounds__(256) k_llr_propose(LlrArgs A) {
  constexpr int NS = 2 * (D - 1), NR = 6 * (D - 1);
  const SweepArgs& a = A.s;
  LlrState* st = A.st;
  const int mode = st->mode;
  if (mode >= DYM_LLR_DONE) return;  // the same for every thread of the grid
  extern __shared__ __align__(16) unsigned char smem[];
  double* s_retr = reinterpret_cast<double*>(smem);
  uint16_t* s_inv = reinterpret_cast<uint16_t*>(s_retr + a.P);
  uint16_t* s_cls = s_inv + a.P;
  uint16_t* s_pool = s_cls + a.P;
  int* s_delta = reinterpret_cast<int*>(smem + ((size_t)a.P * 8 + (size_t)a.P * 4 + (size_t)a.npool * 2 + 15) / 16 * 16);
  for (uint32_t t = threadIdx.x; t < a.P; t += blockDim.x) {
    s_retr[t] = a.retr[t];
    s_inv[t] = a.inv[t];
    s_cls[t] = A.cls16[t];
  }
  for (uint32_t t = threadIdx.x; t < a.npool; t += blockDim.x) s_pool[t] = a.pool[t];
  for (uint32_t t = threadIdx.x; t < 2 * kLlrMaxCls; t += blockDim.x) s_delta[t] = 0;
  __syncthreads();

  const int axis = st->axis;
  const double aa = st->a, bg = st->bg, emid = st->emid, E0 = st->E[axis - 1];
  const bool drive = (mode == DYM_LLR_DRIVE);
  const uint32_t qthr = drive ? q_threshold(st->q) : 0u;
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
    uint32_t stp[NS], re[NR];
    build_staples<D, DIR>(i, geo, T, ld, stp, re);
    uint16_t* own = a.links + (size_t)DIR * V + i;
    uint32_t b = *own;
    const uint32_t b0 = b;
    double r1 = 0, m1 = 0;
#pragma unroll
    for (int j = 0; j < NS; ++j) r1 = DYM_ADD(r1, s_retr[T.mul(b, stp[j])]);
#pragma unroll
    for (int k = 0; k < NR; ++k) m1 = DYM_ADD(m1, s_retr[T.mul(b, re[k])]);
    bool part = true;
    if (drive) {
      const dym_u32x4 r = dym_hit_random(a.seed, a.sweep, i, DIR, 0xFFFFFu, DYM_TAG_LLR);
      part = r.v[0] < qthr;
    }
    double cum = 0;
    for (int h = 0; part && h < a.nhit; ++h) {
      const dym_u32x4 r = dym_hit_random(a.seed, a.sweep, i, DIR, (uint32_t)h, DYM_TAG_LLR);
      const uint32_t bnew = T.mul(b, s_pool[dym_pick(r.v[0], a.npool)]);
      double r1n = 0, m1n = 0;
#pragma unroll
      for (int j = 0; j < NS; ++j) r1n = DYM_ADD(r1n, s_retr[T.mul(bnew, stp[j])]);
#pragma unroll
      for (int k = 0; k < NR; ++k) m1n = DYM_ADD(m1n, s_retr[T.mul(bnew, re[k])]);
      const double dS1 = DYM_SUB(r1n, r1), dS2 = DYM_SUB(m1n, m1);
      const double dEw = axis == 1 ? dS1 : dS2;
      const double dEbg = axis == 1 ? dS2 : dS1;
      bool acc;
      if (drive) {
        const double Ec = DYM_ADD(E0, cum);
        acc = fabs(DYM_SUB(DYM_ADD(Ec, dEw), emid)) < fabs(DYM_SUB(Ec, emid));
      } else {
        const double w = dym_exp(DYM_SUB(DYM_MUL(-aa, dEw), DYM_MUL(bg, dEbg)));
        acc = w > dym_u53(r.v[1], r.v[2]);
      }
      ++hits;
      if (acc) {
        b = bnew;
        r1 = r1n;
        m1 = m1n;
        cum = DYM_ADD(cum, dEw);
        ++accs;
      }
    }
    A.oldv[tid] = (uint16_t)b0;
    if (b != b0) {
      *own = (uint16_t)b;
#pragma unroll
      for (int j = 0; j < NS; ++j) {
        atomicAdd(&s_delta[s_cls[T.mul(b0, stp[j])]], -1);
        atomicAdd(&s_delta[s_cls[T.mul(b, stp[j])]], 1);
      }
#pragma unroll
      for (int k = 0; k < NR; ++k) {
        atomicAdd(&s_delta[kLlrMaxCls + s_cls[T.mul(b0, re[k])]], -1);
        atomicAdd(&s_delta[kLlrMaxCls + s_cls[T.mul(b, re[k])]], 1);
      }
    }
  }
  flush_hits(a.counters, hits, accs);
  __syncthreads();
  for (uint32_t t = threadIdx.x; t < 2 * kLlrMaxCls; t += blockDim.x) {
    const int v = s_delta[t];
    if (v) atomicAdd(reinterpret_cast<unsigned long long*>(&st->d[A.buf][t / kLlrMaxCls][t % kLlrMaxCls]),
                     (unsigned long long)(long long)v);
  }
}

__global__ void k_llr_decide(LlrArgs A) {
  const LlrState* st = A.st;
  if (st->mode >= DYM_LLR_DONE) return;
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= A.s.n) return;
  if (phase_ok(st, A.buf)) return;
  const uint32_t i = A.s.sites[tid];
  uint16_t* own = A.s.links + (size_t)A.dir * A.s.V + i;
  const uint16_t old = A.oldv[tid];
  if (*own != old) *own = old;
}

__global__ void k_llr_commit(LlrArgs A, int last_in_sweep) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  LlrState* st = A.st;
  int mode = st->mode;
  if (mode >= DYM_LLR_DONE) return;
  const int buf = A.buf, w = st->axis - 1;
  const bool ok = phase_ok(st, buf);
  const double Eold = st->E[w];
  const double dE = DYM_SUB(class_sum(st->h[w], st->d[buf][w], st->v, st->ncls), Eold);
  if (ok) {
    for (int c = 0; c < st->ncls; ++c) {
      st->h[0][c] += st->d[buf][0][c];
      st->h[1][c] += st->d[buf][1][c];
    }
    st->E[0] = class_sum(st->h[0], nullptr, st->v, st->ncls);
    st->E[1] = class_sum(st->h[1], nullptr, st->v, st->ncls);
    st->phase_acc++;
  } else {
    st->phase_rej++;
  }
  for (int c = 0; c < kLlrMaxCls; ++c) {
    st->d[buf][0][c] = 0;
    st->d[buf][1][c] = 0;
  }
  if (mode == DYM_LLR_DRIVE) {
    // Aim the next phase's expected move at the remaining distance.
    const double dist = fabs(DYM_SUB(st->emid, st->E[w]));
    const double q = fabs(dE) > 0 ? DYM_MUL(st->q, dist / fabs(dE)) : DYM_MUL(st->q, 2.0);
    st->q = fmin(1.0, fmax(q, 0x1.0p-32));
    if (st->E[w] >= st->elo && st->E[w] <= st->ehi) mode = DYM_LLR_SETTLE;
  }
  if (last_in_sweep) {
    st->sweeps++;
    if (mode == DYM_LLR_DRIVE) {
      if (++st->drive_sweeps >= st->drive_cap) mode = DYM_LLR_UNREACHED;
    } else if (mode == DYM_LLR_SETTLE) {
      mode = DYM_LLR_RM;
      st->k = 0;
      st->m = 0;
      st->sumE = 0;
    } else if (mode == DYM_LLR_RM) {
      st->sumE = DYM_ADD(st->sumE, st->E[w]);
      if (++st->k == st->K) {
        const double g = DYM_SUB(st->sumE / (double)st->K, st->ewin);
        const double step = 12.0 / DYM_MUL(st->w2, (double)(st->m + 1));
        st->a = DYM_ADD(st->a, DYM_MUL(step, g));
        st->a_hist[st->m] = st->a;
        st->m++;
        st->k = 0;
        st->sumE = 0;
        if (st->m >= st->NRM) mode = DYM_LLR_DONE;
      }
    }
  }
  st->mode = mode;
}

template <int D>
cudaError_t llr_d(const LlrArgs& a, bool last, cudaStream_t s) {
  const SweepArgs& sa = a.s;
  const size_t smem = ((size_t)sa.P * 8 + (size_t)sa.P * 4 + (size_t)sa.npool * 2 + 15) / 16 * 16 + 2 * kLlrMaxCls * 4;
  void (*fn)(LlrArgs) = nullptr;
  switch (a.dir) {
    case 0: fn = k_llr_propose<D, 0>; break;
    case 1: fn = k_llr_propose<D, 1>; break;
    case 2: if (D > 2) fn = k_llr_propose<D, (D > 2 ? 2 : 0)>; break;
    case 3: if (D > 3) fn = k_llr_propose<D, (D > 3 ? 3 : 0)>; break;
  }
  if (!fn) return cudaErrorInvalidValue;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const unsigned grid = (sa.n + 255) / 256;
  if (grid) {
    fn<<<grid, 256, smem, s>>>(a);
    k_llr_decide<<<grid, 256, 0, s>>>(a);
  }
  k_llr_commit<<<1, 32, 0, s>>>(a, last ? 1 : 0);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_llr_phase(int D, const LlrArgs& a, bool last_in_sweep, cudaStream_t s) {
  switch (D) {
    case 2: return llr_d<2>(a, last_in_sweep, s);
    case 3: return llr_d<3>(a, last_in_sweep, s);
    case 4: return llr_d<4>(a, last_in_sweep, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace dym
