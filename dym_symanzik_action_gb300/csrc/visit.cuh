// Per-link Metropolis visit of the shared sub-table path, shared by the
// single-chain kernel (sweep.cu) and the batched kernel (batch.cu).
#pragma once
#include <stdint.h>

#include "chain.h"
#include "dym_core.h"
#include "staples.cuh"

namespace dym {

// Asynchronous copy of `bytes` (a multiple of 16; both addresses 16-byte
// aligned) from global into shared memory in 16-byte cp.async transfers, all
// in flight at once without passing through registers.  Completes at
// cp_async_wait_all().
__device__ __forceinline__ void cp_async_stage(void* sdst, const void* gsrc, size_t bytes) {
  const uint32_t s0 = (uint32_t)__cvta_generic_to_shared(sdst);
  const char* g0 = static_cast<const char*>(gsrc);
  for (uint32_t c = threadIdx.x; c < (uint32_t)(bytes / 16); c += blockDim.x)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s0 + 16u * c), "l"(g0 + 16ull * c) : "memory");
  asm volatile("cp.async.commit_group;" ::: "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Copy ReTr, the inverse table and the sub-table sub[k][u] = u * g_k into
// shared memory (s_sub must be 4-byte aligned when P is even).  When both
// copies of the sub-table start on 16 bytes its whole 16-byte chunks go by
// cp.async, so the block's copy costs about one L2 round trip instead of one
// per eight words a thread moves; the caller's __syncthreads() publishes it.
__device__ __forceinline__ void stage_sub_tables(const double* retr, const uint16_t* inv, const uint16_t* sub,
                                                 uint32_t P, uint32_t npool, double* s_retr, uint16_t* s_inv,
                                                 uint16_t* s_sub) {
  const uint32_t nsub = npool * P;
  const bool async = ((reinterpret_cast<uintptr_t>(sub) | (uintptr_t)__cvta_generic_to_shared(s_sub)) & 15u) == 0;
  if (async) {
    const uint32_t nb16 = (nsub * 2u) & ~15u;
    cp_async_stage(s_sub, sub, nb16);
    for (uint32_t t = nb16 / 2 + threadIdx.x; t < nsub; t += blockDim.x) s_sub[t] = sub[t];
  }
  for (uint32_t t = threadIdx.x; t < P; t += blockDim.x) {
    s_retr[t] = retr[t];
    s_inv[t] = inv[t];
  }
  if (async) {
    cp_async_wait_all();
  } else if ((P & 1u) == 0) {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(sub);
    uint32_t* dst = reinterpret_cast<uint32_t*>(s_sub);
    const uint32_t nw = nsub / 2;
#pragma unroll 8
    for (uint32_t t = threadIdx.x; t < nw; t += blockDim.x) dst[t] = src[t];
  } else {
    for (uint32_t t = threadIdx.x; t < nsub; t += blockDim.x) s_sub[t] = sub[t];
  }
}

// Programmatic dependent launch: let the next kernel on the stream begin its
// prologue (table staging, which reads nothing this kernel writes), and wait
// until the previous kernel has completed and its writes are visible.  Both
// are no-ops for a kernel launched without the attribute.
__device__ __forceinline__ void pdl_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait_prior() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Whether this sweep launch is to do nothing because the upload before it in
// the same dym_sweep_host call was refused (SweepArgs::skip).  Read after the
// programmatic wait, so the upload check has completed.
__device__ __forceinline__ bool sweep_skipped(const SweepArgs& a) { return a.skip && *a.skip != 0; }

// The end of a link visit: the link's new value into the lattice when it
// changed, and -- in the final sweep of a host-resident call -- into the
// caller's buffer whether or not it changed (SweepArgs::out, out_ref).
template <int D>
__device__ __forceinline__ void finish_link(const SweepArgs& a, int dir, uint32_t i, uint32_t b, uint32_t b0) {
  if (b != b0) a.links[(size_t)dir * a.V + i] = (uint16_t)b;
  if (a.out) a.out[(size_t)dir * a.V + i] = (uint16_t)b;
  if (a.out_ref) a.out_ref[(size_t)i * D + dir] = (int32_t)b;
}

// The reference's FP64 actions of the current link value b and of a proposal
// bnew (dym-mod-metro.cpp:166-181): beta0 + beta1 r1 + beta2 m1 with r1, m1 the
// sums of ReTr[b s_j] (ReTr[bnew s_j]) over the plaquette and rectangle staples
// in the reference's order.  The staples are recovered from the kernels'
// u_j = s_j b as s_j = u_j b^-1, so the summed elements are the reference's
// own and the sums its bits on any table -- also one whose ReTr differs inside
// a conjugacy class in the last bits (the reference's shipped files), where
// the conjugate u_j g used by the fast path would not do.  Three table
// gathers per term; only hits within the error bound of their threshold come
// here.  need_old false leaves oldact as it is.
// The value-table kernel passes its terms as shared-memory row offsets
// u_j * rb (rb = row bytes); `magic` = ceil(2^32 / rb) recovers u_j exactly
// (__umulhi, since u_j rb < 2^32).  magic 0: the terms are the elements.
template <int D>
__device__ __forceinline__ void exact_actions(const SweepArgs& a, const uint16_t* s_inv, const double* s_retr,
                                              const uint32_t* u, uint32_t b, uint32_t bnew, bool need_old,
                                              double& oldact, double& newact, uint32_t magic = 0) {
  constexpr int NS = 2 * (D - 1), NT = 8 * (D - 1);
  const uint16_t* __restrict__ mult = a.mult;
  const uint32_t P = a.P, bi = s_inv[b];
  double r1 = 0, m1 = 0, r1n = 0, m1n = 0;
#pragma unroll
  for (int j = 0; j < NT; ++j) {
    const uint32_t uj = magic ? __umulhi(u[j], magic) : u[j];
    const uint32_t sj = __ldg(mult + uj * P + bi);
    const double vn = s_retr[__ldg(mult + bnew * P + sj)];
    if (j < NS) r1n = DYM_ADD(r1n, vn);
    else m1n = DYM_ADD(m1n, vn);
    if (need_old) {
      const double vo = s_retr[__ldg(mult + b * P + sj)];
      if (j < NS) r1 = DYM_ADD(r1, vo);
      else m1 = DYM_ADD(m1, vo);
    }
  }
  if (need_old) oldact = dym_action(a.beta0, a.beta1, a.beta2, r1, m1);
  newact = dym_action(a.beta0, a.beta1, a.beta2, r1n, m1n);
}

// One visit of link (i, DIR): build the staples, then nhit hits with the
// per-hit products read from the shared sub-table.  With u_j = s_j * b the
// element u_j * g_k = s_j b g_k is conjugate to bnew s_j = b g_k s_j, so for a
// table whose ReTr is one double per conjugacy class ReTr[u_j g_k] equals the
// reference's ReTr[mult[bnew][s_j]] bit for bit, summed in the same order
// (dym-mod-metro.cpp:166-192).
// kSplit: the draws from the link's precomputed Philox state (dym_metro_hit,
// with the round keys in SweepArgs::rk filled in).
template <int D, int DIR, bool kSplit = false>
__device__ __forceinline__ void visit_sub(const SweepArgs& a, uint32_t i, uint32_t sweep, const double* s_retr,
                                          const uint16_t* s_inv, const uint16_t* s_sub, unsigned& hits,
                                          unsigned& accs) {
  constexpr int NS = 2 * (D - 1), NR = 6 * (D - 1), NT = NS + NR;
  SiteGeo<D> geo;
  site_geo<D>(i, a.Nt, a.Nx, geo);
  GlobalTab T{a.mult, s_inv, a.P};
  const uint16_t* L = a.links;
  const uint32_t V = a.V;
  auto ld = [L, V](uint32_t s, int d) -> uint32_t { return __ldg(L + (size_t)d * V + s); };
  uint32_t u[NT];
  uint16_t* own = a.links + (size_t)DIR * V + i;
  uint32_t b = *own;
  const uint32_t b0 = b;
  build_u_tree<D, DIR>(i, geo, T, ld, b, u, u + NS);  // u_j = s_j * b (associative tables only)
  double r1 = 0, m1 = 0;
#pragma unroll
  for (int j = 0; j < NS; ++j) r1 = DYM_ADD(r1, s_retr[u[j]]);
#pragma unroll
  for (int j = NS; j < NT; ++j) m1 = DYM_ADD(m1, s_retr[u[j]]);
  double oldact = dym_action(a.beta0, a.beta1, a.beta2, r1, m1);  // changes only on accept
  dym_metro_link Lk{};
  if (kSplit) Lk = dym_metro_link_init(a.rk, sweep, i, DIR, DYM_TAG_METRO);
  for (int h = 0; h < a.nhit; ++h) {
    const dym_u32x4 r = kSplit ? dym_metro_hit(a.rk, Lk, (uint32_t)h)
                               : dym_hit_random(a.seed, sweep, i, DIR, (uint32_t)h, DYM_TAG_METRO);
    const uint16_t* row = s_sub + dym_pick(r.v[0], a.npool) * a.P;
    uint32_t e[NT];
    double r1n = 0, m1n = 0;
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      e[j] = row[u[j]];
      r1n = DYM_ADD(r1n, s_retr[e[j]]);
    }
#pragma unroll
    for (int j = NS; j < NT; ++j) {
      e[j] = row[u[j]];
      m1n = DYM_ADD(m1n, s_retr[e[j]]);
    }
    const double newact = dym_action(a.beta0, a.beta1, a.beta2, r1n, m1n);
    ++hits;
    if (dym_accept_fast(oldact, newact, dym_u53(r.v[1], r.v[2]))) {
      b = row[b];
#pragma unroll
      for (int j = 0; j < NT; ++j) u[j] = e[j];
      oldact = newact;
      ++accs;
    }
  }
  finish_link<D>(a, DIR, i, b, b0);
}

// Mixed-precision visit of link (i, DIR): the decisions of visit_sub, taken
// without FP64 arithmetic except near the threshold.
//
// A packed sub-table entry holds the element and its ReTr class (16-bit
// entries: 11 + 5 bits, groups of order <= 2048; 32-bit entries: 16 + 16 bits,
// any order); the class values are staged as int32 fixed point c * 2^S.  A
// proposal's action change is then dS_fast = (b1 dR + b2 dM) 2^-S with dR, dM
// exact integer differences of the plaquette and rectangle sums, evaluated in
// FP32.  a.dmargin bounds |dS_fast - dS_fp64| (class-value rounding, FP32
// rounding, and the reference's own FP64 rounding), and t = -log(u2) is
// computed in FP32 with a bound of 2^-19 + 2^-20 t.  The reference accepts iff
// dS <= 0 or exp(-dS) > u2, i.e. iff dS < t (dym_exp is within an ulp of exp),
// so dS_fast < t - band accepts, dS_fast > t + band rejects, and only the hits
// in between are re-evaluated exactly (exact_actions: FP64 sums over the
// reference's own elements b s_j in its order, dym_accept_fast).  The
// configurations are therefore those of the FP64 path bit for bit, on tables
// whose ReTr is class-constant only up to a spread (the spread is part of
// a.dmargin).  The exact action of the current link is rebuilt lazily when a
// re-evaluation needs it after fast accepts.
// First half of a mixed-precision visit of link (i, DIR): u_j = s_j * b
// (build_u_tree; the shared-table kernels run on associative tables only) and
// the fixed-point sums R, M of the current link (bound by global-memory
// latency).
template <int D, int DIR>
__device__ __forceinline__ void mixed_prepare(const SweepArgs& a, uint32_t i, uint32_t xyz, const uint16_t* s_inv,
                                              const uint8_t* s_cls, const int32_t* s_cfix, uint32_t* u,
                                              uint32_t& b, uint32_t& R, uint32_t& M) {
  constexpr int NS = 2 * (D - 1), NR = 6 * (D - 1), NT = NS + NR;
  SiteGeo<D> geo;
  site_geo_fast<D>(xyz, a.Nt, a.Nx, geo);  // i's coordinates, packed
  GlobalTab T{a.mult, s_inv, a.P};
  const uint16_t* L = a.links;
  const uint32_t V = a.V;
  auto ld = [L, V](uint32_t s, int d) -> uint32_t { return L[(size_t)d * V + s]; };
  b = a.links[(size_t)DIR * V + i];
  build_u_tree<D, DIR>(i, geo, T, ld, b, u, u + NS);  // u_j = s_j * b
  R = 0;
  M = 0;  // fixed-point sums, modular (differences are exact)
#pragma unroll
  for (int j = 0; j < NS; ++j) R += (uint32_t)s_cfix[s_cls[u[j]]];
#pragma unroll
  for (int j = NS; j < NT; ++j) M += (uint32_t)s_cfix[s_cls[u[j]]];
}

// Draws of the HU consecutive hits h0 .. h0+HU-1 of link (i, dir): the pool
// index k = floor(npool u1) and t = -log(u2) in FP32, the threshold of the
// fast decision (u2 rebuilt from its two Philox words to within a relative
// 2^-22).  A hit's draws depend on nothing an earlier hit changes, so a group
// of hits computes its draws first: the Philox rounds of the group are
// independent of one another and of the hits' shared-memory loads, and
// interleave with them.  The draws of hits past nhit in the last group are
// computed and not used.  A hit that needs the exact u2 (re-evaluation)
// draws its Philox words again.
template <int HU>
struct HitDraws {
  uint32_t k[HU];
  float t[HU];
  __device__ __forceinline__ void set(int q, const dym_u32x4& r, uint32_t npool) {
    k[q] = dym_pick(r.v[0], npool);
    t[q] = -__logf(__fmaf_rn((float)r.v[1], 0x1p-32f, (float)(r.v[2] >> 11) * 0x1p-53f));
  }
  __device__ __forceinline__ void fill(const SweepArgs& a, uint32_t sweep, uint32_t i, uint32_t dir, int h0) {
#pragma unroll
    for (int q = 0; q < HU; ++q) set(q, dym_hit_random(a.seed, sweep, i, dir, (uint32_t)(h0 + q), DYM_TAG_METRO), a.npool);
  }
  // The same draws from the link's precomputed Philox state and the round
  // keys (dym_metro_hit: the same bits, fewer instructions); SweepArgs::rk
  // must hold the seed's round keys (kernel parameters in the single-chain
  // kernels, block-uniform values in the batch kernel).
  __device__ __forceinline__ void fill(const SweepArgs& a, const dym_metro_link& L, int h0) {
#pragma unroll
    for (int q = 0; q < HU; ++q) set(q, dym_metro_hit(a.rk, L, (uint32_t)(h0 + q)), a.npool);
  }
};

// Packed sub-table entries: the element in the low kBits bits, its class
// above.  16-bit entries hold ids below 2048; 32-bit entries any uint16 id.
template <class E>
struct Packed {
  static constexpr uint32_t kBits = sizeof(E) == 2 ? 11u : 16u;
  static constexpr uint32_t kMask = (1u << kBits) - 1u;
};

// Second half: the nhit hits of link (i, DIR) from the shared tables, starting
// from mixed_prepare's state, in groups of HU hits whose draws are computed
// ahead (HitDraws); the link is written when it changed.
// kSplit: the draws from the link's precomputed Philox state (HitDraws; the
// round keys in SweepArgs::rk filled in).
template <int D, int DIR, class E = uint16_t, int HU = 1, bool kSplit = false>
__device__ __forceinline__ void mixed_hits(const SweepArgs& a, uint32_t i, uint32_t sweep, const double* s_retr,
                                           const uint16_t* s_inv, const E* s_psub, const int32_t* s_cfix,
                                           uint32_t* u, uint32_t b,
                                           uint32_t R, uint32_t M, unsigned& hits, unsigned& accs,
                                           unsigned& rechecks, float& max_err) {
  constexpr int NS = 2 * (D - 1), NR = 6 * (D - 1), NT = NS + NR;
  constexpr uint32_t kBits = Packed<E>::kBits, kMask = Packed<E>::kMask;
  const uint32_t b0 = b;
  double oldact = 0.0;
  bool old_ok = false;
  dym_metro_link L{};
  if (kSplit) L = dym_metro_link_init(a.rk, sweep, i, DIR, DYM_TAG_METRO);
  for (int h0 = 0; h0 < a.nhit; h0 += HU) {
    HitDraws<HU> dr;
    if (kSplit) dr.fill(a, L, h0);
    else dr.fill(a, sweep, i, DIR, h0);
#pragma unroll
    for (int q = 0; q < HU; ++q) {
      if (HU > 1 && h0 + q >= a.nhit) break;
      const E* row = s_psub + dr.k[q] * a.P;
      uint32_t e[NT];
      uint32_t Rn = 0, Mn = 0;
#pragma unroll
      for (int j = 0; j < NS; ++j) {
        e[j] = row[u[j]];
        Rn += (uint32_t)s_cfix[e[j] >> kBits];
      }
#pragma unroll
      for (int j = NS; j < NT; ++j) {
        e[j] = row[u[j]];
        Mn += (uint32_t)s_cfix[e[j] >> kBits];
      }
      const float dR = (float)(int32_t)(Rn - R), dM = (float)(int32_t)(Mn - M);
      const float ds = __fmaf_rn(a.b2f, dM, __fmul_rn(a.b1f, dR)) * a.dscale;
      const float t = dr.t[q];
      const float band = a.dmargin + __fmaf_rn(t, 0x1p-20f, 0x1p-19f);
      bool acc;
      bool exact = false;
      if (ds < t - band) {
        acc = true;
      } else if (ds > t + band) {
        acc = false;
      } else {  // too close to call (also u2 == 0, where t - band is NaN)
        const dym_u32x4 r = dym_hit_random(a.seed, sweep, i, DIR, (uint32_t)(h0 + q), DYM_TAG_METRO);
        double newact;
        exact_actions<D>(a, s_inv, s_retr, u, b, row[b] & kMask, !old_ok, oldact, newact);
        old_ok = true;
        acc = dym_accept_fast(oldact, newact, dym_u53(r.v[1], r.v[2]));
        max_err = fmaxf(max_err, fabsf(ds - (float)DYM_SUB(newact, oldact)));
        ++rechecks;
        exact = true;
        if (acc) oldact = newact;
      }
      ++hits;
      if (acc) {
        b = row[b] & kMask;
#pragma unroll
        for (int j = 0; j < NT; ++j) u[j] = e[j] & kMask;
        R = Rn;
        M = Mn;
        old_ok = exact;
        ++accs;
      }
    }
  }
  finish_link<D>(a, DIR, i, b, b0);
}

__device__ __forceinline__ void flush_counters(unsigned long long* ctr, unsigned hits, unsigned accs,
                                               unsigned rechecks) {
  hits = __reduce_add_sync(0xffffffffu, hits);
  accs = __reduce_add_sync(0xffffffffu, accs);
  rechecks = __reduce_add_sync(0xffffffffu, rechecks);
  if ((threadIdx.x & 31) == 0) {
    if (hits) atomicAdd(ctr + 0, (unsigned long long)hits);
    if (accs) atomicAdd(ctr + 1, (unsigned long long)accs);
    if (rechecks) atomicAdd(ctr + 2, (unsigned long long)rechecks);
  }
}


template <int D, int DIR, class E = uint16_t, int HU = 1, bool kSplit = false>
__device__ __forceinline__ void visit_mixed(const SweepArgs& a, uint32_t i, uint32_t xyz, uint32_t sweep,
                                            const double* s_retr, const uint16_t* s_inv, const E* s_psub,
                                            const uint8_t* s_cls, const int32_t* s_cfix, unsigned& hits,
                                            unsigned& accs, unsigned& rechecks, float& max_err) {
  constexpr int NT = 8 * (D - 1);
  uint32_t u[NT];
  uint32_t b, R, M;
  mixed_prepare<D, DIR>(a, i, xyz, s_inv, s_cls, s_cfix, u, b, R, M);
  mixed_hits<D, DIR, E, HU, kSplit>(a, i, sweep, s_retr, s_inv, s_psub, s_cfix, u, b, R, M, hits, accs, rechecks,
                                    max_err);
}

// Value-table form of the mixed visit.  The shared table holds, for pool
// element g_k and element u, the int16 fixed-point value of ReTr(u * g_k)
// (scale 2^S) rather than the element, so a hit is 24 shared loads and
// integer adds; the new elements of an accepted (or re-evaluated) proposal,
// u_j * g_k, come from the L2-resident Cayley table.  Decisions as visit_mixed.
// The table is element-major, s_vsub[u * npool + k]: the pool products of one
// element are adjacent, so lanes whose staple elements coincide (ordered
// lattices) read one or two shared-memory rows instead of one row per pool
// element picked.
template <int D, int DIR>
__device__ __forceinline__ void vt_prepare(const SweepArgs& a, uint32_t i, uint32_t xyz, const uint16_t* s_inv,
                                           const int16_t* s_val, uint32_t* u, uint32_t& b, int32_t& R, int32_t& M) {
  constexpr int NS = 2 * (D - 1), NR = 6 * (D - 1), NT = NS + NR;
  SiteGeo<D> geo;
  site_geo_fast<D>(xyz, a.Nt, a.Nx, geo);
  GlobalTab T{a.mult, s_inv, a.P};
  const uint16_t* L = a.links;
  const uint32_t V = a.V;
  // Plain loads of the links rather than the read-only path (measured 1.5%
  // faster here); either is valid, since no link a launch writes is read by
  // another of its visits.
  auto ld = [L, V](uint32_t s, int d) -> uint32_t { return L[(size_t)d * V + s]; };
  b = a.links[(size_t)DIR * V + i];
  build_u_tree<D, DIR>(i, geo, T, ld, b, u, u + NS);  // u_j = s_j * b
  R = 0;
  M = 0;
#pragma unroll
  for (int j = 0; j < NS; ++j) R += s_val[u[j]];
#pragma unroll
  for (int j = NS; j < NT; ++j) M += s_val[u[j]];
}

// The hits of a value-table visit.  HU = 1: one hit at a time.  HU = 2: the
// hits are taken in pairs whose sums are both formed from the current state
// before the first is decided (48 independent shared loads instead of two
// dependent rounds of 24); when the first is accepted the second's sums are
// formed again from the new state, so the decisions are HU = 1's exactly.
// HU = 5 or 10: the draws of a group are computed ahead (HitDraws), the hits
// then taken one at a time.
template <int D, int DIR, int HU = 1>
__device__ __forceinline__ void vt_hits(const SweepArgs& a, uint32_t i, uint32_t sweep, const double* s_retr,
                                        const uint16_t* s_inv, const int16_t* s_vsub, const uint16_t* s_pool,
                                        uint32_t* u, uint32_t b, int32_t R, int32_t M, unsigned& hits,
                                        unsigned& accs, unsigned& rechecks, float& max_err) {
  constexpr int NS = 2 * (D - 1), NR = 6 * (D - 1), NT = NS + NR;
  const uint32_t b0 = b;
  const uint16_t* __restrict__ mult = a.mult;
  const uint32_t P = a.P;
  // The terms are kept as byte offsets of their rows in the element-major
  // table, u_j * rb: a hit's 24 loads then need one integer add each (ALU
  // pipe) instead of a multiply-add (FMA pipe, which the Philox rounds and
  // the FP32 decision also use).  `magic` recovers u_j for the rare paths.
  const uint32_t rb = 2u * a.npool, magic = 0xFFFFFFFFu / rb + 1u;
#pragma unroll
  for (int j = 0; j < NT; ++j) u[j] *= rb;
  double oldact = 0.0;
  bool old_ok = false;
  // The fixed-point sums of proposal k from the current terms.
  auto sums = [&](uint32_t k, int32_t& Rn, int32_t& Mn) {
    const char* col = reinterpret_cast<const char*>(s_vsub) + 2u * k;
    Rn = 0;
    Mn = 0;
#pragma unroll
    for (int j = 0; j < NS; ++j) Rn += *reinterpret_cast<const int16_t*>(col + u[j]);
#pragma unroll
    for (int j = NS; j < NT; ++j) Mn += *reinterpret_cast<const int16_t*>(col + u[j]);
  };
  // Decide hit h (proposal k, threshold t, sums Rn, Mn) and apply it;
  // returns whether it was accepted.
  auto hit = [&](int h, uint32_t k, float t, int32_t Rn, int32_t Mn) -> bool {
    const float ds = __fmaf_rn(a.b2f, (float)(Mn - M), __fmul_rn(a.b1f, (float)(Rn - R))) * a.dscale;
    const float band = a.dmargin + __fmaf_rn(t, 0x1p-20f, 0x1p-19f);
    bool acc;
    bool exact = false;
    if (ds < t - band) {
      acc = true;
    } else if (ds > t + band) {
      acc = false;
    } else {
      const dym_u32x4 r = dym_hit_random(a.seed, sweep, i, DIR, (uint32_t)h, DYM_TAG_METRO);
      const uint32_t g = s_pool[k];
      double newact;
      exact_actions<D>(a, s_inv, s_retr, u, b, __ldg(mult + b * P + g), !old_ok, oldact, newact, magic);
      old_ok = true;
      acc = dym_accept_fast(oldact, newact, dym_u53(r.v[1], r.v[2]));
      max_err = fmaxf(max_err, fabsf(ds - (float)DYM_SUB(newact, oldact)));
      ++rechecks;
      exact = true;
      if (acc) oldact = newact;
    }
    ++hits;
    if (acc) {
      const uint32_t g = s_pool[k];
      b = __ldg(mult + b * P + g);
#pragma unroll
      for (int j = 0; j < NT; ++j) u[j] = (uint32_t)__ldg(mult + __umulhi(u[j], magic) * P + g) * rb;
      R = Rn;
      M = Mn;
      old_ok = exact;
      ++accs;
    }
    return acc;
  };
  const dym_metro_link L = dym_metro_link_init(a.rk, sweep, i, DIR, DYM_TAG_METRO);
  if constexpr (HU == 2) {
    for (int h0 = 0; h0 < a.nhit; h0 += 2) {
      HitDraws<2> dr;
      dr.fill(a, L, h0);
      const bool two = h0 + 1 < a.nhit;
      int32_t R0, M0, R1 = 0, M1 = 0;
      sums(dr.k[0], R0, M0);
      if (two) sums(dr.k[1], R1, M1);
      if (hit(h0, dr.k[0], dr.t[0], R0, M0) && two) sums(dr.k[1], R1, M1);  // the state moved
      if (two) hit(h0 + 1, dr.k[1], dr.t[1], R1, M1);
    }
  } else {
    for (int h0 = 0; h0 < a.nhit; h0 += HU) {
      HitDraws<HU> dr;
      dr.fill(a, L, h0);
#pragma unroll
      for (int q = 0; q < HU; ++q) {
        if (HU > 1 && h0 + q >= a.nhit) break;
        int32_t Rn, Mn;
        sums(dr.k[q], Rn, Mn);
        hit(h0 + q, dr.k[q], dr.t[q], Rn, Mn);
      }
    }
  }
  finish_link<D>(a, DIR, i, b, b0);
}

// Two lanes per link (vt2): the value-table visit with a link's work split
// over an adjacent lane pair.  Lane `back` (odd lane) holds the u_j of the -f
// side of every plane (build_u_half), lane !back those of the +f side: 3(D-1)
// terms each.  A hit's sums are the pair's two partial sums (two shuffles);
// the pair draws two hits' random numbers at once, one hit per lane, and
// exchanges them; both lanes then take the same decision from the same
// integers, so the decisions, re-evaluations and counts are the one-lane
// visit's (vt_hits) exactly.  `pm` is the pair's shuffle mask.
__device__ __forceinline__ unsigned pair_mask() { return 3u << (threadIdx.x & 30u); }

template <int D, int DIR>
__device__ __forceinline__ void vt2_prepare(const SweepArgs& a, uint32_t i, uint32_t xyz, bool back, unsigned pm,
                                            const uint16_t* s_inv, const int16_t* s_val, uint32_t* up, uint32_t* ur,
                                            uint32_t& b, int32_t& R, int32_t& M) {
  constexpr int NP = D - 1, NQ = 3 * (D - 1);
  SiteGeo<D> geo;
  site_geo_fast<D>(xyz, a.Nt, a.Nx, geo);
  GlobalTab T{a.mult, s_inv, a.P};
  const uint16_t* L = a.links;
  const uint32_t V = a.V;
  auto ld = [L, V](uint32_t s, int d) -> uint32_t { return __ldg(L + (size_t)d * V + s); };
  b = a.links[(size_t)DIR * V + i];
  build_u_half<D, DIR>(i, geo, T, ld, b, back, up, ur);
  int32_t r = 0, m = 0;
#pragma unroll
  for (int j = 0; j < NP; ++j) r += s_val[up[j]];
#pragma unroll
  for (int j = 0; j < NQ; ++j) m += s_val[ur[j]];
  R = r + __shfl_xor_sync(pm, r, 1);
  M = m + __shfl_xor_sync(pm, m, 1);
}

// exact_actions for a lane pair (four dimensions): the FP64 sums of
// ReTr[bnew s_j] (and of ReTr[b s_j] when need_old) over the pair's 24 terms,
// added in build_u_tree's order (plaquettes plane by plane, +f side then -f
// side; rectangles plane by plane, 1-3 then 4-6), so that both lanes get the
// reference's bits.  Each lane evaluates its own terms and receives its
// partner's by shuffles, one term pair at a time.  Not inlined: a hit comes
// here about once in 10^5, and the call keeps this path's registers out of
// the hit loop's allocation; the terms are passed by value (an array would
// have to live in local memory).
struct ActPair {
  double oldact, newact;
};

static __device__ __noinline__ ActPair vt2_exact4(const uint16_t* __restrict__ mult, uint32_t P,
                                                  const uint16_t* s_inv, const double* s_retr, double beta0,
                                                  double beta1, double beta2, bool back, unsigned pm, uint32_t p0,
                                                  uint32_t p1, uint32_t p2, uint32_t q0, uint32_t q1, uint32_t q2,
                                                  uint32_t q3, uint32_t q4, uint32_t q5, uint32_t q6, uint32_t q7,
                                                  uint32_t q8, uint32_t b, uint32_t bnew, bool need_old,
                                                  double oldact) {
  const uint32_t bi = s_inv[b];
  double r1 = 0, m1 = 0, r1n = 0, m1n = 0;
  // own term of u and the partner's, as (+f side, -f side)
  auto pair_terms = [&](uint32_t u, double& fo, double& bo, double& fn, double& bn) {
    const uint32_t sj = __ldg(mult + u * P + bi);
    const double vn = s_retr[__ldg(mult + bnew * P + sj)];
    const double vo = need_old ? s_retr[__ldg(mult + b * P + sj)] : 0.0;
    const double pn = __shfl_xor_sync(pm, vn, 1), po = __shfl_xor_sync(pm, vo, 1);
    fn = back ? pn : vn;
    bn = back ? vn : pn;
    fo = back ? po : vo;
    bo = back ? vo : po;
  };
  const uint32_t up[3] = {p0, p1, p2};
  const uint32_t ur[9] = {q0, q1, q2, q3, q4, q5, q6, q7, q8};
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    double fo, bo, fn, bn;
    pair_terms(up[p], fo, bo, fn, bn);
    r1n = DYM_ADD(DYM_ADD(r1n, fn), bn);
    r1 = DYM_ADD(DYM_ADD(r1, fo), bo);
  }
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    double fo[3], bo[3], fn[3], bn[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) pair_terms(ur[3 * p + r], fo[r], bo[r], fn[r], bn[r]);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      m1n = DYM_ADD(m1n, fn[r]);
      m1 = DYM_ADD(m1, fo[r]);
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      m1n = DYM_ADD(m1n, bn[r]);
      m1 = DYM_ADD(m1, bo[r]);
    }
  }
  ActPair out;
  out.oldact = need_old ? dym_action(beta0, beta1, beta2, r1, m1) : oldact;
  out.newact = dym_action(beta0, beta1, beta2, r1n, m1n);
  return out;
}

template <int D, int DIR>
__device__ __forceinline__ void vt2_hits(const SweepArgs& a, uint32_t i, uint32_t sweep, bool back, unsigned pm,
                                         const double* s_retr, const uint16_t* s_inv, const int16_t* s_vsub,
                                         const uint16_t* s_pool, uint32_t* up, uint32_t* ur, uint32_t b, int32_t R,
                                         int32_t M, unsigned& hits, unsigned& accs, unsigned& rechecks,
                                         float& max_err) {
  constexpr int NP = D - 1, NQ = 3 * (D - 1);
  const uint32_t b0 = b;
  const uint16_t* __restrict__ mult = a.mult;
  const uint32_t P = a.P, np = a.npool;
  double oldact = 0.0;
  bool old_ok = false;
  const dym_metro_link L = dym_metro_link_init(a.rk, sweep, i, DIR, DYM_TAG_METRO);
  for (int h0 = 0; h0 < a.nhit; h0 += 2) {
    // This lane draws hit h0 + back; the pair swaps them.
    const dym_u32x4 rr = dym_metro_hit(a.rk, L, (uint32_t)h0 + (back ? 1u : 0u));
    const uint32_t kown = dym_pick(rr.v[0], np);
    const float town = -__logf(__fmaf_rn((float)rr.v[1], 0x1p-32f, (float)(rr.v[2] >> 11) * 0x1p-53f));
    const uint32_t koth = __shfl_xor_sync(pm, kown, 1);
    const float toth = __shfl_xor_sync(pm, town, 1);
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (q == 1 && h0 + 1 >= a.nhit) break;
      const bool mine = (q == 1) == back;
      const uint32_t k = mine ? kown : koth;
      const float t = mine ? town : toth;
      const int16_t* col = s_vsub + k;
      int32_t rp = 0, mp = 0;
#pragma unroll
      for (int j = 0; j < NP; ++j) rp += col[up[j] * np];
#pragma unroll
      for (int j = 0; j < NQ; ++j) mp += col[ur[j] * np];
      const int32_t Rn = rp + __shfl_xor_sync(pm, rp, 1), Mn = mp + __shfl_xor_sync(pm, mp, 1);
      const float ds = __fmaf_rn(a.b2f, (float)(Mn - M), __fmul_rn(a.b1f, (float)(Rn - R))) * a.dscale;
      const float band = a.dmargin + __fmaf_rn(t, 0x1p-20f, 0x1p-19f);
      bool acc;
      bool exact = false;
      if (ds < t - band) {
        acc = true;
      } else if (ds > t + band) {
        acc = false;
      } else {  // both lanes of the pair (same ds and t)
        const dym_u32x4 r = dym_hit_random(a.seed, sweep, i, DIR, (uint32_t)(h0 + q), DYM_TAG_METRO);
        const uint32_t g = s_pool[k];
        static_assert(D == 4, "the pair's exact re-evaluation is written for four dimensions");
        const ActPair ap = vt2_exact4(mult, P, s_inv, s_retr, a.beta0, a.beta1, a.beta2, back, pm, up[0], up[1],
                                      up[2], ur[0], ur[1], ur[2], ur[3], ur[4], ur[5], ur[6], ur[7], ur[8], b,
                                      __ldg(mult + b * P + g), !old_ok, oldact);
        oldact = ap.oldact;
        const double newact = ap.newact;
        old_ok = true;
        acc = dym_accept_fast(oldact, newact, dym_u53(r.v[1], r.v[2]));
        max_err = fmaxf(max_err, fabsf(ds - (float)DYM_SUB(newact, oldact)));
        rechecks += back ? 0u : 1u;
        exact = true;
        if (acc) oldact = newact;
      }
      hits += back ? 0u : 1u;
      if (acc) {
        const uint32_t g = s_pool[k];
        b = __ldg(mult + b * P + g);
#pragma unroll
        for (int j = 0; j < NP; ++j) up[j] = __ldg(mult + up[j] * P + g);
#pragma unroll
        for (int j = 0; j < NQ; ++j) ur[j] = __ldg(mult + ur[j] * P + g);
        R = Rn;
        M = Mn;
        old_ok = exact;
        accs += back ? 0u : 1u;
      }
    }
  }
  if (!back) finish_link<D>(a, DIR, i, b, b0);
}

// Largest |dS_fast - dS_fp64| seen at a re-evaluation, into the low word of
// *ctr (non-negative floats order like their bit patterns).
__device__ __forceinline__ void flush_max_err(unsigned long long* ctr, float err) {
  const unsigned bits = __reduce_max_sync(0xffffffffu, __float_as_uint(err));
  if ((threadIdx.x & 31) == 0 && bits) atomicMax(reinterpret_cast<unsigned int*>(ctr), bits);
}

}  // namespace dym

namespace dym {

// dym_weight_accept(x, u2) with u2 = dym_u53(r1, r2), deciding most hits in
// FP32.  For -38 <= x < 0, ef = __expf((float)x) is within a relative
// 2^-17 of exp(x) (the conversion of x costs |x| 2^-24 <= 2^-18.7, __expf at
// most 2 + floor(1.173 |x|) <= 46 ulp = 2^-17.5), u2f within 2^-22 of u2
// (exact when r1 == 0; every nonzero u2 is >= 2^-53, a normal float) and
// dym_exp within an ulp of exp; so ef above u2f (1 + 2^-10) implies
// dym_exp(x) > u2, ef below u2f (1 - 2^-10) implies the opposite, and only the
// hits in between evaluate dym_exp.  The decision is dym_weight_accept's, bit
// for bit, and the FP64 pipe (the limit of the LLR sweep on this part)
// evaluates the exponential for at most 2^-9 of the hits with x < 0 instead of
// for all of them.
__device__ __forceinline__ bool llr_weight_accept(double x, uint32_t r1, uint32_t r2) {
  if (x >= 0.0) return true;
  const bool u2_zero = (r1 | (r2 >> 11)) == 0u;
  if (x < -38.0) return u2_zero && dym_exp(x) > 0.0;
  const float ef = __expf(__double2float_rn(x));
  const float u2f = __fmaf_rn((float)r1, 0x1p-32f, (float)(r2 >> 11) * 0x1p-53f);
  if (ef > __fmul_rn(u2f, 1.0f + 0x1p-10f)) return true;
  if (ef < __fmul_rn(u2f, 1.0f - 0x1p-10f)) return false;
  return dym_exp(x) > dym_u53(r1, r2);
}

// Weights of an LLR hit: exponent -a dE_w - bg dE_bg with dE = d 2^-S for the
// exact integer sums d (d_w of the windowed action, d_bg of the other).
struct LlrWeight {
  double naa, bg, scale;  // -a, bg, 2^-S
  float naf, bgf, sf;     // the same in FP32
};

// dym_weight_accept(x, u2), x = -a dE_w - bg dE_bg formed in FP64 as the
// oracle does, decided in FP32 for all but the hits near a threshold.
// xf = (-a_f d_w - bg_f d_bg) 2^-S from FP32 copies of a, bg and d: each
// conversion and product is within 2^-24 relative and the difference adds one
// rounding, so |xf - x| <= 2^-22 T + 2^-52 T with T = (|p| + |q|) 2^-S, and
// B = 2^-20 T bounds it twice over.  xf - B >= 0 implies x >= 0 (accept).
// When B <= 2^-12 and xf lies in [-38 + B, -B], x is in [-38, 0) and
// exp(xf) is within a factor exp(2^-14) of exp(x); with __expf's documented
// error (at most 46 ulp there) and u2f within 2^-22 of u2 the FP32 test of
// llr_weight_accept (band 2^-10) decides.  Every other hit forms x in FP64
// and runs llr_weight_accept.  The decision is dym_weight_accept's, bit for
// bit.
__device__ __forceinline__ bool llr_fix_accept(int32_t dw, int32_t dbg, const LlrWeight& wt, uint32_t r1,
                                               uint32_t r2) {
  const float p = __fmul_rn(wt.naf, (float)dw), q = __fmul_rn(wt.bgf, (float)dbg);
  const float xf = __fmul_rn(__fsub_rn(p, q), wt.sf);
  const float B = __fmul_rn(__fadd_rn(fabsf(p), fabsf(q)), __fmul_rn(wt.sf, 0x1p-20f));
  if (__fsub_rn(xf, B) >= 0.0f) return true;
  if (B <= 0x1p-12f && __fadd_rn(xf, B) < 0.0f && __fsub_rn(xf, B) >= -38.0f) {
    const float ef = __expf(xf);
    const float u2f = __fmaf_rn((float)r1, 0x1p-32f, (float)(r2 >> 11) * 0x1p-53f);
    if (ef > __fmul_rn(u2f, 1.0f + 0x1p-10f)) return true;
    if (ef < __fmul_rn(u2f, 1.0f - 0x1p-10f)) return false;
  }
  const double dEw = DYM_MUL((double)dw, wt.scale), dEbg = DYM_MUL((double)dbg, wt.scale);
  return llr_weight_accept(DYM_SUB(DYM_MUL(wt.naa, dEw), DYM_MUL(wt.bg, dEbg)), r1, r2);
}

// Closer to the window centre (fixed-point energies; a two-dimensional cell
// compares squared normalised distances) -- the drive-in test of the hits and
// of the commit's scan.
__device__ __forceinline__ double llr_drive_nsq(const LlrDrive& d, long long e1, long long e2) {
  const double x = DYM_MUL((double)(e1 - d.mid[0]), d.sc[0]), y = DYM_MUL((double)(e2 - d.mid[1]), d.sc[1]);
  return DYM_ADD(DYM_MUL(x, x), DYM_MUL(y, y));
}

__device__ __forceinline__ bool llr_drive_closer(const LlrDrive& d, long long e1, long long e2, long long q1,
                                                 long long q2) {
  if (d.dims == 2) return llr_drive_nsq(d, e1, e2) < llr_drive_nsq(d, q1, q2);
  const long long e = d.axis == 1 ? e1 : e2, q = d.axis == 1 ? q1 : q2;
  return llabs(e - d.mid[0]) < llabs(q - d.mid[0]);
}

// One LLR visit of link (i, DIR) with the shared sub-table (llr.cpp:186-216
// per hit): nhit hits with weight exp(-a dE_w - bg dE_bg), or, in drive-in
// mode, greedy moves of the link's running energy towards the centre.  The
// sub-table's entries pack element and class (Packed<E>), so a term's value
// is one read of the class-value table s_cv (one word per bank: no bank
// conflicts); a hit's dS1, dS2 are exact integer sums of its terms' class
// values at scale 2^evshift, and the weight's exponent is formed from them
// (llr_fix_accept: in FP32, in FP64 near a threshold).  The link is written in place; returns its value before the visit, and
// in de1, de2 the exact change of S1 and S2 at scale 2^kLlrFixShift (vf: class
// values), which the commit's scan tests against the window.  The classes of
// the initial u_j are kept packed, 5 bits each, and the two hit loops are
// separate so that neither holds the other's state.
template <int D, int DIR, class E>
__device__ __forceinline__ uint32_t visit_llr(const SweepArgs& a, uint32_t i, uint32_t sweep, const int32_t* s_cv,
                                              int evshift, const uint16_t* s_inv, const E* s_psub,
                                              const uint16_t* s_cls, const long long* __restrict__ vf, int axis,
                                              double aa, double bg, const LlrDrive& dr, bool drive, long long& de1,
                                              long long& de2, unsigned& hits, unsigned& accs) {
  constexpr int NS = 2 * (D - 1), NR = 6 * (D - 1), NT = NS + NR;
  constexpr uint32_t kBits = Packed<E>::kBits, kMask = Packed<E>::kMask;
  constexpr int NW = (NT + 5) / 6;  // words of six 5-bit classes
  static_assert(kLlrMaxCls <= 32, "classes are packed in 5 bits");
  SiteGeo<D> geo;
  site_geo<D>(i, a.Nt, a.Nx, geo);
  GlobalTab T{a.mult, s_inv, a.P};
  const uint16_t* L = a.links;
  const uint32_t V = a.V;
  auto ld = [L, V](uint32_t s, int d) -> uint32_t { return __ldg(L + (size_t)d * V + s); };
  uint32_t u[NT];
  uint16_t* own = a.links + (size_t)DIR * V + i;
  uint32_t b = *own;
  const uint32_t b0 = b;
  build_u_tree<D, DIR>(i, geo, T, ld, b, u, u + NS);  // u_j = s_j * b
  uint32_t c0[NW];
#pragma unroll
  for (int w = 0; w < NW; ++w) c0[w] = 0;
  int32_t R = 0, M = 0;  // exact sums (the differences below fit int32: dym_fix_shift)
#pragma unroll
  for (int j = 0; j < NT; ++j) {
    const uint32_t cj = s_cls[u[j]];
    c0[j / 6] |= cj << (5 * (j % 6));
    if (j < NS) R += s_cv[cj];
    else M += s_cv[cj];
  }
  if (drive) {
    const int up = kLlrFixShift - evshift;
    long long cum1 = 0, cum2 = 0;  // the link's kept moves, scale 2^kLlrFixShift
    for (int h = 0; h < a.nhit; ++h) {
      const dym_u32x4 r = dym_hit_random(a.seed, sweep, i, DIR, (uint32_t)h, DYM_TAG_LLR);
      const E* row = s_psub + dym_pick(r.v[0], a.npool) * a.P;
      uint32_t e[NT];
      int32_t Rn = 0, Mn = 0;
#pragma unroll
      for (int j = 0; j < NS; ++j) {
        e[j] = row[u[j]];
        Rn += s_cv[e[j] >> kBits];
      }
#pragma unroll
      for (int j = NS; j < NT; ++j) {
        e[j] = row[u[j]];
        Mn += s_cv[e[j] >> kBits];
      }
      const long long n1 = cum1 + (long long)(Rn - R) * (1ll << up), n2 = cum2 + (long long)(Mn - M) * (1ll << up);
      ++hits;
      if (llr_drive_closer(dr, dr.E[0] + n1, dr.E[1] + n2, dr.E[0] + cum1, dr.E[1] + cum2)) {
        b = row[b] & kMask;
#pragma unroll
        for (int j = 0; j < NT; ++j) u[j] = e[j] & kMask;
        R = Rn;
        M = Mn;
        cum1 = n1;
        cum2 = n2;
        ++accs;
      }
    }
  } else {
    LlrWeight wt;
    wt.naa = -aa;
    wt.bg = bg;
    wt.scale = ldexp(1.0, -evshift);
    wt.naf = __double2float_rn(-aa);
    wt.bgf = __double2float_rn(bg);
    wt.sf = ldexpf(1.0f, -evshift);
    for (int h = 0; h < a.nhit; ++h) {
      const dym_u32x4 r = dym_hit_random(a.seed, sweep, i, DIR, (uint32_t)h, DYM_TAG_LLR);
      const E* row = s_psub + dym_pick(r.v[0], a.npool) * a.P;
      uint32_t e[NT];
      int32_t Rn = 0, Mn = 0;
#pragma unroll
      for (int j = 0; j < NS; ++j) {
        e[j] = row[u[j]];
        Rn += s_cv[e[j] >> kBits];
      }
#pragma unroll
      for (int j = NS; j < NT; ++j) {
        e[j] = row[u[j]];
        Mn += s_cv[e[j] >> kBits];
      }
      const int32_t d1 = Rn - R, d2 = Mn - M;
      ++hits;
      if (llr_fix_accept(axis == 1 ? d1 : d2, axis == 1 ? d2 : d1, wt, r.v[1], r.v[2])) {
        b = row[b] & kMask;
#pragma unroll
        for (int j = 0; j < NT; ++j) u[j] = e[j] & kMask;
        R = Rn;
        M = Mn;
        ++accs;
      }
    }
  }
  de1 = 0;
  de2 = 0;
  if (b != b0) {
    *own = (uint16_t)b;
    // Class of b s_j equals the class of its conjugate s_j b = u_j.
#pragma unroll
    for (int j = 0; j < NT; ++j) {
      const long long dv = __ldg(vf + s_cls[u[j]]) - __ldg(vf + ((c0[j / 6] >> (5 * (j % 6))) & 31u));
      if (j < NS) de1 += dv;
      else de2 += dv;
    }
  }
  return b0;
}

}  // namespace dym
