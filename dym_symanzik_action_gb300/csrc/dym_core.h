// Shared host/device arithmetic of the Metropolis engine: the random stream
// and the exponential used by the accept test.  Everything here must give the
// same bits on the CPU (x86-64 or aarch64, compiled with -ffp-contract=off)
// and on the GPU (explicit __dmul_rn/__dadd_rn/__fma_rn), because the link
// configuration after every sweep is compared bit for bit between the two.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define DYM_HD __host__ __device__ __forceinline__
#else
#define DYM_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define DYM_MUL(a, b) __dmul_rn((a), (b))
#define DYM_ADD(a, b) __dadd_rn((a), (b))
#define DYM_SUB(a, b) __dsub_rn((a), (b))
#define DYM_FMA(a, b, c) __fma_rn((a), (b), (c))
#else
#include <math.h>
#define DYM_MUL(a, b) ((a) * (b))
#define DYM_ADD(a, b) ((a) + (b))
#define DYM_SUB(a, b) ((a) - (b))
#define DYM_FMA(a, b, c) fma((a), (b), (c))
#endif

// ---------------------------------------------------------------------------
// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, "Parallel
// random numbers: as easy as 1, 2, 3", SC'11).  Multipliers and Weyl key
// increments are the ones published with the algorithm.
// ---------------------------------------------------------------------------
typedef struct { uint32_t v[4]; } dym_u32x4;

#define DYM_PHILOX_M0 0xD2511F53u
#define DYM_PHILOX_M1 0xCD9E8D57u
#define DYM_PHILOX_W0 0x9E3779B9u
#define DYM_PHILOX_W1 0xBB67AE85u

DYM_HD dym_u32x4 dym_philox4x32_10(dym_u32x4 c, uint32_t k0, uint32_t k1) {
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)DYM_PHILOX_M0 * c.v[0];
    uint64_t p1 = (uint64_t)DYM_PHILOX_M1 * c.v[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    dym_u32x4 o;
    o.v[0] = hi1 ^ c.v[1] ^ k0;
    o.v[1] = lo1;
    o.v[2] = hi0 ^ c.v[3] ^ k1;
    o.v[3] = lo0;
    c = o;
    k0 += DYM_PHILOX_W0;
    k1 += DYM_PHILOX_W1;
  }
  return c;
}

// Stream tags: word 3 of the counter, so that different uses of one seed never
// share a counter.
#define DYM_TAG_METRO 0x4D455452u  // Metropolis hits
#define DYM_TAG_HOT   0x484F5453u  // hot-start link draws
#define DYM_TAG_LLR   0x4C4C5231u  // interval-restricted (LLR) hits

// Counter layout of one Metropolis hit.  The key is the 64-bit chain seed.
// The colour of a link is a function of (site, dir), so the tuple
// (seed, sweep, link, hit) identifies the hit uniquely.
DYM_HD dym_u32x4 dym_hit_random(uint64_t seed, uint32_t sweep, uint32_t site,
                                uint32_t dir, uint32_t hit, uint32_t tag) {
  dym_u32x4 c;
  c.v[0] = site;
  c.v[1] = sweep;
  c.v[2] = (dir << 20) | (hit & 0xFFFFFu);
  c.v[3] = tag;
  return dym_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

// The same block for the hits of one link, with the work that does not
// depend on the hit index done once.  Round keys rk[2r], rk[2r+1] = k0 + r W0,
// k1 + r W1 (dym_philox_round_keys; in a kernel's parameters they are
// constant-bank operands).  In the counter (site, sweep, dir<<20 | hit, tag)
// only word 2 changes with the hit: round 0's product of word 0 and the words
// it feeds, and round 1's product of word 2 (made of those), are the link's.
typedef struct {
  uint32_t s0;    // sweep ^ rk[0]: round 0's word-1 operand
  uint32_t c1;    // round 1: hi(M1 (hi(M0 site) ^ tag ^ rk[1])) ^ rk[2]
  uint32_t e1;    // round 1: lo(M1 (hi(M0 site) ^ tag ^ rk[1])), its output word 1
  uint32_t b1;    // round 1: lo(M0 site) ^ rk[3]
  uint32_t dir20; // dir << 20
} dym_metro_link;

DYM_HD void dym_philox_round_keys(uint64_t seed, uint32_t rk[20]) {
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (int r = 0; r < 10; ++r) {
    rk[2 * r] = k0;
    rk[2 * r + 1] = k1;
    k0 += DYM_PHILOX_W0;
    k1 += DYM_PHILOX_W1;
  }
}

DYM_HD dym_metro_link dym_metro_link_init(const uint32_t* rk, uint32_t sweep, uint32_t site, uint32_t dir,
                                          uint32_t tag) {
  const uint64_t p0 = (uint64_t)DYM_PHILOX_M0 * site;
  const uint32_t a = (uint32_t)(p0 >> 32) ^ tag ^ rk[1];  // round 0 output word 2
  const uint64_t p1 = (uint64_t)DYM_PHILOX_M1 * a;
  dym_metro_link L;
  L.s0 = sweep ^ rk[0];
  L.c1 = (uint32_t)(p1 >> 32) ^ rk[2];
  L.e1 = (uint32_t)p1;
  L.b1 = (uint32_t)p0 ^ rk[3];
  L.dir20 = dir << 20;
  return L;
}

// Equal to dym_hit_random(seed, sweep, site, dir, hit, tag) for the link of
// dym_metro_link_init(rk of seed, sweep, site, dir, tag).
DYM_HD dym_u32x4 dym_metro_hit(const uint32_t* rk, dym_metro_link L, uint32_t hit) {
  // round 0: only word 2's product depends on the hit
  const uint64_t q1 = (uint64_t)DYM_PHILOX_M1 * (L.dir20 | (hit & 0xFFFFFu));
  const uint32_t o0 = (uint32_t)(q1 >> 32) ^ L.s0, o1 = (uint32_t)q1;
  // round 1: word 0's product depends on the hit, word 2's is the link's
  const uint64_t q0 = (uint64_t)DYM_PHILOX_M0 * o0;
  dym_u32x4 c;
  c.v[0] = L.c1 ^ o1;
  c.v[1] = L.e1;
  c.v[2] = (uint32_t)(q0 >> 32) ^ L.b1;
  c.v[3] = (uint32_t)q0;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int r = 2; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)DYM_PHILOX_M0 * c.v[0];
    const uint64_t p1 = (uint64_t)DYM_PHILOX_M1 * c.v[2];
    dym_u32x4 o;
    o.v[0] = (uint32_t)(p1 >> 32) ^ c.v[1] ^ rk[2 * r];
    o.v[1] = (uint32_t)p1;
    o.v[2] = (uint32_t)(p0 >> 32) ^ c.v[3] ^ rk[2 * r + 1];
    o.v[3] = (uint32_t)p0;
    c = o;
  }
  return c;
}

// u1 = r0 * 2^-32 in [0,1); the proposal index floor(n * u1) equals
// (r0 * n) >> 32 exactly for n < 2^21 (both products are exact in double).
DYM_HD uint32_t dym_pick(uint32_t r0, uint32_t n) {
  return (uint32_t)(((uint64_t)r0 * n) >> 32);
}

// u2 in [0,1) with 53 random bits: (r1 * 2^21 + (r2 >> 11)) * 2^-53.
DYM_HD double dym_u53(uint32_t r1, uint32_t r2) {
  uint64_t m = ((uint64_t)r1 << 21) | (r2 >> 11);
  return (double)m * 0x1.0p-53;
}

// ---------------------------------------------------------------------------
// exp(x) for the Metropolis ratio.  Cody-Waite argument reduction
// x = k ln2 + r with ln2 split into a 24-bit head (k*LN2_HI exact for |k| <
// 2^28) and a tail, then the Taylor series of e^r to degree 13 by Horner's rule
// with fused multiply-adds (|r| <= ln2/2, truncation < 0.05 ulp), then scaling
// by 2^k built from its bit pattern.  Accuracy is about 1 ulp; what matters is
// that host and device produce identical bits.
// ---------------------------------------------------------------------------
DYM_HD double dym_bits_to_double(uint64_t b) {
  union { uint64_t u; double d; } x; x.u = b; return x.d;
}

DYM_HD double dym_exp(double x) {
  if (!(x == x)) return x;                 // NaN
  if (x > 709.0) return dym_bits_to_double(0x7FF0000000000000ull);  // +inf
  if (x < -745.5) return 0.0;
  const double LOG2E = 0x1.71547652b82fep+0;
  const double LN2_HI = 0x1.62e42f0000000p-1;
  const double LN2_LO = 0x1.df473de6af279p-26;
  double kd = DYM_MUL(x, LOG2E);
#if defined(__CUDA_ARCH__)
  kd = rint(kd);
#else
  kd = nearbyint(kd);
#endif
  int k = (int)kd;
  double r = DYM_FMA(-kd, LN2_HI, x);
  r = DYM_FMA(-kd, LN2_LO, r);
  // 1/n!, n = 13 .. 0, each the double nearest the exact rational.
  double p = 0x1.6124613a86d09p-33;
  p = DYM_FMA(p, r, 0x1.1eed8eff8d898p-29);
  p = DYM_FMA(p, r, 0x1.ae64567f544e4p-26);
  p = DYM_FMA(p, r, 0x1.27e4fb7789f5cp-22);
  p = DYM_FMA(p, r, 0x1.71de3a556c734p-19);
  p = DYM_FMA(p, r, 0x1.a01a01a01a01ap-16);
  p = DYM_FMA(p, r, 0x1.a01a01a01a01ap-13);
  p = DYM_FMA(p, r, 0x1.6c16c16c16c17p-10);
  p = DYM_FMA(p, r, 0x1.1111111111111p-7);
  p = DYM_FMA(p, r, 0x1.5555555555555p-5);
  p = DYM_FMA(p, r, 0x1.5555555555555p-3);
  p = DYM_FMA(p, r, 0.5);
  p = DYM_FMA(p, r, 1.0);
  p = DYM_FMA(p, r, 1.0);
  if (k >= -1020) {
    return DYM_MUL(p, dym_bits_to_double((uint64_t)(k + 1023) << 52));
  }
  // Result near or below the normal range: scale in two exact-or-rounded steps.
  double s1 = dym_bits_to_double((uint64_t)(k + 54 + 1023) << 52);
  return DYM_MUL(DYM_MUL(p, s1), 0x1.0p-54);
}

// Reference accept rule (dym-mod-metro.cpp:180-187): with
//   oldact = beta0 + beta1*r1    + beta2*m1
//   newact = beta0 + beta1*r1new + beta2*m1new
// accept iff (newact <= oldact ? 1 : exp(-(newact-oldact))) > u2.
DYM_HD double dym_action(double b0, double b1, double b2, double r1, double m1) {
  return DYM_ADD(DYM_ADD(b0, DYM_MUL(b1, r1)), DYM_MUL(b2, m1));
}

DYM_HD int dym_accept(double oldact, double newact, double u2) {
  double probrat = (newact <= oldact) ? 1.0 : dym_exp(-DYM_SUB(newact, oldact));
  return probrat > u2;
}

// The same decision with the exponential skipped where it cannot matter: for
// d = newact - oldact > 38, exp(-d) < 3.2e-17 (and dym_exp is within a few ulp
// of it) while every nonzero u2 is >= 2^-53 = 1.1e-16, so the test can only
// pass for u2 == 0, which is then decided by dym_exp itself.
/* Mixed-precision decisions.  Bound on |x_fast - x_fp64| for
 *   x = c0 + c1 dE1 + c2 dE2  (dE1 a difference of two sums of n1 class values,
 *                              dE2 of two sums of n2)
 * when x_fast comes from exact integer sums of class values rounded to the
 * fixed point (error q per term: half a unit plus the class spread, |value| <=
 * amax) scaled in FP32 (four roundings of 2^-24 relative), and x_fp64 is the
 * FP64 evaluation of the same expression in the reference's order; doubled,
 * plus 1e-7.  A decision x < t whose |x_fast - t| exceeds this bound plus the
 * error of t is the FP64 decision. */
DYM_HD double dym_mixed_margin(double c0, double c1, double n1, double c2, double n2, double q, double amax) {
  const double w = fabs(c1) * 2.0 * n1 + fabs(c2) * 2.0 * n2;
  const double quant = w * q;
  const double feval = 0x1p-22 * w * (amax + q);
  const double rref = 0x1p-45 * (fabs(c0) + (fabs(c1) * n1 + fabs(c2) * n2) * amax + 1.0);
  return 2.0 * (quant + feval + rref) + 1e-7;
}

/* The LLR weighted test exp(x) > u2 (llr.cpp:211-212, x = -a dE_w - bg dE_bg)
 * with the exponential evaluated only where it can change the outcome: x >= 0
 * accepts (exp(x) >= 1 > u2), x < -38 rejects unless u2 == 0 (exp(x) < 3.2e-17
 * while every nonzero u2 is >= 2^-53); otherwise dym_exp(x) > u2. */
DYM_HD int dym_weight_accept(double x, double u2) {
  if (x >= 0.0) return 1;
  if (x < -38.0 && u2 != 0.0) return 0;
  return dym_exp(x) > u2;
}

DYM_HD int dym_accept_fast(double oldact, double newact, double u2) {
  if (newact <= oldact) return 1.0 > u2;
  const double d = DYM_SUB(newact, oldact);
  if (d > 38.0 && u2 != 0.0) return 0;
  return dym_exp(-d) > u2;
}

// ---------------------------------------------------------------------------
// LLR window scan: links per block.  After a colour class's links have run
// their hits, the scan keeps or reverts the moves of consecutive blocks of
// this many links (in site-list order) by the window test on the running
// energy.  It is the largest power of two up to 32 for which a block's largest
// possible change of every windowed action -- links x terms a link changes
// (2(D-1) plaquettes, 6(D-1) rectangles) x the ReTr range -- is at most a
// quarter of that window's width (half its half-width), and 1 at least; so a
// block moving away from one wall can never pass the other.
// dims 2: both actions windowed (half-widths hw, hw2); else axis 1 (S1) or 2.
// ---------------------------------------------------------------------------
DYM_HD int dym_llr_block_links(int D, double retr_range, int dims, int axis, double hw, double hw2) {
  const double t1 = 2.0 * (D - 1) * retr_range, t2 = 6.0 * (D - 1) * retr_range;
  int s = 32;
  while (s > 1) {
    const int ok = dims == 2 ? (s * t1 <= 0.5 * hw && s * t2 <= 0.5 * hw2)
                             : (s * (axis == 1 ? t1 : t2) <= 0.5 * hw);
    if (ok) break;
    s >>= 1;
  }
  return s;
}

// ---------------------------------------------------------------------------
// Fixed-point scale 2^S of ReTr class values for exact integer sums of a
// link's staple terms: the largest S <= 24 for which the difference of two
// sums of 6(D-1) terms, each at most amax 2^S + 1/2 in magnitude (amax the
// largest |ReTr|), stays inside int32.
// ---------------------------------------------------------------------------
DYM_HD int dym_fix_shift(double amax, int D) {
  const double NR = 6.0 * (D - 1);
  const double a = amax > 1e-3 ? amax : 1e-3;
  const double lim = (2147483647.0 - 2.0 * NR) / (2.0 * NR * a);
  int S = 24;
  while (S > 0 && ldexp(1.0, S) > lim) --S;
  return S;
}
