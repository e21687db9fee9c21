// Device-side lattice geometry and staple construction.
//
// Site index i = t + Nt*(x1 + Nx*(x2 + ...)) with periodic wrap (lattice.c
// getidx/getpos, lattice.c:119-132 of the reference).  Links are stored
// direction-major: links[dir*V + site], uint16 element ids.
#pragma once
#include <stdint.h>

namespace dym {

// Relative index offsets for a move of -2..+2 along each axis from the site's
// own coordinates: off[b][k] = (wrap(x_b + k - 2) - x_b) * stride_b.
template <int D>
struct SiteGeo {
  int off[D][5];
};

// Periodic wrap of c = x + s, 0 <= x < N, |s| <= 2 (two corrections each way
// cover N = 1).
__device__ __forceinline__ int wrap_near(int c, int N) {
  if (c < 0) c += N;
  if (c < 0) c += N;
  if (c >= N) c -= N;
  if (c >= N) c -= N;
  return c;
}

// Offsets from the site's coordinates x[0..D-1] (x[0] temporal).
template <int D>
__device__ __forceinline__ void site_geo_xyz(const int* x, int Nt, int Nx, SiteGeo<D>& g) {
  int stride = 1;
#pragma unroll
  for (int b = 0; b < D; ++b) {
    const int N = (b == 0) ? Nt : Nx;
#pragma unroll
    for (int k = 0; k < 5; ++k) g.off[b][k] = (wrap_near(x[b] + k - 2, N) - x[b]) * stride;
    stride *= N;
  }
}

template <int D>
__device__ __forceinline__ void site_geo(uint32_t i, int Nt, int Nx, SiteGeo<D>& g) {
  int x[D];
#pragma unroll
  for (int b = 0; b < D; ++b) {
    const uint32_t N = (uint32_t)((b == 0) ? Nt : Nx);
    x[b] = (int)(i % N);
    i /= N;
  }
  site_geo_xyz<D>(x, Nt, Nx, g);
}

// Coordinates packed 8 bits per axis (x[0] in the low byte), extents <= 256.
template <int D>
__device__ __forceinline__ void site_geo_packed(uint32_t xyz, int Nt, int Nx, SiteGeo<D>& g) {
  int x[D];
#pragma unroll
  for (int b = 0; b < D; ++b) x[b] = (int)((xyz >> (8 * b)) & 0xFFu);
  site_geo_xyz<D>(x, Nt, Nx, g);
}

// The same offsets with one compare and one select each: for an axis of
// extent N and stride s, a move of -2..+2 wraps at most once (N >= 2; N = 1
// maps every move to 0), so each offset is one of two per-axis constants.
// Equal to site_geo_packed for every extent.
template <int D>
__device__ __forceinline__ void site_geo_fast(uint32_t xyz, int Nt, int Nx, SiteGeo<D>& g) {
  int stride = 1;
#pragma unroll
  for (int b = 0; b < D; ++b) {
    const int N = (b == 0) ? Nt : Nx;
    const int x = (int)((xyz >> (8 * b)) & 0xFFu);
    const int s = stride;
    g.off[b][0] = (x < 2) ? (N >= 2 ? (N - 2) * s : 0) : -2 * s;
    g.off[b][1] = (x == 0) ? (N - 1) * s : -s;
    g.off[b][2] = 0;
    g.off[b][3] = (x == N - 1) ? (1 - N) * s : s;
    g.off[b][4] = (x >= N - 2) ? (N >= 2 ? (2 - N) * s : 0) : 2 * s;
    stride *= N;
  }
}

// Table access policies.  `Tab` provides mul(g, h), inv(g) for uint32 ids.
// Opt-in self-checking build (-DDYM_BOUNDS_CHECK): every table and lattice
// index is checked; the first bad one is recorded in *status as
// (code << 32 | value) and the access is skipped.
#ifdef DYM_BOUNDS_CHECK
__device__ __forceinline__ bool dym_bc(bool ok, unsigned long long* status, uint32_t code, uint32_t val) {
  if (!ok) {
    printf("bounds check failed: code %u value %u thread %u block %u status %p\n", code, val, threadIdx.x,
           blockIdx.x, (void*)status);
    if (status) atomicCAS(status, 0ull, ((unsigned long long)code << 32) | val);
  }
  return ok;
}
#define DYM_BC(ok, st, code, val) dym_bc((ok), (st), (code), (val))
#else
#define DYM_BC(ok, st, code, val) true
#endif

struct GlobalTab {
  const uint16_t* __restrict__ mult;  // P*P, L2-resident
  const uint16_t* inv;                // shared memory copy
  uint32_t P;
  unsigned long long* status = nullptr;  // only read by the self-checking build
  __device__ __forceinline__ uint32_t mul(uint32_t g, uint32_t h) const {
    if (!DYM_BC(g < P && h < P, status, 3, g < P ? h : g)) return 0;
    return __ldg(mult + g * P + h);
  }
  __device__ __forceinline__ uint32_t iv(uint32_t g) const {
    if (!DYM_BC(g < P, status, 4, g)) return 0;
    return inv[g];
  }
};

struct SharedTab {  // whole Cayley table staged in shared memory (small groups)
  const uint16_t* mult;
  const uint16_t* inv;
  uint32_t P;
  __device__ __forceinline__ uint32_t mul(uint32_t g, uint32_t h) const { return mult[g * P + h]; }
  __device__ __forceinline__ uint32_t iv(uint32_t g) const { return inv[g]; }
};

// Build the 2(D-1) plaquette staples then the 6(D-1) rectangle staples of link
// (i, DIR), element for element as get_staples (dym-mod-metro.cpp:63-78) and
// get_rect_loops (dym-mod-metro.cpp:83-142).  The reference's leading
// mult[id][x] in each rectangle is the identity map and is skipped.
// e = e_DIR, f = e_d1.  LD(site, dir) loads a link.
template <int D, int DIR, class Tab, class LD>
__device__ __forceinline__ void build_staples(uint32_t i, const SiteGeo<D>& geo, const Tab& T, LD ld,
                                              uint32_t* st /* 2(D-1) */, uint32_t* re /* 6(D-1) */) {
#define DYM_S(de, df) ((uint32_t)((int)i + geo.off[DIR][(de) + 2] + geo.off[d1][(df) + 2]))
  int k = 0, kr = 0;
#pragma unroll
  for (int d1 = 0; d1 < D; ++d1) {
    if (d1 == DIR) continue;
    // Loads shared by the staples of this (DIR, d1) plane.
    const uint32_t a_e_f1 = ld(DYM_S(1, 0), d1);      // a[i+e, d1]
    const uint32_t a_0_d1 = ld(DYM_S(0, 0), d1);      // a[i, d1]
    const uint32_t a_f_d = ld(DYM_S(0, 1), DIR);      // a[i+f, d]
    const uint32_t a_emf_f = ld(DYM_S(1, -1), d1);    // a[i+e-f, d1]
    const uint32_t a_mf_d = ld(DYM_S(0, -1), DIR);    // a[i-f, d]
    const uint32_t a_mf_f = ld(DYM_S(0, -1), d1);     // a[i-f, d1]
    const uint32_t a_e_d = ld(DYM_S(1, 0), DIR);      // a[i+e, d]
    const uint32_t a_me_d = ld(DYM_S(-1, 0), DIR);    // a[i-e, d]
    const uint32_t a_me_f = ld(DYM_S(-1, 0), d1);     // a[i-e, d1]
    // Plaquette staples (dym-mod-metro.cpp:68-76).
    {
      uint32_t g = T.mul(a_e_f1, T.iv(a_f_d));
      st[k++] = T.mul(g, T.iv(a_0_d1));
      g = T.mul(T.iv(a_emf_f), T.iv(a_mf_d));
      st[k++] = T.mul(g, a_mf_f);
    }
    // Rectangle 1 (:88-95): a[i+e,f] a[i+e+f,f] a[i+2f,d]^-1 a[i+f,f]^-1 a[i,f]^-1
    {
      uint32_t g = T.mul(a_e_f1, ld(DYM_S(1, 1), d1));
      g = T.mul(g, T.iv(ld(DYM_S(0, 2), DIR)));
      g = T.mul(g, T.iv(ld(DYM_S(0, 1), d1)));
      re[kr++] = T.mul(g, T.iv(a_0_d1));
    }
    // Rectangle 2 (:97-104): a[i+e,d] a[i+2e,f] a[i+e+f,d]^-1 a[i+f,d]^-1 a[i,f]^-1
    {
      uint32_t g = T.mul(a_e_d, ld(DYM_S(2, 0), d1));
      g = T.mul(g, T.iv(ld(DYM_S(1, 1), DIR)));
      g = T.mul(g, T.iv(a_f_d));
      re[kr++] = T.mul(g, T.iv(a_0_d1));
    }
    // Rectangle 3 (:106-113): a[i+e,f] a[i+f,d]^-1 a[i+f-e,d]^-1 a[i-e,f]^-1 a[i-e,d]
    {
      uint32_t g = T.mul(a_e_f1, T.iv(a_f_d));
      g = T.mul(g, T.iv(ld(DYM_S(-1, 1), DIR)));
      g = T.mul(g, T.iv(a_me_f));
      re[kr++] = T.mul(g, a_me_d);
    }
    // Rectangle 4 (:115-122): a[i+e-f,f]^-1 a[i+e-2f,f]^-1 a[i-2f,d]^-1 a[i-2f,f] a[i-f,f]
    {
      uint32_t g = T.mul(T.iv(a_emf_f), T.iv(ld(DYM_S(1, -2), d1)));
      g = T.mul(g, T.iv(ld(DYM_S(0, -2), DIR)));
      g = T.mul(g, ld(DYM_S(0, -2), d1));
      re[kr++] = T.mul(g, a_mf_f);
    }
    // Rectangle 5 (:124-131): a[i+e,d] a[i+2e-f,f]^-1 a[i+e-f,d]^-1 a[i-f,d]^-1 a[i-f,f]
    {
      uint32_t g = T.mul(a_e_d, T.iv(ld(DYM_S(2, -1), d1)));
      g = T.mul(g, T.iv(ld(DYM_S(1, -1), DIR)));
      g = T.mul(g, T.iv(a_mf_d));
      re[kr++] = T.mul(g, a_mf_f);
    }
    // Rectangle 6 (:133-140): a[i+e-f,f]^-1 a[i-f,d]^-1 a[i-f-e,d]^-1 a[i-e-f,f] a[i-e,d]
    {
      uint32_t g = T.mul(T.iv(a_emf_f), T.iv(a_mf_d));
      g = T.mul(g, T.iv(ld(DYM_S(-1, -1), DIR)));
      g = T.mul(g, ld(DYM_S(-1, -1), d1));
      re[kr++] = T.mul(g, a_me_d);
    }
  }
#undef DYM_S
}

// u_j = s_j * b for the staples of build_staples, in its order (2(D-1)
// plaquette terms into up, 6(D-1) rectangle terms into ur), for associative
// tables.  Each u_j is the product of the same factors in the same order as
// build_staples' s_j followed by b; only the grouping differs.  The tails
// a[i,f]^-1 b (plaquette 1, rectangles 1 and 2), a[i-f,f] b (plaquette 2,
// rectangles 4 and 5) and a[i-e,d] b (rectangles 3 and 6) and the heads
// a[i+e,f] a[i+f,d]^-1 (plaquette 1, rectangle 3) and
// a[i+e-f,f]^-1 a[i-f,d]^-1 (plaquette 2, rectangle 6) are formed once, and
// the rest is grouped pairwise: 29 table products per plane instead of 36,
// at most three dependent on one another instead of five, and 11 inverse
// lookups.
template <int D, int DIR, class Tab, class LD>
__device__ __forceinline__ void build_u_tree(uint32_t i, const SiteGeo<D>& geo, const Tab& T, LD ld, uint32_t b,
                                             uint32_t* up /* 2(D-1) */, uint32_t* ur /* 6(D-1) */) {
#define DYM_S(de, df) ((uint32_t)((int)i + geo.off[DIR][(de) + 2] + geo.off[d1][(df) + 2]))
  int k = 0, kr = 0;
#pragma unroll
  for (int d1 = 0; d1 < D; ++d1) {
    if (d1 == DIR) continue;
    const uint32_t a_e_f1 = ld(DYM_S(1, 0), d1);    // a[i+e, f]
    const uint32_t a_0_d1 = ld(DYM_S(0, 0), d1);    // a[i, f]
    const uint32_t a_f_d = ld(DYM_S(0, 1), DIR);    // a[i+f, d]
    const uint32_t a_emf_f = ld(DYM_S(1, -1), d1);  // a[i+e-f, f]
    const uint32_t a_mf_d = ld(DYM_S(0, -1), DIR);  // a[i-f, d]
    const uint32_t a_mf_f = ld(DYM_S(0, -1), d1);   // a[i-f, f]
    const uint32_t a_e_d = ld(DYM_S(1, 0), DIR);    // a[i+e, d]
    const uint32_t a_me_d = ld(DYM_S(-1, 0), DIR);  // a[i-e, d]
    const uint32_t a_me_f = ld(DYM_S(-1, 0), d1);   // a[i-e, f]
    const uint32_t l_ef_f = ld(DYM_S(1, 1), d1);    // a[i+e+f, f]
    const uint32_t l_2f_d = ld(DYM_S(0, 2), DIR);   // a[i+2f, d]
    const uint32_t l_f_f = ld(DYM_S(0, 1), d1);     // a[i+f, f]
    const uint32_t l_2e_f = ld(DYM_S(2, 0), d1);    // a[i+2e, f]
    const uint32_t l_ef_d = ld(DYM_S(1, 1), DIR);   // a[i+e+f, d]
    const uint32_t l_fme_d = ld(DYM_S(-1, 1), DIR);  // a[i+f-e, d]
    const uint32_t l_e2f_f = ld(DYM_S(1, -2), d1);  // a[i+e-2f, f]
    const uint32_t l_m2f_d = ld(DYM_S(0, -2), DIR);  // a[i-2f, d]
    const uint32_t l_m2f_f = ld(DYM_S(0, -2), d1);  // a[i-2f, f]
    const uint32_t l_2emf_f = ld(DYM_S(2, -1), d1);  // a[i+2e-f, f]
    const uint32_t l_emf_d = ld(DYM_S(1, -1), DIR);  // a[i+e-f, d]
    const uint32_t l_mfme_d = ld(DYM_S(-1, -1), DIR);  // a[i-f-e, d]
    const uint32_t l_mfme_f = ld(DYM_S(-1, -1), d1);   // a[i-e-f, f]
    // First level: every product of two links (or link and b).  A product of
    // two inverses is taken as the inverse of the reversed product, x^-1 y^-1
    // = (y x)^-1: one inverse lookup instead of two, the same element.
    const uint32_t q0 = T.mul(T.iv(a_0_d1), b);
    const uint32_t q1 = T.mul(a_mf_f, b);
    const uint32_t q2 = T.mul(a_me_d, b);
    const uint32_t h0 = T.mul(a_e_f1, T.iv(a_f_d));
    const uint32_t h1 = T.iv(T.mul(a_mf_d, a_emf_f));
    const uint32_t p1a = T.mul(a_e_f1, l_ef_f), p1b = T.iv(T.mul(l_f_f, l_2f_d));
    const uint32_t p2a = T.mul(a_e_d, l_2e_f), p2b = T.iv(T.mul(a_f_d, l_ef_d));
    const uint32_t p3b = T.iv(T.mul(a_me_f, l_fme_d));
    const uint32_t p4a = T.iv(T.mul(l_e2f_f, a_emf_f)), p4b = T.mul(T.iv(l_m2f_d), l_m2f_f);
    const uint32_t p5a = T.mul(a_e_d, T.iv(l_2emf_f)), p5b = T.iv(T.mul(a_mf_d, l_emf_d));
    const uint32_t p6b = T.mul(T.iv(l_mfme_d), l_mfme_f);
    // Plaquettes (dym-mod-metro.cpp:68-76) and rectangles 1-6 (:88-140), times b.
    up[k++] = T.mul(h0, q0);
    up[k++] = T.mul(h1, q1);
    ur[kr++] = T.mul(T.mul(p1a, p1b), q0);
    ur[kr++] = T.mul(T.mul(p2a, p2b), q0);
    ur[kr++] = T.mul(T.mul(h0, p3b), q2);
    ur[kr++] = T.mul(T.mul(p4a, p4b), q1);
    ur[kr++] = T.mul(T.mul(p5a, p5b), q1);
    ur[kr++] = T.mul(T.mul(h1, p6b), q2);
  }
#undef DYM_S
}

// One side of the u_j = s_j * b of build_u_tree, for a lane pair sharing
// link (i, DIR): per plane (DIR, f), f = e_d1, the staples on the +f side
// (back false: plaquette 1 and rectangles 1-3 of build_staples) or on the -f
// side (back true: plaquette 2 and rectangles 4-6, which are the +f staples
// with f reflected).  With sg = +1 or -1 and F(y, s) the step from y along
// s f (a[y,f] for s = +1, a[y-f,f]^-1 for s = -1), the four elements are
//   plaquette    F(i+e, sg) a[i+sg f,d]^-1 F(i+sg f, -sg) b
//   rectangle 1  F(i+e, sg) F(i+e+sg f, sg) a[i+2sg f,d]^-1 F(i+2sg f, -sg) F(i+sg f, -sg) b
//   rectangle 2  a[i+e,d] F(i+2e, sg) a[i+e+sg f,d]^-1 a[i+sg f,d]^-1 F(i+sg f, -sg) b
//   rectangle 3  F(i+e, sg) a[i+sg f,d]^-1 a[i+sg f-e,d]^-1 F(i-e+sg f, -sg) a[i-e,d] b
// (for sg = -1 these are rectangles 4, 5 and 6).  Both lanes run the same
// instructions: the side only selects site offsets and which loaded links
// are inverted.  12 link loads and 15 table products per plane and lane.
// up gets D-1 plaquette terms, ur 3(D-1) rectangle terms, plane by plane.
template <int D, int DIR, class Tab, class LD>
__device__ __forceinline__ void build_u_half(uint32_t i, const SiteGeo<D>& geo, const Tab& T, LD ld, uint32_t b,
                                             bool back, uint32_t* up /* D-1 */, uint32_t* ur /* 3(D-1) */) {
  int k = 0, kr = 0;
#pragma unroll
  for (int d1 = 0; d1 < D; ++d1) {
    if (d1 == DIR) continue;
    // f offsets of this side: +-1, +-2 and the F steps' site shifts.
    const int* fo = geo.off[d1];
    const int f1 = back ? fo[1] : fo[3];    // sg f
    const int f2 = back ? fo[0] : fo[4];    // 2 sg f
    const int fF = back ? fo[1] : fo[2];    // site of F(y, sg): y - f or y
    const int fF1 = back ? fo[0] : fo[3];   // site of F(y + sg f, sg)
    const int fB = back ? fo[1] : fo[2];    // site of F(y + sg f, -sg): y - f or y
    const int fB2 = back ? fo[0] : fo[3];   // site of F(y + 2 sg f, -sg)
    const int* eo = geo.off[DIR];
    const int ip = (int)i;
    auto maybe_inv = [&](uint32_t x, bool inv) -> uint32_t {
      const uint32_t xi = T.iv(x);
      return inv ? xi : x;
    };
    // F(., sg) is inverted on the -f side, F(., -sg) on the +f side.
    const uint32_t F1 = maybe_inv(ld((uint32_t)(ip + eo[3] + fF), d1), back);     // F(i+e, sg)
    const uint32_t F2 = maybe_inv(ld((uint32_t)(ip + eo[3] + fF1), d1), back);    // F(i+e+sg f, sg)
    const uint32_t F3 = maybe_inv(ld((uint32_t)(ip + eo[4] + fF), d1), back);     // F(i+2e, sg)
    const uint32_t G1 = maybe_inv(ld((uint32_t)(ip + fB), d1), !back);            // F(i+sg f, -sg)
    const uint32_t G2 = maybe_inv(ld((uint32_t)(ip + fB2), d1), !back);           // F(i+2sg f, -sg)
    const uint32_t G3 = maybe_inv(ld((uint32_t)(ip + eo[1] + fB), d1), !back);    // F(i-e+sg f, -sg)
    const uint32_t Bd = T.iv(ld((uint32_t)(ip + f1), DIR));                        // a[i+sg f,d]^-1
    const uint32_t B2 = T.iv(ld((uint32_t)(ip + f2), DIR));                        // a[i+2sg f,d]^-1
    const uint32_t Be = T.iv(ld((uint32_t)(ip + eo[3] + f1), DIR));                // a[i+e+sg f,d]^-1
    const uint32_t Bm = T.iv(ld((uint32_t)(ip + eo[1] + f1), DIR));                // a[i+sg f-e,d]^-1
    const uint32_t Ae = ld((uint32_t)(ip + eo[3]), DIR);                           // a[i+e,d]
    const uint32_t Am = ld((uint32_t)(ip + eo[1]), DIR);                           // a[i-e,d]
    const uint32_t Cq = T.mul(G1, b);
    const uint32_t q2 = T.mul(Am, b);
    const uint32_t h = T.mul(F1, Bd);
    const uint32_t r1a = T.mul(F1, F2), r1b = T.mul(B2, G2);
    const uint32_t r2a = T.mul(Ae, F3), r2b = T.mul(Be, Bd);
    const uint32_t r3b = T.mul(Bm, G3);
    up[k++] = T.mul(h, Cq);
    ur[kr++] = T.mul(T.mul(r1a, r1b), Cq);
    ur[kr++] = T.mul(T.mul(r2a, r2b), Cq);
    ur[kr++] = T.mul(T.mul(h, r3b), q2);
  }
}

}  // namespace dym
