// Metropolis sweep kernels: one thread per link of one colour phase.
//
// Two kernels implement the hit loop of dym-mod-metro.cpp:161-192:
//
//  * k_sweep_direct  -- the reference's arithmetic verbatim: every hit gathers
//    mult[bnew][staple] for all 24 staples (4D) from the L2-resident Cayley
//    table and sums ReTr in FP64 in the reference's order.
//
//  * k_sweep_fast    -- same decisions, restructured.  With u_j = s_j * b
//    (staple times current link), Tr(bnew s_j) = Tr(b g s_j) = Tr(g s_j b)
//    = Tr(g u_j): the proposal's terms depend only on (g, u_j).  For the
//    nearest-to-identity pool (72 elements for S(1080)) the products u*g and
//    their ReTr class fit in shared memory as one uint16 table sub[k][u] =
//    (u*g_k) | class << shift (155 KB for S(1080)), so a hit is 24 shared
//    loads instead of 24 L2 gathers; an accepted hit advances u_j <- u_j*g_k
//    from the same entries.  dS is summed in FP32 from per-class values; a
//    decision closer to its threshold than the proven error bound is
//    re-evaluated in FP64 in the reference's order, so accepted
//    configurations are identical to the FP64 path.
#include <cuda_runtime.h>

#include "chain.h"
#include "dym_core.h"
#include "staples.cuh"

namespace dym {

namespace {

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

// Max of non-negative doubles via their ordered bit patterns.
__device__ __forceinline__ void atomic_max_nonneg(double* addr, double v) {
  atomicMax((unsigned long long*)addr, (unsigned long long)__double_as_longlong(v));
}

template <int D, int DIR>
__global__ void __launch_bounds__(256) k_sweep_direct(SweepArgs a) {
  constexpr int NS = 2 * (D - 1), NR = 6 * (D - 1);
  extern __shared__ __align__(16) unsigned char smem[];
  double* s_retr = reinterpret_cast<double*>(smem);
  uint16_t* s_inv = reinterpret_cast<uint16_t*>(s_retr + a.P);
  uint16_t* s_pool = s_inv + a.P;
  for (uint32_t t = threadIdx.x; t < a.P; t += blockDim.x) {
    s_retr[t] = a.retr[t];
    s_inv[t] = a.inv[t];
  }
  for (uint32_t t = threadIdx.x; t < a.npool; t += blockDim.x) s_pool[t] = a.pool[t];
  __syncthreads();

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
    uint32_t st[NS], re[NR];
    build_staples<D, DIR>(i, geo, T, ld, st, re);

    uint16_t* own = a.links + (size_t)DIR * V + i;
    uint32_t b = *own;
    const uint32_t b0 = b;
    double r1 = 0, m1 = 0;
#pragma unroll
    for (int j = 0; j < NS; ++j) r1 = DYM_ADD(r1, s_retr[T.mul(b, st[j])]);
#pragma unroll
    for (int k = 0; k < NR; ++k) m1 = DYM_ADD(m1, s_retr[T.mul(b, re[k])]);
    for (int h = 0; h < a.nhit; ++h) {
      const dym_u32x4 r = dym_hit_random(a.seed, a.sweep, i, DIR, (uint32_t)h, DYM_TAG_METRO);
      const uint32_t g = s_pool[dym_pick(r.v[0], a.npool)];
      const uint32_t bnew = T.mul(b, g);
      double r1n = 0, m1n = 0;
#pragma unroll
      for (int j = 0; j < NS; ++j) r1n = DYM_ADD(r1n, s_retr[T.mul(bnew, st[j])]);
#pragma unroll
      for (int k = 0; k < NR; ++k) m1n = DYM_ADD(m1n, s_retr[T.mul(bnew, re[k])]);
      const double oldact = dym_action(a.beta0, a.beta1, a.beta2, r1, m1);
      const double newact = dym_action(a.beta0, a.beta1, a.beta2, r1n, m1n);
      ++hits;
      if (dym_accept(oldact, newact, dym_u53(r.v[1], r.v[2]))) {
        b = bnew;
        r1 = r1n;
        m1 = m1n;
        ++accs;
      }
    }
    if (b != b0) *own = (uint16_t)b;
  }
  flush_counters(a.counters, hits, accs, 0);
}

// ---------------------------------------------------------------------------
// Mixed-precision shared sub-table kernel.
// ---------------------------------------------------------------------------
template <int D, int DIR>
__global__ void __launch_bounds__(512, 1) k_sweep_fast(SweepArgs a, FastTables ft, double* maxerr) {
  constexpr int NS = 2 * (D - 1), NR = 6 * (D - 1), NT = NS + NR;
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t P = a.P;
  uint16_t* s_sub = reinterpret_cast<uint16_t*>(smem);                       // npool*P
  double* s_retr = reinterpret_cast<double*>(smem + ((size_t)a.npool * P * 2 + 15) / 16 * 16);  // P
  double* s_cv64 = s_retr + P;                                               // ncls
  float* s_cv32 = reinterpret_cast<float*>(s_cv64 + ft.ncls);                // ncls
  uint16_t* s_inv = reinterpret_cast<uint16_t*>(s_cv32 + ft.ncls);           // P
  uint8_t* s_cls = reinterpret_cast<uint8_t*>(s_inv + P);                    // P

  {
    const uint4* src = reinterpret_cast<const uint4*>(ft.sub);
    uint4* dst = reinterpret_cast<uint4*>(s_sub);
    const uint32_t nsub = a.npool * P;
    const uint32_t n16 = nsub / 8;
    for (uint32_t t = threadIdx.x; t < n16; t += blockDim.x) dst[t] = __ldg(src + t);
    for (uint32_t t = n16 * 8 + threadIdx.x; t < nsub; t += blockDim.x) s_sub[t] = ft.sub[t];
    for (uint32_t t = threadIdx.x; t < P; t += blockDim.x) {
      s_retr[t] = a.retr[t];
      s_inv[t] = a.inv[t];
      s_cls[t] = ft.cls[t];
    }
    for (uint32_t t = threadIdx.x; t < (uint32_t)ft.ncls; t += blockDim.x) {
      s_cv64[t] = ft.cls_val64[t];
      s_cv32[t] = ft.cls_val32[t];
    }
  }
  __syncthreads();

  const uint32_t mask = (1u << ft.shift) - 1u;
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned hits = 0, accs = 0, rechecks = 0;
  double lmaxerr = 0;
  if (tid < a.n) {
    const uint32_t i = a.sites[tid];
    SiteGeo<D> geo;
    site_geo<D>(i, a.Nt, a.Nx, geo);
    GlobalTab T{a.mult, s_inv, P};
    const uint16_t* L = a.links;
    const uint32_t V = a.V;
    auto ld = [L, V](uint32_t s, int d) -> uint32_t { return __ldg(L + (size_t)d * V + s); };
    uint32_t u[NT];
    build_staples<D, DIR>(i, geo, T, ld, u, u + NS);

    uint16_t* own = a.links + (size_t)DIR * V + i;
    uint32_t b = *own;
    const uint32_t b0 = b;
#pragma unroll
    for (int j = 0; j < NT; ++j) u[j] = T.mul(u[j], b);  // u_j = s_j * b
    const float b1f = (float)a.beta1, b2f = (float)a.beta2;
    float r1 = 0.f, m1 = 0.f;
#pragma unroll
    for (int j = 0; j < NS; ++j) r1 += s_cv32[s_cls[u[j]]];
#pragma unroll
    for (int j = NS; j < NT; ++j) m1 += s_cv32[s_cls[u[j]]];

    for (int h = 0; h < a.nhit; ++h) {
      const dym_u32x4 r = dym_hit_random(a.seed, a.sweep, i, DIR, (uint32_t)h, DYM_TAG_METRO);
      const uint32_t k = dym_pick(r.v[0], a.npool);
      const uint16_t* row = s_sub + k * P;
      uint32_t e[NT];
#pragma unroll
      for (int j = 0; j < NT; ++j) e[j] = row[u[j]];
      float r1n = 0.f, m1n = 0.f;
#pragma unroll
      for (int j = 0; j < NS; ++j) r1n += s_cv32[e[j] >> ft.shift];
#pragma unroll
      for (int j = NS; j < NT; ++j) m1n += s_cv32[e[j] >> ft.shift];
      const float ds = b1f * (r1n - r1) + b2f * (m1n - m1);
      const double u2 = dym_u53(r.v[1], r.v[2]);
      const float epsf = (float)ft.eps;
      int decision;  // 1 accept, 0 reject, -1 recheck
      if (ds < -epsf) {
        decision = 1;
      } else if (ds > epsf) {
        // __expf has at most 2 + 1.173|x| ulp of error; the rest of the
        // margin covers rounding u2 and q*(1+-m) to FP32.
        const float q = __expf(-ds);
        const float m = 2.0f * epsf + (4.0f + 1.2f * ds) * 1.2e-7f + 1e-6f;
        const float u2f = (float)u2;
        if (u2f < q * (1.0f - m)) decision = 1;
        else if (u2f > q * (1.0f + m)) decision = 0;
        else decision = -1;
      } else {
        decision = -1;
      }
      if (decision < 0) {
        // FP64 re-evaluation in the reference's order (dym-mod-metro.cpp:166-187).
        ++rechecks;
        double r1d = 0, m1d = 0, r1nd = 0, m1nd = 0;
        if (ft.exact) {
#pragma unroll
          for (int j = 0; j < NS; ++j) {
            r1d = DYM_ADD(r1d, s_cv64[s_cls[u[j]]]);
            r1nd = DYM_ADD(r1nd, s_cv64[e[j] >> ft.shift]);
          }
#pragma unroll
          for (int j = NS; j < NT; ++j) {
            m1d = DYM_ADD(m1d, s_cv64[s_cls[u[j]]]);
            m1nd = DYM_ADD(m1nd, s_cv64[e[j] >> ft.shift]);
          }
        } else {
          // ReTr of the exact elements b*s_j and bnew*s_j, s_j = u_j * b^-1.
          const uint32_t bi = s_inv[b];
          const uint32_t bnew = row[b] & mask;
#pragma unroll
          for (int j = 0; j < NT; ++j) {
            const uint32_t s = T.mul(u[j], bi);
            const double vo = s_retr[T.mul(b, s)];
            const double vn = s_retr[T.mul(bnew, s)];
            if (j < NS) { r1d = DYM_ADD(r1d, vo); r1nd = DYM_ADD(r1nd, vn); }
            else { m1d = DYM_ADD(m1d, vo); m1nd = DYM_ADD(m1nd, vn); }
          }
        }
        const double oldact = dym_action(a.beta0, a.beta1, a.beta2, r1d, m1d);
        const double newact = dym_action(a.beta0, a.beta1, a.beta2, r1nd, m1nd);
        decision = dym_accept(oldact, newact, u2) ? 1 : 0;
        const double err = fabs((double)ds - DYM_SUB(newact, oldact));
        lmaxerr = fmax(lmaxerr, err);
      }
      ++hits;
      if (decision) {
        b = row[b] & mask;
#pragma unroll
        for (int j = 0; j < NT; ++j) u[j] = e[j] & mask;
        r1 = r1n;
        m1 = m1n;
        ++accs;
      }
    }
    if (b != b0) *own = (uint16_t)b;
  }
  flush_counters(a.counters, hits, accs, rechecks);
  if (lmaxerr > 0) atomic_max_nonneg(maxerr, lmaxerr);
}

__global__ void k_hot_start(uint16_t* links, uint32_t V, int D, uint32_t P, uint64_t seed) {
  const size_t n = (size_t)V * D;
  for (size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) {
    const uint32_t dir = (uint32_t)(l / V), site = (uint32_t)(l % V);
    dym_u32x4 c;
    c.v[0] = site;
    c.v[1] = 0;
    c.v[2] = dir;
    c.v[3] = DYM_TAG_HOT;
    const dym_u32x4 r = dym_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    links[l] = (uint16_t)dym_pick(r.v[0], P);
  }
}

__global__ void k_fill(uint16_t* p, size_t n, uint16_t v) {
  for (size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x; l < n; l += (size_t)gridDim.x * blockDim.x) p[l] = v;
}

template <int D, int DIR>
__global__ void k_staples(SweepArgs a, const uint32_t* sites, uint32_t n, uint16_t* out) {
  constexpr int NS = 2 * (D - 1), NR = 6 * (D - 1);
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= n) return;
  const uint32_t i = sites[tid];
  SiteGeo<D> geo;
  site_geo<D>(i, a.Nt, a.Nx, geo);
  GlobalTab T{a.mult, a.inv, a.P};
  const uint16_t* L = a.links;
  const uint32_t V = a.V;
  auto ld = [L, V](uint32_t s, int d) -> uint32_t { return L[(size_t)d * V + s]; };
  uint32_t st[NS], re[NR];
  build_staples<D, DIR>(i, geo, T, ld, st, re);
  for (int j = 0; j < NS; ++j) out[(size_t)tid * (NS + NR) + j] = (uint16_t)st[j];
  for (int j = 0; j < NR; ++j) out[(size_t)tid * (NS + NR) + NS + j] = (uint16_t)re[j];
}

template <int D>
cudaError_t direct_dispatch(int dir, const SweepArgs& a, cudaStream_t s) {
  const size_t smem = (size_t)a.P * 8 + (size_t)a.P * 2 + (size_t)a.npool * 2 + 16;
  const unsigned grid = (a.n + 255) / 256;
  void (*fn)(SweepArgs) = nullptr;
  switch (dir) {
    case 0: fn = k_sweep_direct<D, 0>; break;
    case 1: fn = k_sweep_direct<D, 1>; break;
    case 2: if (D > 2) fn = k_sweep_direct<D, (D > 2 ? 2 : 0)>; break;
    case 3: if (D > 3) fn = k_sweep_direct<D, (D > 3 ? 3 : 0)>; break;
  }
  if (!fn) return cudaErrorInvalidValue;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  if (grid == 0) return cudaSuccess;
  fn<<<grid, 256, smem, s>>>(a);
  return cudaGetLastError();
}

template <int D>
cudaError_t fast_dispatch(int dir, const SweepArgs& a, const FastTables& ft, double* maxerr, cudaStream_t s) {
  const size_t smem = fast_smem_bytes(a.P, a.npool, ft.ncls);
  const unsigned threads = 512;
  const unsigned grid = (a.n + threads - 1) / threads;
  void (*fn)(SweepArgs, FastTables, double*) = nullptr;
  switch (dir) {
    case 0: fn = k_sweep_fast<D, 0>; break;
    case 1: fn = k_sweep_fast<D, 1>; break;
    case 2: if (D > 2) fn = k_sweep_fast<D, (D > 2 ? 2 : 0)>; break;
    case 3: if (D > 3) fn = k_sweep_fast<D, (D > 3 ? 3 : 0)>; break;
  }
  if (!fn) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (grid == 0) return cudaSuccess;
  fn<<<grid, threads, smem, s>>>(a, ft, maxerr);
  return cudaGetLastError();
}

template <int D>
cudaError_t staples_dispatch(int dir, const SweepArgs& a, const uint32_t* sites, uint32_t n, uint16_t* out,
                             cudaStream_t s) {
  void (*fn)(SweepArgs, const uint32_t*, uint32_t, uint16_t*) = nullptr;
  switch (dir) {
    case 0: fn = k_staples<D, 0>; break;
    case 1: fn = k_staples<D, 1>; break;
    case 2: if (D > 2) fn = k_staples<D, (D > 2 ? 2 : 0)>; break;
    case 3: if (D > 3) fn = k_staples<D, (D > 3 ? 3 : 0)>; break;
  }
  if (!fn) return cudaErrorInvalidValue;
  if (n == 0) return cudaSuccess;
  fn<<<(n + 127) / 128, 128, 0, s>>>(a, sites, n, out);
  return cudaGetLastError();
}

}  // namespace

size_t fast_smem_bytes(uint32_t P, uint32_t npool, int ncls) {
  size_t sub = ((size_t)npool * P * 2 + 15) / 16 * 16;
  return sub + (size_t)P * 8 + (size_t)ncls * 12 + (size_t)P * 3 + 16;
}

cudaError_t launch_sweep_direct(int D, int dir, const SweepArgs& a, cudaStream_t s) {
  switch (D) {
    case 2: return direct_dispatch<2>(dir, a, s);
    case 3: return direct_dispatch<3>(dir, a, s);
    case 4: return direct_dispatch<4>(dir, a, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_sweep_fast(int D, int dir, const SweepArgs& a, const FastTables& ft, double* maxerr,
                              cudaStream_t s) {
  switch (D) {
    case 2: return fast_dispatch<2>(dir, a, ft, maxerr, s);
    case 3: return fast_dispatch<3>(dir, a, ft, maxerr, s);
    case 4: return fast_dispatch<4>(dir, a, ft, maxerr, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_staples(int D, int dir, const SweepArgs& a, const uint32_t* sites, uint32_t n, uint16_t* out,
                           cudaStream_t s) {
  switch (D) {
    case 2: return staples_dispatch<2>(dir, a, sites, n, out, s);
    case 3: return staples_dispatch<3>(dir, a, sites, n, out, s);
    case 4: return staples_dispatch<4>(dir, a, sites, n, out, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_hot_start(uint16_t* links, uint32_t V, int D, uint32_t P, uint64_t seed, cudaStream_t s) {
  const size_t n = (size_t)V * D;
  unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 16);
  if (grid == 0) return cudaSuccess;
  k_hot_start<<<grid, 256, 0, s>>>(links, V, D, P, seed);
  return cudaGetLastError();
}

cudaError_t launch_fill(uint16_t* links, size_t n, uint16_t v, cudaStream_t s) {
  unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 16);
  if (grid == 0) return cudaSuccess;
  k_fill<<<grid, 256, 0, s>>>(links, n, v);
  return cudaGetLastError();
}

}  // namespace dym
