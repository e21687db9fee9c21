// Observables: plaquette, 1x2 rectangle, Polyakov loop and the Wilson-loop grid
// (dym-mod-metro.cpp:282-318; loop products lattice.c:157-205).
//
// Every loop is computed as a group element and counted in an exact integer
// histogram over the P elements (block-local shared-memory bins flushed with
// 64-bit atomics), so the sums are order-independent; the host then takes one
// FP64 dot product with ReTr/ImTr per observable.
//
// Wilson loops W(k+1, l+1) in the (d1, t) plane use line products: with
// X_k(i) the product of the k+1 links along d1 from i and T_l(i) the l+1
// temporal links from i, the reference's walk (lattice.c:197-205) equals
// X_k(i) * T_l(i + (k+1) e_d1) * X_k(i + (l+1) e_t)^-1 * T_l(i)^-1 by
// associativity of the group table, i.e. three table products per loop instead
// of 2(k+l+2).  Tables that fail the associativity check use the walk as
// written.
#include <cuda_runtime.h>

#include "chain.h"
#include "staples.cuh"

namespace dym {

namespace {

struct Geo {
  int Nt, Nx;
  uint32_t V;
};

template <int D>
__device__ __forceinline__ void coords(uint32_t i, int Nt, int Nx, int* x) {
  x[0] = (int)(i % (uint32_t)Nt);
  i /= (uint32_t)Nt;
#pragma unroll
  for (int b = 1; b < D; ++b) {
    x[b] = (int)(i % (uint32_t)Nx);
    i /= (uint32_t)Nx;
  }
}

template <int D>
__device__ __forceinline__ uint32_t index_of(const int* x, int Nt, int Nx) {
  uint32_t idx = 0;
#pragma unroll
  for (int b = D - 1; b > 0; --b) idx = (uint32_t)(((x[b] % Nx) + Nx) % Nx) + (uint32_t)Nx * idx;
  return (uint32_t)(((x[0] % Nt) + Nt) % Nt) + (uint32_t)Nt * idx;
}

// Site reached from i by moving s along axis b.
template <int D>
__device__ __forceinline__ uint32_t shift_site(uint32_t i, int b, int s, int Nt, int Nx) {
  int x[D];
  coords<D>(i, Nt, Nx, x);
#pragma unroll
  for (int c = 0; c < D; ++c)
    if (c == b) x[c] += s;
  return index_of<D>(x, Nt, Nx);
}

__device__ __forceinline__ uint32_t lnk(const MeasArgs& m, uint32_t site, int dir) {
  return m.links[(size_t)dir * m.V + site];
}
__device__ __forceinline__ uint32_t mul(const MeasArgs& m, uint32_t g, uint32_t h) {
  return __ldg(m.mult + g * m.P + h);
}

__device__ __forceinline__ void flush_hist(const uint32_t* s, unsigned long long* g, uint32_t P) {
  for (uint32_t t = threadIdx.x; t < P; t += blockDim.x)
    if (s[t]) atomicAdd(g + t, (unsigned long long)s[t]);
}

// Plaquettes, rectangles and Polyakov loops: one thread per site.
template <int D>
__global__ void k_hist_local(MeasArgs m, unsigned long long* hist) {
  extern __shared__ uint32_t sh[];
  uint32_t* hp = sh;
  uint32_t* hr = sh + m.P;
  uint32_t* hy = sh + 2 * m.P;
  for (uint32_t t = threadIdx.x; t < 3 * m.P; t += blockDim.x) sh[t] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m.V; i += gridDim.x * blockDim.x) {
    int x[D];
    coords<D>(i, m.Nt, m.Nx, x);
    for (int d1 = 0; d1 < D; ++d1) {
      const uint32_t i1 = shift_site<D>(i, d1, 1, m.Nt, m.Nx);
      const uint32_t i2 = shift_site<D>(i1, d1, 1, m.Nt, m.Nx);
      for (int d2 = 0; d2 < D; ++d2) {
        if (d2 == d1) continue;
        const uint32_t j = shift_site<D>(i, d2, 1, m.Nt, m.Nx);
        if (d2 > d1) {
          // plaquette(i,d1,d2) (lattice.c:157-164)
          uint32_t g = mul(m, lnk(m, i, d1), lnk(m, i1, d2));
          g = mul(m, g, m.inv[lnk(m, j, d1)]);
          g = mul(m, g, m.inv[lnk(m, i, d2)]);
          atomicAdd(hp + g, 1u);
        }
        // wilson(i,d1,d2,2,1) (dym-mod-metro.cpp:302)
        const uint32_t j1 = shift_site<D>(j, d1, 1, m.Nt, m.Nx);
        uint32_t g = mul(m, lnk(m, i, d1), lnk(m, i1, d1));
        g = mul(m, g, lnk(m, i2, d2));
        g = mul(m, g, m.inv[lnk(m, j1, d1)]);
        g = mul(m, g, m.inv[lnk(m, j, d1)]);
        g = mul(m, g, m.inv[lnk(m, i, d2)]);
        atomicAdd(hr + g, 1u);
      }
    }
    if (x[0] == 0) {  // polyakov(i) (lattice.c:167-175)
      uint32_t r = m.id, s = i;
      for (int t = 0; t < m.Nt; ++t) {
        r = mul(m, r, lnk(m, s, 0));
        s = shift_site<D>(s, 0, 1, m.Nt, m.Nx);
      }
      atomicAdd(hy + r, 1u);
    }
  }
  __syncthreads();
  flush_hist(hp, hist, m.P);
  flush_hist(hr, hist + m.P, m.P);
  flush_hist(hy, hist + 2 * m.P, m.P);
}

// X_k(i, d1) for k < nk, d1 = 1..D-1: xs[((d1-1)*nk + k)*V + i].
template <int D>
__global__ void k_lines_x(MeasArgs m, int nk, uint16_t* xs) {
  const uint32_t n = m.V * (D - 1);
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int d1 = 1 + (int)(t / m.V);
    const uint32_t i = t % m.V;
    uint32_t g = lnk(m, i, d1), s = i;
    xs[((size_t)(d1 - 1) * nk) * m.V + i] = (uint16_t)g;
    for (int k = 1; k < nk; ++k) {
      s = shift_site<D>(s, d1, 1, m.Nt, m.Nx);
      g = mul(m, g, lnk(m, s, d1));
      xs[((size_t)(d1 - 1) * nk + k) * m.V + i] = (uint16_t)g;
    }
  }
}

// T_l(i) for l < nl: ts[l*V + i].
template <int D>
__global__ void k_lines_t(MeasArgs m, int nl, uint16_t* ts) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m.V; i += gridDim.x * blockDim.x) {
    uint32_t g = lnk(m, i, 0), s = i;
    ts[i] = (uint16_t)g;
    for (int l = 1; l < nl; ++l) {
      s = shift_site<D>(s, 0, 1, m.Nt, m.Nx);
      g = mul(m, g, lnk(m, s, 0));
      ts[(size_t)l * m.V + i] = (uint16_t)g;
    }
  }
}

// Histogram of W(k+1, l+1) for one (k, l) per blockIdx.y; (site, d1) items
// strided over blockIdx.x.  xs/ts may be null (walk as written).
template <int D>
__global__ void k_hist_wilson(MeasArgs m, int nk, int nl, const uint16_t* xs, const uint16_t* ts,
                              unsigned long long* hist) {
  extern __shared__ uint32_t sh[];
  const int slot = blockIdx.y;
  const int k = slot / nl, l = slot % nl;
  for (uint32_t t = threadIdx.x; t < m.P; t += blockDim.x) sh[t] = 0;
  __syncthreads();
  const uint32_t n = m.V * (D - 1);
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int d1 = 1 + (int)(t / m.V);
    const uint32_t i = t % m.V;
    int x[D];
    coords<D>(i, m.Nt, m.Nx, x);
    uint32_t g;
    if (xs) {
      int y[D];
#pragma unroll
      for (int c = 0; c < D; ++c) y[c] = x[c];
      y[d1] += k + 1;
      const uint32_t ia = index_of<D>(y, m.Nt, m.Nx);        // i + (k+1) e_d1
      y[d1] -= k + 1;
      y[0] += l + 1;
      const uint32_t ib = index_of<D>(y, m.Nt, m.Nx);        // i + (l+1) e_t
      const size_t xo = ((size_t)(d1 - 1) * nk + k) * m.V;
      g = mul(m, xs[xo + i], ts[(size_t)l * m.V + ia]);
      g = mul(m, g, m.inv[xs[xo + ib]]);
      g = mul(m, g, m.inv[ts[(size_t)l * m.V + i]]);
    } else {  // wilson(i, d1, 0, k+1, l+1) step by step (lattice.c:197-205)
      uint32_t s = i;
      g = m.id;
      for (int j = 0; j <= k; ++j) { g = mul(m, g, lnk(m, s, d1)); s = shift_site<D>(s, d1, 1, m.Nt, m.Nx); }
      for (int j = 0; j <= l; ++j) { g = mul(m, g, lnk(m, s, 0)); s = shift_site<D>(s, 0, 1, m.Nt, m.Nx); }
      for (int j = 0; j <= k; ++j) { s = shift_site<D>(s, d1, -1, m.Nt, m.Nx); g = mul(m, g, m.inv[lnk(m, s, d1)]); }
      for (int j = 0; j <= l; ++j) { s = shift_site<D>(s, 0, -1, m.Nt, m.Nx); g = mul(m, g, m.inv[lnk(m, s, 0)]); }
    }
    atomicAdd(sh + g, 1u);
  }
  __syncthreads();
  flush_hist(sh, hist + (size_t)slot * m.P, m.P);
}

template <int D>
cudaError_t measure_d(const MeasArgs& m, int nk, int nl, bool assoc, unsigned long long* hist, uint16_t* scratch,
                      cudaStream_t s) {
  const unsigned threads = 256;
  size_t smem = (size_t)3 * m.P * 4;
  cudaError_t e;
  if (smem > 48 * 1024) {
    e = cudaFuncSetAttribute(k_hist_local<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  unsigned grid = (unsigned)std::min<uint32_t>((m.V + threads - 1) / threads, 152 * 4);
  k_hist_local<D><<<grid, threads, smem, s>>>(m, hist);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (nk <= 0 || nl <= 0) return cudaSuccess;
  uint16_t* xs = nullptr;
  uint16_t* ts = nullptr;
  if (assoc) {
    xs = scratch;
    ts = scratch + (size_t)(D - 1) * nk * m.V;
    const uint32_t nx = m.V * (D - 1);
    k_lines_x<D><<<std::min<uint32_t>((nx + 255) / 256, 152 * 8), 256, 0, s>>>(m, nk, xs);
    k_lines_t<D><<<std::min<uint32_t>((m.V + 255) / 256, 152 * 8), 256, 0, s>>>(m, nl, ts);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  const uint32_t n = m.V * (D - 1);
  const unsigned gx = std::max<unsigned>(1, std::min<uint32_t>((n + 255) / 256, (152 * 8 + nk * nl - 1) / (nk * nl) + 1));
  dim3 grid2(gx, (unsigned)(nk * nl));
  smem = (size_t)m.P * 4;
  if (smem > 48 * 1024) {
    e = cudaFuncSetAttribute(k_hist_wilson<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  k_hist_wilson<D><<<grid2, 256, smem, s>>>(m, nk, nl, xs, ts, hist + (size_t)3 * m.P);
  return cudaGetLastError();
}

}  // namespace

size_t measure_scratch_elems(const MeasArgs& m, int wl_nx, int wl_nt, bool assoc) {
  if (!assoc || wl_nx <= 0 || wl_nt <= 0) return 0;
  return ((size_t)(m.D - 1) * wl_nx + wl_nt) * m.V;
}

cudaError_t launch_measure(const MeasArgs& m, int wl_nx, int wl_nt, bool assoc, unsigned long long* hist,
                           uint16_t* scratch, cudaStream_t s) {
  switch (m.D) {
    case 2: return measure_d<2>(m, wl_nx, wl_nt, assoc, hist, scratch, s);
    case 3: return measure_d<3>(m, wl_nx, wl_nt, assoc, hist, scratch, s);
    case 4: return measure_d<4>(m, wl_nx, wl_nt, assoc, hist, scratch, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace dym
