// dym_measure_noalloc: the observables of dym_measure without any memory
// allocation.
//
// dym_measure keeps per-chain histogram buffers (device memory and pinned host
// memory) that it allocates on first use and re-allocates when a larger
// Wilson grid is asked for.  Some callers cannot allow that: a server that has
// given its whole device-memory budget to resident chains, where a new
// cudaMalloc fails or pushes the budget over; and callers that keep other
// streams of the device busy, which cudaMalloc and cudaFree can stall because
// they may synchronise the whole device.  This entry point takes the same
// measurements with no allocation on the success path:
//
//  * the element histograms live in one fixed device array that is part of
//    the library's device image (g_noalloc_scratch below), so it exists as
//    soon as the library's device code is loaded;
//  * Wilson loops are walked link by link (lattice.c:197-205), so no
//    line-product tables, whose size grows with the lattice, are needed;
//  * the FP64 dot products with ReTr/ImTr run on the device in the same order
//    and with the same roundings as dym_measure's host loop, so the results
//    are identical, and only the finished doubles are copied back, straight
//    into the caller's memory.
//
// There is one array per device, shared by every chain on it: calls whose
// device work overlaps (several host threads, or chains on different streams
// of one device) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "chain.h"
#include "dymgpu.h"
#include "engine.h"
#include "util.h"

namespace dym {

namespace {

constexpr size_t kBins = DYM_NOALLOC_HIST_BINS;
constexpr int kMaxLoops = DYM_NOALLOC_MAX_LOOPS;
constexpr int kOut = 4 + kMaxLoops;  // plaquette, rectangle, Polyakov Re/Im, Wilson grid

// Histogram bins [0, kBins) (must be zero when the histogram kernels start;
// every call clears the part it uses), then kOut doubles of results.
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kBins + kOut];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
unsigned long long* g_scratch_ptr[kMaxDevices];  // device address of g_noalloc_scratch, per device

// Looks up the array's address on `device` the first time that device is
// seen; the caller has made `device` current.
int scratch_for(int device, unsigned long long** out) {
  if (device < 0 || device >= kMaxDevices) return fail(DYM_EINVAL, "dym_measure_noalloc: device index out of range");
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "dym_measure_noalloc: cudaGetSymbolAddress");
    g_scratch_ptr[device] = static_cast<unsigned long long*>(p);
  }
  *out = g_scratch_ptr[device];
  return DYM_OK;
}

// Output o: 0 plaquette, 1 rectangle, 2 / 3 Polyakov Re / Im, 4 + j Wilson
// loop j (histogram slot 3 + j).  One thread per output sums the P terms in
// ascending element order, multiply then add, each rounded (as dym_measure's
// host loop, compiled without contraction), then divides by the loop count.
__global__ void k_obs_dot(const unsigned long long* __restrict__ hist, const double* __restrict__ retr,
                          const double* __restrict__ imtr, uint32_t P, int nout, double n_plaq, double n_rect,
                          double n_poly, double n_wl, double* __restrict__ out) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= nout) return;
  const int slot = o < 3 ? o : (o == 3 ? 2 : o - 1);
  const double* w = o == 3 ? imtr : retr;
  const double norm = o == 0 ? n_plaq : o == 1 ? n_rect : o < 4 ? n_poly : n_wl;
  const unsigned long long* h = hist + (size_t)slot * P;
  double s = 0.0;
  for (uint32_t n = 0; n < P; ++n) s = __dadd_rn(s, __dmul_rn((double)h[n], w[n]));
  out[o] = __ddiv_rn(s, norm);
}

}  // namespace

}  // namespace dym

using namespace dym;

extern "C" int dym_measure_noalloc(dym_chain* c, const dym_meas_opts* opts, dym_obs* out, double* wloop) {
  if (!c || !out) return fail(DYM_EINVAL, "dym_measure_noalloc: null argument");
  const Group& g = *c->grp->g;
  int nk = opts && opts->wl_nx > 0 ? opts->wl_nx : c->p.Nx;
  int nl = opts && opts->wl_nt > 0 ? opts->wl_nt : c->p.Nt;
  if (opts && (opts->wl_nx < 0 || opts->wl_nt < 0)) nk = nl = 0;
  const long long loops = (long long)nk * nl;
  if (loops > kMaxLoops)
    return fail(DYM_ERANGE, "dym_measure_noalloc: a " + std::to_string(nk) + "x" + std::to_string(nl) +
                                " Wilson grid has " + std::to_string(loops) + " loops; at most " +
                                std::to_string(kMaxLoops) + " fit the fixed result area");
  const size_t bins = (size_t)(3 + loops) * g.P;
  if (bins > kBins)
    return fail(DYM_ERANGE, "dym_measure_noalloc: " + std::to_string(3 + loops) + " histograms of " +
                                std::to_string(g.P) + " elements need " + std::to_string(bins) +
                                " bins; the fixed scratch holds " + std::to_string(kBins));
  DYM_CUDA(cudaSetDevice(c->p.device), "cudaSetDevice");
  unsigned long long* scratch = nullptr;
  if (int rc = scratch_for(c->p.device, &scratch)) return rc;
  double* res = reinterpret_cast<double*>(scratch + kBins);

  MeasArgs m{c->dev.links, c->dev.V, c->p.D, c->p.Nt, c->p.Nx, (const uint16_t*)g.d_mult,
             (const uint16_t*)g.d_inv, g.P, g.id};
  DYM_CUDA(cudaMemsetAsync(scratch, 0, bins * sizeof(unsigned long long), c->stream), "clear histograms");
  // assoc = false: Wilson loops walked, no line-product scratch.
  DYM_CUDA(launch_measure(m, nk, nl, false, scratch, nullptr, c->stream), "measure launch");
  const uint32_t V = c->dev.V;
  const int D = c->p.D;
  const int nout = 4 + (int)loops;
  k_obs_dot<<<(nout + 127) / 128, 128, 0, c->stream>>>(
      scratch, (const double*)g.d_retr, (const double*)g.d_imtr, g.P, nout, (double)(V * D * (D - 1) / 2),
      (double)(V * D * (D - 1)), (double)(V / c->p.Nt), (double)(V * (D - 1)), res);
  DYM_CUDA(cudaGetLastError(), "observable dot products");
  double head[4];
  DYM_CUDA(cudaMemcpyAsync(head, res, sizeof head, cudaMemcpyDeviceToHost, c->stream), "read observables");
  if (wloop && loops > 0)
    DYM_CUDA(cudaMemcpyAsync(wloop, res + 4, (size_t)loops * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
             "read Wilson loops");
  DYM_CUDA(cudaStreamSynchronize(c->stream), "measure");
  out->plaq = head[0];
  out->rect = head[1];
  out->poly_re = head[2];
  out->poly_im = head[3];
  out->wl_nx = nk;
  out->wl_nt = nl;
  return DYM_OK;
}
