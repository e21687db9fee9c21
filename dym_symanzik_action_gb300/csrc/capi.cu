// C ABI of libdymgpu (declared in include/dymgpu.h): group and chain handles,
// sweeps, observables and configuration transfer.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>

#include "batch.h"
#include "chain.h"
#include "dym_core.h"
#include "util.h"

namespace dym {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int group_to_device(Group* g) {
  int dev = 0;
  DYM_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
  if (g->device == dev) return DYM_OK;
  if (g->device >= 0) return fail(DYM_ENOTSUP, "a group handle is bound to one device; load it again for another");
  const size_t P = g->P;
  DYM_CUDA(dmalloc((uint16_t**)&g->d_mult, P * P), "cudaMalloc(mult)");
  DYM_CUDA(dmalloc((uint16_t**)&g->d_inv, P), "cudaMalloc(inv)");
  DYM_CUDA(dmalloc((double**)&g->d_retr, P), "cudaMalloc(retr)");
  DYM_CUDA(dmalloc((double**)&g->d_imtr, P), "cudaMalloc(imtr)");
  DYM_CUDA(dmalloc((uint8_t**)&g->d_cls, P), "cudaMalloc(cls)");
  DYM_CUDA(dmalloc((uint16_t**)&g->d_cls16, P), "cudaMalloc(cls16)");
  DYM_CUDA(dmalloc((double**)&g->d_clsval, std::max(g->ncls, 1)), "cudaMalloc(clsval)");
  DYM_CUDA(copy_sync(g->d_mult, g->mult.data(), P * P * 2, cudaMemcpyHostToDevice, cudaStreamLegacy), "upload mult");
  DYM_CUDA(copy_sync(g->d_inv, g->inv.data(), P * 2, cudaMemcpyHostToDevice, cudaStreamLegacy), "upload inv");
  DYM_CUDA(copy_sync(g->d_retr, g->retr.data(), P * 8, cudaMemcpyHostToDevice, cudaStreamLegacy), "upload retr");
  DYM_CUDA(copy_sync(g->d_imtr, g->imtr.data(), P * 8, cudaMemcpyHostToDevice, cudaStreamLegacy), "upload imtr");
  DYM_CUDA(copy_sync(g->d_cls, g->cls.data(), P, cudaMemcpyHostToDevice, cudaStreamLegacy), "upload cls");
  {
    std::vector<uint16_t> c16(g->cls.begin(), g->cls.end());
    DYM_CUDA(copy_sync(g->d_cls16, c16.data(), P * 2, cudaMemcpyHostToDevice, cudaStreamLegacy), "upload cls16");
  }
  DYM_CUDA(copy_sync(g->d_clsval, g->cls_val.data(), g->ncls * 8, cudaMemcpyHostToDevice, cudaStreamLegacy), "upload clsval");
  g->device = dev;
  return DYM_OK;
}

void group_free(Group* g) {
  if (!g) return;
  if (g->device >= 0) {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(g->device);
    cudaFree(g->d_mult);
    cudaFree(g->d_inv);
    cudaFree(g->d_retr);
    cudaFree(g->d_imtr);
    cudaFree(g->d_cls);
    cudaFree(g->d_cls16);
    cudaFree(g->d_clsval);
    cudaSetDevice(cur);
  }
  delete g;
}

// Whether the shared-table kernels apply at all: D = 4 and an associative
// table whose ReTr classes (values equal to 1e-9) are unions of conjugacy
// classes, so that ReTr[u_j g] and ReTr[bnew s_j] fall in one class.  The
// D = 2 and D = 3 instantiations of the shared-table kernels faulted on the
// GPU (illegal address / invalid address space) while their source runs
// bit-exact under AddressSanitizer in a host emulation; no cause was found,
// so they are not built and those lattices use the FP64 direct kernel.
static bool shared_structure_ok(const Group& g, int D) { return D == 4 && g.assoc_ok && g.cls_conj_invariant; }

// The FP64 shared sub-table kernel sums ReTr of the conjugates u_j g_k, which
// equal the reference's terms bit for bit only when ReTr is one double per
// class (true of generated tables, not of the reference's shipped files,
// whose traces carry ~1e-16 of rounding noise); its tables must also fit the
// shared-memory opt-in.
static bool sub_eligible(const Group& g, uint32_t npool, int device, int D) {
  if (!shared_structure_ok(g, D) || !g.cls_exact) return false;
  int optin = 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess) return false;
  return sub_smem_bytes(g.P, npool) <= (size_t)optin;
}

static int build_sub_table(dym_chain* c, const std::vector<uint16_t>& pool) {
  const Group& g = *c->grp->g;
  const uint32_t P = g.P, np = (uint32_t)pool.size();
  std::vector<uint16_t> sub((size_t)np * P);
  for (uint32_t k = 0; k < np; ++k)
    for (uint32_t u = 0; u < P; ++u) sub[(size_t)k * P + u] = g.mult[(size_t)u * P + pool[k]];
  DYM_CUDA(dmalloc(&c->dev.sub, sub.size()), "cudaMalloc(sub)");
  DYM_CUDA(copy_sync(c->dev.sub, sub.data(), sub.size() * 2, cudaMemcpyHostToDevice, c->stream), "upload sub");
  c->dev.sub_ok = true;
  return DYM_OK;
}

// The mixed-precision kernel applies on top of the sub-table path when the
// classes fit 5 bits and its shared tables the opt-in limit: with 16-bit
// packed entries (element in 11 bits) for groups of order <= 2048, with 32-bit
// entries above.
static size_t mixed_entry_bytes(const Group& g) { return g.P > kMixedMaxP ? 4 : 2; }

// The mixed kernels take their fast decisions from class values with the
// class spread inside the error bound and re-evaluate the rest on the
// reference's own elements (visit.cuh exact_actions), so they need no
// class-exact table.
static bool mixed_eligible(const Group& g, uint32_t npool, int device, int D) {
  if (!shared_structure_ok(g, D) || g.ncls > kMixedMaxCls || g.ncls < 1) return false;
  int optin = 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess) return false;
  return mixed_smem_bytes(g.P, npool, mixed_entry_bytes(g)) <= (size_t)optin;
}

static int build_mixed_tables(dym_chain* c, const std::vector<uint16_t>& pool) {
  const Group& g = *c->grp->g;
  const uint32_t P = g.P, np = (uint32_t)pool.size();
  const bool wide = mixed_entry_bytes(g) == 4;
  if (wide) {
    std::vector<uint32_t> psub((size_t)np * P);
    for (uint32_t k = 0; k < np; ++k)
      for (uint32_t u = 0; u < P; ++u) {
        const uint32_t e = g.mult[(size_t)u * P + pool[k]];
        psub[(size_t)k * P + u] = e | ((uint32_t)g.cls[e] << 16);
      }
    DYM_CUDA(dmalloc(&c->dev.psub32, psub.size()), "cudaMalloc(psub32)");
    DYM_CUDA(copy_sync(c->dev.psub32, psub.data(), psub.size() * 4, cudaMemcpyHostToDevice, c->stream),
             "upload psub32");
  } else {
    std::vector<uint16_t> psub((size_t)np * P);
    for (uint32_t k = 0; k < np; ++k)
      for (uint32_t u = 0; u < P; ++u) {
        const uint16_t e = g.mult[(size_t)u * P + pool[k]];
        psub[(size_t)k * P + u] = (uint16_t)(e | (g.cls[e] << 11));
      }
    DYM_CUDA(dmalloc(&c->dev.psub, psub.size()), "cudaMalloc(psub)");
    DYM_CUDA(copy_sync(c->dev.psub, psub.data(), psub.size() * 2, cudaMemcpyHostToDevice, c->stream), "upload psub");
  }
  c->dev.mixed_wide = wide;
  const int S = fix_shift(g, c->p.D);
  std::vector<int32_t> cfix(kMixedMaxCls, 0);
  for (int k = 0; k < g.ncls; ++k) cfix[k] = (int32_t)std::llrint(std::ldexp(g.cls_val[k], S));
  DYM_CUDA(dmalloc(&c->dev.cls8, (size_t)P), "cudaMalloc(cls8)");
  DYM_CUDA(dmalloc(&c->dev.cfix, (size_t)kMixedMaxCls), "cudaMalloc(cfix)");
  DYM_CUDA(copy_sync(c->dev.cls8, g.cls.data(), P, cudaMemcpyHostToDevice, c->stream), "upload cls8");
  DYM_CUDA(copy_sync(c->dev.cfix, cfix.data(), kMixedMaxCls * 4, cudaMemcpyHostToDevice, c->stream), "upload cfix");
  // Packed coordinates of every schedule entry (8 bits per axis).
  const Schedule& sc = c->sched;
  std::vector<uint32_t> xyz(sc.sites.size());
  for (size_t k = 0; k < sc.sites.size(); ++k) {
    uint32_t i = sc.sites[k], w = 0;
    for (int b = 0; b < c->p.D; ++b) {
      const uint32_t N = (uint32_t)(b == 0 ? c->p.Nt : c->p.Nx);
      w |= (i % N) << (8 * b);
      i /= N;
    }
    xyz[k] = w;
  }
  DYM_CUDA(dmalloc(&c->dev.xyz, xyz.size()), "cudaMalloc(xyz)");
  DYM_CUDA(copy_sync(c->dev.xyz, xyz.data(), xyz.size() * 4, cudaMemcpyHostToDevice, c->stream), "upload xyz");
  c->dev.fix_shift = S;
  c->dev.mixed_ok = true;
  return DYM_OK;
}

// Value-table kernel tables: int16 fixed-point ReTr of u * g_k and of u, at
// the largest scale 2^S for which |ReTr| 2^S fits int16.  The table is
// element-major (vsub[u * np + k]) and zero-padded to vt_table_bytes.
static int build_vt_tables(dym_chain* c, const std::vector<uint16_t>& pool) {
  const Group& g = *c->grp->g;
  const uint32_t P = g.P, np = (uint32_t)pool.size();
  int S = 14;
  while (S > 0 && std::ldexp(std::max(g.max_abs_retr, 1e-3), S) > 32767.0) --S;
  std::vector<int16_t> vsub(vt_table_bytes(P, np) / 2, 0), val((size_t)P);
  for (uint32_t u = 0; u < P; ++u) val[u] = (int16_t)std::lrint(std::ldexp(g.cls_val[g.cls[u]], S));
  for (uint32_t u = 0; u < P; ++u)
    for (uint32_t k = 0; k < np; ++k) vsub[(size_t)u * np + k] = val[g.mult[(size_t)u * P + pool[k]]];
  DYM_CUDA(dmalloc(&c->dev.vsub, vsub.size()), "cudaMalloc(vsub)");
  DYM_CUDA(dmalloc(&c->dev.val16, (size_t)P), "cudaMalloc(val16)");
  DYM_CUDA(copy_sync(c->dev.vsub, vsub.data(), vsub.size() * 2, cudaMemcpyHostToDevice, c->stream), "upload vsub");
  DYM_CUDA(copy_sync(c->dev.val16, val.data(), P * 2, cudaMemcpyHostToDevice, c->stream), "upload val16");
  c->dev.vt_shift = S;
  c->dev.vt_ok = true;
  return DYM_OK;
}

// Hits per group whose draws the mixed kernels compute ahead (1, 2, 5 or
// 10; for the value-table kernel 2 means speculative pairs, visit.cuh
// vt_hits).  The default is per kernel, the measured faster one:
// value-table 2, element-table 1; DYM_HIT_UNROLL overrides both.
static int hit_unroll_setting(int kernel) {
  const char* e = std::getenv("DYM_HIT_UNROLL");
  const int v = e ? std::atoi(e) : kernel == DYM_KERNEL_MIXED_VALUES ? kDefaultHitUnrollValues : kDefaultHitUnroll;
  return v >= 10 ? 10 : v >= 5 ? 5 : v >= 2 ? 2 : 1;
}

// Threads sharing a link visit in the value-table kernel (DYM_LANES_PER_LINK
// overrides the default): 1 or 2.
static int lanes_per_link_setting() {
  const char* e = std::getenv("DYM_LANES_PER_LINK");
  const int v = e ? std::atoi(e) : kDefaultLanesPerLink;
  return v >= 2 ? 2 : 1;
}

// Largest acceptance of a chain's previous call for which its next call runs
// the value-table kernel (DYM_VT_MAX_ACCEPT overrides the default).
static double vt_max_accept() {
  const char* e = std::getenv("DYM_VT_MAX_ACCEPT");
  return e ? std::atof(e) : kDefaultVtMaxAccept;
}

// The kernel dym_sweep runs for this call (DYM_KERNEL_*).  Both mixed kernels
// take the same decisions; the value-table one is faster while accepted moves
// are rare, since each accepted move fetches its 25 new elements from L2.
static int sweep_kernel(const dym_chain* c) {
  if (c->dev.vt_ok && c->dev.last_acc < vt_max_accept()) return DYM_KERNEL_MIXED_VALUES;
  if (c->dev.mixed_ok) return DYM_KERNEL_MIXED;
  if (c->dev.sub_ok) return DYM_KERNEL_SHARED;
  return DYM_KERNEL_DIRECT;
}

static SweepArgs sweep_args(dym_chain* c, int kernel = DYM_KERNEL_MIXED) {
  const Group& g = *c->grp->g;
  SweepArgs a{};
  a.links = c->dev.links;
  a.V = c->dev.V;
  a.Nt = c->p.Nt;
  a.Nx = c->p.Nx;
  a.mult = (const uint16_t*)g.d_mult;
  a.inv = (const uint16_t*)g.d_inv;
  a.retr = (const double*)g.d_retr;
  a.pool = c->dev.pool;
  a.P = g.P;
  a.npool = c->dev.npool;
  a.id = g.id;
  a.beta0 = c->p.beta0;
  a.beta1 = c->p.beta1;
  a.beta2 = c->p.beta2;
  a.seed = c->p.seed;
  dym_philox_round_keys(c->p.seed, a.rk);
  a.counters = c->dev.counters;
  if (c->dev.mixed_ok) {
    a.cls8 = c->dev.cls8;
    a.cfix = c->dev.cfix;
    a.b1f = (float)c->p.beta1;
    a.b2f = (float)c->p.beta2;
    a.dscale = std::ldexp(1.0f, -c->dev.fix_shift);
    a.dmargin = mixed_margin(g, c->p.D, c->dev.fix_shift, c->p.beta0, c->p.beta1, c->p.beta2);
  }
  if (kernel == DYM_KERNEL_MIXED_VALUES) {
    a.val16 = c->dev.val16;
    a.dscale = std::ldexp(1.0f, -c->dev.vt_shift);
    a.dmargin = mixed_margin(g, c->p.D, c->dev.vt_shift, c->p.beta0, c->p.beta1, c->p.beta2);
  }
#ifdef DYM_BOUNDS_CHECK
  a.status = c->dev.counters + 4;
#endif
  return a;
}

// Persisting-L2 set-aside shared by the chains that pin their group's table
// (dym_chain_set_l2_window): per device, how many windows are open and the
// set-aside in force before the first was opened, restored when the last
// closes.
struct L2SetAside {
  int users = 0;
  size_t prev = 0;
};
static std::mutex g_l2_mu;
static std::map<int, L2SetAside> g_l2;

static int l2_acquire(int device, size_t bytes, size_t* granted) {
  std::lock_guard<std::mutex> lock(g_l2_mu);
  L2SetAside& s = g_l2[device];
  if (s.users == 0) DYM_CUDA(cudaDeviceGetLimit(&s.prev, cudaLimitPersistingL2CacheSize), "cudaDeviceGetLimit");
  size_t cur = 0;
  DYM_CUDA(cudaDeviceGetLimit(&cur, cudaLimitPersistingL2CacheSize), "cudaDeviceGetLimit");
  if (cur < bytes) {
    DYM_CUDA(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, bytes), "cudaDeviceSetLimit(persisting L2)");
    DYM_CUDA(cudaDeviceGetLimit(&cur, cudaLimitPersistingL2CacheSize), "cudaDeviceGetLimit");
  }
  ++s.users;
  *granted = cur;
  return DYM_OK;
}

static void l2_release(int device) {
  std::lock_guard<std::mutex> lock(g_l2_mu);
  auto it = g_l2.find(device);
  if (it == g_l2.end() || it->second.users == 0) return;
  if (--it->second.users == 0) {
    cudaCtxResetPersistingL2Cache();
    cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, it->second.prev);
  }
}

static void chain_release(dym_chain* c) {
  if (!c) return;
  cudaSetDevice(c->p.device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  cudaFree(c->dev.links);
  cudaFree(c->dev.sites);
  cudaFree(c->dev.pool);
  cudaFree(c->dev.counters);
  cudaFree(c->dev.sub);
  cudaFree(c->dev.psub);
  cudaFree(c->dev.psub32);
  cudaFree(c->dev.cls8);
  cudaFree(c->dev.cfix);
  cudaFree(c->dev.xyz);
  cudaFree(c->dev.vsub);
  cudaFree(c->dev.val16);
  cudaFree(c->d_hist);
  cudaFree(c->d_meas_scratch);
  cudaFree(c->d_llr);
  cudaFree(c->d_llr_rec);
  cudaFree(c->d_llr_blk);
  cudaFree(c->d_llr_bref);
  cudaFree(c->d_stage);
  cudaFree(c->d_ref32);
  if (c->h_counters) cudaFreeHost(c->h_counters);
  if (c->h_hist) cudaFreeHost(c->h_hist);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  if (c->l2_window) l2_release(c->p.device);
  delete c;
}

int chain_reset(dym_chain* c, uint64_t seed, int start) {
  if (start != DYM_START_HOT && start != DYM_START_COLD) return fail(DYM_EINVAL, "start must be hot or cold");
  DYM_CUDA(cudaSetDevice(c->p.device), "cudaSetDevice");
  c->p.seed = seed;
  c->p.start = start;
  c->sweep = 0;
  c->dev.last_acc = 1.0;
  const Group& g = *c->grp->g;
  if (start == DYM_START_HOT)
    DYM_CUDA(launch_hot_start(c->dev.links, c->dev.V, c->p.D, g.P, seed, c->stream), "hot start");
  else
    DYM_CUDA(launch_fill(c->dev.links, (size_t)c->dev.V * c->p.D, (uint16_t)g.id, c->stream), "cold start");
  DYM_CUDA(cudaStreamSynchronize(c->stream), "start configuration");
  return DYM_OK;
}

}  // namespace dym

using namespace dym;

extern "C" {

const char* dym_last_error(void) { return g_last_error.c_str(); }
const char* dym_version(void) { return "dymgpu 0.1 (sm_103a)"; }

int dym_group_load(const char* path, dym_group** out) {
  if (!out) return fail(DYM_EINVAL, "dym_group_load: out is NULL");
  *out = nullptr;
  Group* g = nullptr;
  int rc = group_load(path, &g);
  if (rc) return rc;
  *out = new dym_group{g};
  return DYM_OK;
}

int dym_group_free(dym_group* g) {
  if (!g) return DYM_OK;
  group_free(g->g);
  delete g;
  return DYM_OK;
}

int dym_group_get_info(const dym_group* gh, dym_group_info* out) {
  if (!gh || !out) return fail(DYM_EINVAL, "dym_group_get_info: null argument");
  const Group& g = *gh->g;
  out->order = g.P;
  out->identity = g.id;
  out->pool_nearest = (uint32_t)g.pool_nearest.size();
  out->min_retr = g.min_retr;
  out->nn_retr = g.nn_retr;
  out->n_classes = g.ncls;
  out->classes_exact = g.cls_exact ? 1 : 0;
  int dev = 0;
  cudaGetDevice(&dev);
  out->fast_path = 0;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) == cudaSuccess && ndev > 0)
    out->fast_path = mixed_eligible(g, (uint32_t)g.pool_nearest.size(), dev, 4) ? 1 : 0;
  else
    cudaGetLastError();
  out->class_spread = g.cls_spread;
  return DYM_OK;
}

int dym_group_get_tables(const dym_group* gh, int32_t* mult, int32_t* inv, double* retr, double* imtr,
                         int32_t* pool) {
  if (!gh) return fail(DYM_EINVAL, "dym_group_get_tables: null group");
  const Group& g = *gh->g;
  if (mult) for (size_t k = 0; k < g.mult.size(); ++k) mult[k] = g.mult[k];
  if (inv) for (uint32_t k = 0; k < g.P; ++k) inv[k] = g.inv[k];
  if (retr) std::memcpy(retr, g.retr.data(), g.P * 8);
  if (imtr) std::memcpy(imtr, g.imtr.data(), g.P * 8);
  if (pool) for (size_t k = 0; k < g.pool_nearest.size(); ++k) pool[k] = g.pool_nearest[k];
  return DYM_OK;
}

int dym_schedule_check(int32_t D, int32_t Nt, int32_t Nx, int32_t* nphase, uint64_t* conflicts) {
  Schedule s;
  int rc = schedule_build(D, Nt, Nx, &s);
  if (rc) return rc;
  if (nphase) *nphase = (int32_t)s.phase_dir.size();
  if (conflicts) *conflicts = schedule_conflicts(s);
  return DYM_OK;
}

int dym_schedule_get(int32_t D, int32_t Nt, int32_t Nx, uint32_t* V, int32_t* nphase, int32_t* phase_dir,
                     uint32_t* phase_len, uint32_t* sites) {
  Schedule s;
  int rc = schedule_build(D, Nt, Nx, &s);
  if (rc) return rc;
  if (V) *V = s.V;
  if (nphase) *nphase = (int32_t)s.phase_dir.size();
  if (phase_dir) for (size_t p = 0; p < s.phase_dir.size(); ++p) phase_dir[p] = s.phase_dir[p];
  if (phase_len) for (size_t p = 0; p < s.phase_len.size(); ++p) phase_len[p] = s.phase_len[p];
  if (sites) std::memcpy(sites, s.sites.data(), s.sites.size() * 4);
  return DYM_OK;
}

int dym_chain_create(const dym_group* gh, const dym_chain_params* p, dym_chain** out) {
  if (!gh || !p || !out) return fail(DYM_EINVAL, "dym_chain_create: null argument");
  *out = nullptr;
  if (p->start != DYM_START_HOT && p->start != DYM_START_COLD) return fail(DYM_EINVAL, "start must be hot or cold");
  if (p->pool != DYM_POOL_NEAREST && p->pool != DYM_POOL_ALL) return fail(DYM_EINVAL, "unknown proposal pool");
  if (p->precision != DYM_PREC_FP64 && p->precision != DYM_PREC_MIXED && p->precision != DYM_PREC_SHARED)
    return fail(DYM_EINVAL, "unknown precision");
  std::unique_ptr<dym_chain, void (*)(dym_chain*)> c(new dym_chain, chain_release);
  c->grp = const_cast<dym_group*>(gh);
  c->p = *p;
  int rc = schedule_build(p->D, p->Nt, p->Nx, &c->sched);
  if (rc) return rc;
  int ndev = 0;
  DYM_CUDA(cudaGetDeviceCount(&ndev), "cudaGetDeviceCount");
  if (p->device < 0 || p->device >= ndev) return fail(DYM_EINVAL, "bad device ordinal");
  DYM_CUDA(cudaSetDevice(p->device), "cudaSetDevice");
  Group& g = *gh->g;
  rc = group_to_device(&g);
  if (rc) return rc;
  if (g.pool_nearest.empty() && p->pool == DYM_POOL_NEAREST)
    return fail(DYM_EINVAL, "group has an empty nearest-to-identity proposal pool");
  const uint32_t V = c->sched.V;
  ChainDev& d = c->dev;
  d.D = p->D; d.Nt = p->Nt; d.Nx = p->Nx; d.V = V;
  DYM_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate");
  DYM_CUDA(cudaEventCreate(&c->ev0), "cudaEventCreate");
  DYM_CUDA(cudaEventCreate(&c->ev1), "cudaEventCreate");
  DYM_CUDA(dmalloc(&d.links, (size_t)V * p->D), "cudaMalloc(links)");
  DYM_CUDA(dmalloc(&d.sites, c->sched.sites.size()), "cudaMalloc(sites)");
  DYM_CUDA(copy_sync(d.sites, c->sched.sites.data(), c->sched.sites.size() * 4, cudaMemcpyHostToDevice, c->stream),
           "upload sites");
  std::vector<uint16_t> pool;
  if (p->pool == DYM_POOL_NEAREST) pool = g.pool_nearest;
  else for (uint32_t k = 0; k < g.P; ++k) pool.push_back((uint16_t)k);
  d.npool = (uint32_t)pool.size();
  DYM_CUDA(dmalloc(&d.pool, pool.size()), "cudaMalloc(pool)");
  DYM_CUDA(copy_sync(d.pool, pool.data(), pool.size() * 2, cudaMemcpyHostToDevice, c->stream), "upload pool");
  DYM_CUDA(dmalloc(&d.counters, 6), "cudaMalloc(counters)");
  // Pinned copy of the six words (ChainDev::counters).
  DYM_CUDA(cudaHostAlloc((void**)&c->h_counters, 6 * sizeof(unsigned long long), cudaHostAllocMapped),
           "cudaHostAlloc");
  DYM_CUDA(cudaHostGetDevicePointer((void**)&c->h_counters_dev, c->h_counters, 0), "cudaHostGetDevicePointer");
  if (p->precision != DYM_PREC_FP64 && shared_structure_ok(g, p->D)) {
    if (sub_eligible(g, d.npool, p->device, p->D)) {
      rc = build_sub_table(c.get(), pool);
      if (rc) return rc;
    }
    if (p->precision == DYM_PREC_MIXED && mixed_eligible(g, d.npool, p->device, p->D) &&
        p->Nt <= kMixedMaxExtent && p->Nx <= kMixedMaxExtent) {
      rc = build_mixed_tables(c.get(), pool);
      if (rc) return rc;
      int optin = 0;
      DYM_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device), "attribute");
      if (!d.mixed_wide && vt_smem_bytes(g.P, d.npool) <= (size_t)optin) {
        rc = build_vt_tables(c.get(), pool);
        if (rc) return rc;
      }
    }
  }
  if (p->start == DYM_START_HOT)
    DYM_CUDA(launch_hot_start(d.links, V, p->D, g.P, p->seed, c->stream), "hot start");
  else
    DYM_CUDA(launch_fill(d.links, (size_t)V * p->D, (uint16_t)g.id, c->stream), "cold start");
  DYM_CUDA(cudaStreamSynchronize(c->stream), "start configuration");
  *out = c.release();
  return DYM_OK;
}

int dym_chain_free(dym_chain* c) {
  chain_release(c);
  return DYM_OK;
}

int dym_chain_set_l2_window(dym_chain* c, int32_t on) {
  if (!c) return fail(DYM_EINVAL, "dym_chain_set_l2_window: null chain");
  DYM_CUDA(cudaSetDevice(c->p.device), "cudaSetDevice");
  if ((on != 0) == c->l2_window) return DYM_OK;
  cudaStreamAttrValue v{};
  if (on) {
    int max_set_aside = 0, max_window = 0;
    DYM_CUDA(cudaDeviceGetAttribute(&max_set_aside, cudaDevAttrMaxPersistingL2CacheSize, c->p.device), "attribute");
    DYM_CUDA(cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, c->p.device), "attribute");
    if (max_set_aside <= 0 || max_window <= 0) return fail(DYM_ENOTSUP, "device has no persisting L2");
    const Group& g = *c->grp->g;
    const size_t table = (size_t)g.P * g.P * sizeof(uint16_t);
    const size_t window = std::min(table, (size_t)max_window);
    size_t granted = 0;
    int rc = l2_acquire(c->p.device, std::min(window, (size_t)max_set_aside), &granted);
    if (rc) return rc;
    v.accessPolicyWindow.base_ptr = g.d_mult;
    v.accessPolicyWindow.num_bytes = window;
    v.accessPolicyWindow.hitRatio = (float)std::min(1.0, (double)granted / (double)window);
    v.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    v.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    const cudaError_t e = cudaStreamSetAttribute(c->stream, cudaStreamAttributeAccessPolicyWindow, &v);
    if (e != cudaSuccess) {
      l2_release(c->p.device);
      return cuda_fail(e, "cudaStreamSetAttribute(access policy window)");
    }
    c->l2_window = true;
  } else {
    v.accessPolicyWindow.num_bytes = 0;  // no window
    DYM_CUDA(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    DYM_CUDA(cudaStreamSetAttribute(c->stream, cudaStreamAttributeAccessPolicyWindow, &v), "cudaStreamSetAttribute");
    c->l2_window = false;
    l2_release(c->p.device);
  }
  return DYM_OK;
}

int dym_chain_set_beta(dym_chain* c, double beta0, double beta1, double beta2) {
  if (!c) return fail(DYM_EINVAL, "dym_chain_set_beta: null chain");
  c->p.beta0 = beta0;
  c->p.beta1 = beta1;
  c->p.beta2 = beta2;
  return DYM_OK;
}

// Clear the chain's six counter words (sweep counters and upload check) on
// its stream; every call that sweeps or uploads starts with it.
static int counters_reset(dym_chain* c) {
  if (c->counters_dirty)
    DYM_CUDA(cudaMemsetAsync(c->dev.counters, 0, 6 * sizeof(unsigned long long), c->stream), "reset counters");
  c->counters_dirty = true;  // until counters_readback is enqueued
  return DYM_OK;
}

// The end of a call's device work: the six counter words into h_counters and
// cleared on the device (k_counters_out, behind everything the call
// enqueued, since the upload check word may still be read before it).
static int counters_readback(dym_chain* c) {
  DYM_CUDA(launch_counters_out(c->dev.counters, c->h_counters_dev, 6, c->stream), "read counters");
  c->counters_dirty = false;
  return DYM_OK;
}

// Whether the upload check read back into h_counters refused the upload, and
// the smallest bad index if so.
static bool upload_refused(const dym_chain* c, unsigned long long* index) {
  *index = ~c->h_counters[5];
  return c->h_counters[5] != 0;
}

// Enqueue nsweeps sweeps of the chain on its stream, between the events
// ev0 and ev1 (after counters_reset; the caller ends with
// counters_readback); `skip` (see SweepArgs) may make every launch a
// no-op, and the final sweep writes every link into `out` / `out_ref` when
// given (SweepArgs).  Advances c->sweep.
static int sweep_enqueue(dym_chain* c, int32_t nsweeps, int32_t nhit, const unsigned long long* skip,
                         int* kernel_out, uint16_t* out = nullptr, int32_t* out_ref = nullptr) {
  const int kernel = sweep_kernel(c);
  SweepArgs a = sweep_args(c, kernel);
  a.nhit = nhit;
  a.hit_unroll = hit_unroll_setting(kernel);
  a.lanes_per_link = lanes_per_link_setting();
  a.skip = skip;
  const Schedule& s = c->sched;
  DYM_CUDA(cudaEventRecord(c->ev0, c->stream), "cudaEventRecord");
  for (int k = 0; k < nsweeps; ++k) {
    a.sweep = c->sweep;
    if (k == nsweeps - 1) {
      a.out = out;
      a.out_ref = out_ref;
    }
    for (size_t p = 0; p < s.phase_dir.size(); ++p) {
      a.sites = c->dev.sites + s.phase_off[p];
      a.xyz = c->dev.xyz ? c->dev.xyz + s.phase_off[p] : nullptr;
      a.n = s.phase_len[p];
      cudaError_t e;
      switch (kernel) {
        case DYM_KERNEL_MIXED_VALUES: e = launch_sweep_vt(c->p.D, s.phase_dir[p], a, c->dev.vsub, c->stream); break;
        case DYM_KERNEL_MIXED:
          e = c->dev.mixed_wide ? launch_sweep_mixed_wide(c->p.D, s.phase_dir[p], a, c->dev.psub32, c->stream)
                                : launch_sweep_mixed(c->p.D, s.phase_dir[p], a, c->dev.psub, c->stream);
          break;
        case DYM_KERNEL_SHARED: e = launch_sweep_sub(c->p.D, s.phase_dir[p], a, c->dev.sub, c->stream); break;
        default: e = launch_sweep_direct(c->p.D, s.phase_dir[p], a, c->stream);
      }
      if (e != cudaSuccess) return cuda_fail(e, "sweep launch");
    }
    ++c->sweep;
  }
  DYM_CUDA(cudaEventRecord(c->ev1, c->stream), "cudaEventRecord");
  *kernel_out = kernel;
  return DYM_OK;
}

// After the stream has synchronised: the counters of sweep_enqueue into *out.
static int sweep_report(dym_chain* c, int kernel, int32_t nsweeps, dym_stats* out) {
  if (c->h_counters[4])
    return fail(DYM_ECUDA, "bounds check: code " + std::to_string(c->h_counters[4] >> 32) + " value " +
                               std::to_string(c->h_counters[4] & 0xFFFFFFFFull));
  if (c->h_counters[0]) c->dev.last_acc = (double)c->h_counters[1] / (double)c->h_counters[0];
  if (out) {
    out->kernel = kernel;
    out->hits = c->h_counters[0];
    out->accepts = c->h_counters[1];
    out->rechecks = c->h_counters[2];
    float me;  // FP32 bits in the low word of counter 3
    const uint32_t bits = (uint32_t)(c->h_counters[3] & 0xFFFFFFFFull);
    std::memcpy(&me, &bits, 4);
    out->max_ds_err = me;
    out->sweep = c->sweep;
    out->launches = (uint32_t)(nsweeps * c->sched.phase_dir.size());
    float ms = 0;
    DYM_CUDA(cudaEventElapsedTime(&ms, c->ev0, c->ev1), "cudaEventElapsedTime");
    out->device_ms = ms;
  }
  return DYM_OK;
}

int dym_sweep(dym_chain* c, int32_t nsweeps, int32_t nhit, dym_stats* out) {
  NvtxRange nvtx("dym_sweep");
  if (!c) return fail(DYM_EINVAL, "dym_sweep: null chain");
  if (nsweeps < 0 || nhit < 0 || nhit > (1 << 20)) return fail(DYM_EINVAL, "dym_sweep: bad nsweeps or nhit");
  DYM_CUDA(cudaSetDevice(c->p.device), "cudaSetDevice");
  int kernel = 0;
  if (int rc = counters_reset(c)) return rc;
  if (int rc = sweep_enqueue(c, nsweeps, nhit, nullptr, &kernel)) return rc;
  if (int rc = counters_readback(c)) return rc;
  DYM_CUDA(cudaStreamSynchronize(c->stream), "sweep");
  return sweep_report(c, kernel, nsweeps, out);
}

int dym_measure(dym_chain* c, const dym_meas_opts* opts, dym_obs* out, double* wloop) {
  NvtxRange nvtx("dym_measure");
  if (!c || !out) return fail(DYM_EINVAL, "dym_measure: null argument");
  DYM_CUDA(cudaSetDevice(c->p.device), "cudaSetDevice");
  const Group& g = *c->grp->g;
  int nk = opts && opts->wl_nx > 0 ? opts->wl_nx : c->p.Nx;
  int nl = opts && opts->wl_nt > 0 ? opts->wl_nt : c->p.Nt;
  if (opts && (opts->wl_nx < 0 || opts->wl_nt < 0)) nk = nl = 0;
  MeasArgs m{c->dev.links, c->dev.V, c->p.D, c->p.Nt, c->p.Nx, (const uint16_t*)g.d_mult,
             (const uint16_t*)g.d_inv, g.P, g.id};
  const size_t slots = 3 + (size_t)nk * nl;
  const size_t hist_elems = slots * g.P;
  if (hist_elems > c->hist_elems) {
    cudaFree(c->d_hist);
    c->d_hist = nullptr;
    if (c->h_hist) cudaFreeHost(c->h_hist);
    c->h_hist = nullptr;
    DYM_CUDA(dmalloc(&c->d_hist, hist_elems), "cudaMalloc(hist)");
    DYM_CUDA(cudaHostAlloc((void**)&c->h_hist, hist_elems * 8, cudaHostAllocDefault), "cudaHostAlloc(hist)");
    c->hist_elems = hist_elems;
  }
  const size_t scr = measure_scratch_elems(m, nk, nl, g.assoc_ok);
  if (scr > c->meas_scratch_elems) {
    cudaFree(c->d_meas_scratch);
    c->d_meas_scratch = nullptr;
    DYM_CUDA(dmalloc(&c->d_meas_scratch, scr), "cudaMalloc(measure scratch)");
    c->meas_scratch_elems = scr;
  }
  DYM_CUDA(cudaMemsetAsync(c->d_hist, 0, hist_elems * 8, c->stream), "clear hist");
  DYM_CUDA(launch_measure(m, nk, nl, g.assoc_ok, c->d_hist, c->d_meas_scratch, c->stream), "measure launch");
  DYM_CUDA(cudaMemcpyAsync(c->h_hist, c->d_hist, hist_elems * 8, cudaMemcpyDeviceToHost, c->stream), "read hist");
  DYM_CUDA(cudaStreamSynchronize(c->stream), "measure");
  const unsigned long long* h = c->h_hist;
  const uint32_t P = g.P, V = c->dev.V;
  const int D = c->p.D;
  auto dot = [&](const unsigned long long* hh, const std::vector<double>& w) {
    double s = 0;
    for (uint32_t n = 0; n < P; ++n) s += (double)hh[n] * w[n];
    return s;
  };
  out->plaq = dot(h, g.retr) / (double)(V * D * (D - 1) / 2);
  out->rect = dot(h + P, g.retr) / (double)(V * D * (D - 1));
  out->poly_re = dot(h + 2 * P, g.retr) / (double)(V / c->p.Nt);
  out->poly_im = dot(h + 2 * P, g.imtr) / (double)(V / c->p.Nt);
  out->wl_nx = nk;
  out->wl_nt = nl;
  if (wloop)
    for (int k = 0; k < nk; ++k)
      for (int l = 0; l < nl; ++l)
        wloop[k * nl + l] = dot(h + (3 + (size_t)k * nl + l) * P, g.retr) / (double)(V * (D - 1));
  return DYM_OK;
}

// The device address of page-locked host memory (allocated or registered with
// CUDA, hence mapped for the device), or nullptr for any other pointer.
static void* mapped_host(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // clear the error of an unknown pointer
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int dym_links_get(dym_chain* c, uint16_t* host_out) {
  if (!c || !host_out) return fail(DYM_EINVAL, "dym_links_get: null argument");
  DYM_CUDA(cudaSetDevice(c->p.device), "cudaSetDevice");
  const size_t n = (size_t)c->dev.V * c->p.D;
  DYM_CUDA(cudaMemcpyAsync(host_out, c->dev.links, n * 2, cudaMemcpyDeviceToHost, c->stream), "download links");
  DYM_CUDA(cudaStreamSynchronize(c->stream), "download links");
  return DYM_OK;
}

// Enqueue the upload of a configuration from host memory into the chain's
// stage and its check on the device (after counters_reset): the complement
// of the first id >= P into counter word 5, the stage copied into the chain's
// links only if there is none, so a refused configuration leaves the chain as
// it was.
static int links_upload_enqueue(dym_chain* c, const uint16_t* host_in) {
  const uint32_t P = c->grp->g->P;
  const size_t n = (size_t)c->dev.V * c->p.D;
  if (!c->d_stage) DYM_CUDA(dmalloc(&c->d_stage, n), "cudaMalloc(links stage)");
  unsigned long long* check = c->dev.counters + 5;
  if (const void* mh = mapped_host(host_in)) {  // page-locked: read by the checking kernel itself
    DYM_CUDA(launch_links_from_host(c->dev.links, c->d_stage, static_cast<const uint16_t*>(mh), n, P, check,
                                    c->stream),
             "check links");
  } else {
    DYM_CUDA(cudaMemcpyAsync(c->d_stage, host_in, n * 2, cudaMemcpyHostToDevice, c->stream), "upload links");
    DYM_CUDA(launch_links_commit(c->dev.links, c->d_stage, n, P, check, c->stream), "check links");
  }
  return DYM_OK;
}

int dym_links_set(dym_chain* c, const uint16_t* host_in) {
  if (!c || !host_in) return fail(DYM_EINVAL, "dym_links_set: null argument");
  DYM_CUDA(cudaSetDevice(c->p.device), "cudaSetDevice");
  if (int rc = counters_reset(c)) return rc;
  if (int rc = links_upload_enqueue(c, host_in)) return rc;
  if (int rc = counters_readback(c)) return rc;
  DYM_CUDA(cudaStreamSynchronize(c->stream), "upload links");
  unsigned long long bad;
  if (upload_refused(c, &bad))
    return fail(DYM_EINVAL, "dym_links_set: element id out of range at " + std::to_string(bad));
  return DYM_OK;
}

int dym_sweep_host(dym_chain* c, const uint16_t* host_in, uint16_t* host_out, int32_t nsweeps, int32_t nhit,
                   dym_stats* out) {
  NvtxRange nvtx("dym_sweep_host");
  if (!c) return fail(DYM_EINVAL, "dym_sweep_host: null chain");
  if (nsweeps < 0 || nhit < 0 || nhit > (1 << 20)) return fail(DYM_EINVAL, "dym_sweep_host: bad nsweeps or nhit");
  DYM_CUDA(cudaSetDevice(c->p.device), "cudaSetDevice");
  if (int rc = counters_reset(c)) return rc;
  if (host_in)
    if (int rc = links_upload_enqueue(c, host_in)) return rc;
  // A page-locked host_out is written by the final sweep itself; any other
  // (or no sweep) by a copy after the sweeps.
  uint16_t* out_mapped = host_out && nsweeps > 0 ? static_cast<uint16_t*>(mapped_host(host_out)) : nullptr;
  int kernel = 0;
  const uint32_t sweep0 = c->sweep;
  if (int rc = sweep_enqueue(c, nsweeps, nhit, host_in ? c->dev.counters + 5 : nullptr, &kernel, out_mapped))
    return rc;
  const size_t bytes = (size_t)c->dev.V * c->p.D * 2;
  if (host_out && !out_mapped)
    DYM_CUDA(cudaMemcpyAsync(host_out, c->dev.links, bytes, cudaMemcpyDeviceToHost, c->stream), "download links");
  if (int rc = counters_readback(c)) return rc;
  DYM_CUDA(cudaStreamSynchronize(c->stream), "dym_sweep_host");
  unsigned long long bad;
  if (host_in && upload_refused(c, &bad)) {
    c->sweep = sweep0;  // the sweeps did nothing
    if (out_mapped)     // nor wrote host_out: it receives the unchanged configuration
      DYM_CUDA(copy_sync(host_out, c->dev.links, bytes, cudaMemcpyDeviceToHost, c->stream), "download links");
    return fail(DYM_EINVAL, "dym_sweep_host: element id out of range at " + std::to_string(bad));
  }
  return sweep_report(c, kernel, nsweeps, out);
}

int dym_sweep_refarray(dym_chain* c, int32_t* a, int32_t nsweeps, int32_t nhit, dym_stats* out) {
  NvtxRange nvtx("dym_sweep_refarray");
  if (!c || !a) return fail(DYM_EINVAL, "dym_sweep_refarray: null argument");
  if (nsweeps < 0 || nhit < 0 || nhit > (1 << 20)) return fail(DYM_EINVAL, "dym_sweep_refarray: bad nsweeps or nhit");
  DYM_CUDA(cudaSetDevice(c->p.device), "cudaSetDevice");
  const uint32_t P = c->grp->g->P, V = c->dev.V;
  const int D = c->p.D;
  const size_t n = (size_t)V * D;
  if (!c->d_stage) DYM_CUDA(dmalloc(&c->d_stage, n), "cudaMalloc(links stage)");
  // Page-locked arrays are read by the checking kernel and written back by a
  // coalesced pass through their device mapping; any other goes through a
  // device copy of the array, which the final sweep writes.
  int32_t* mapped = static_cast<int32_t*>(mapped_host(a));
  if (!mapped && !c->d_ref32) DYM_CUDA(dmalloc(&c->d_ref32, n), "cudaMalloc(reference-layout array)");
  int32_t* dev_a = mapped ? mapped : c->d_ref32;
  if (int rc = counters_reset(c)) return rc;
  if (!mapped)
    DYM_CUDA(cudaMemcpyAsync(c->d_ref32, a, n * 4, cudaMemcpyHostToDevice, c->stream), "upload reference array");
  DYM_CUDA(launch_links_from_ref(c->dev.links, c->d_stage, dev_a, V, D, P, c->dev.counters + 5, c->stream),
           "check reference array");
  int kernel = 0;
  const uint32_t sweep0 = c->sweep;
  // The array is written after the last sweep (not at all when nsweeps is 0:
  // it then already holds the configuration).
  if (int rc = sweep_enqueue(c, nsweeps, nhit, c->dev.counters + 5, &kernel, nullptr, mapped ? nullptr : dev_a))
    return rc;
  if (mapped && nsweeps > 0)
    DYM_CUDA(launch_links_to_ref(mapped, c->dev.links, V, D, c->dev.counters + 5, c->stream), "write reference array");
  if (int rc = counters_readback(c)) return rc;  // after the write-back, which reads the check word
  DYM_CUDA(cudaStreamSynchronize(c->stream), "dym_sweep_refarray");
  unsigned long long bad;
  if (upload_refused(c, &bad)) {
    c->sweep = sweep0;  // the sweeps did nothing, `a` was not written
    return fail(DYM_EINVAL, "dym_sweep_refarray: element id out of range at a[" + std::to_string(bad) + "]");
  }
  if (!mapped && nsweeps > 0)
    DYM_CUDA(copy_sync(a, c->d_ref32, n * 4, cudaMemcpyDeviceToHost, c->stream), "download reference array");
  return sweep_report(c, kernel, nsweeps, out);
}

static dym_checkpoint_info chain_checkpoint_info(const dym_chain* c) {
  dym_checkpoint_info h{};
  h.D = c->p.D;
  h.Nt = c->p.Nt;
  h.Nx = c->p.Nx;
  h.order = c->grp->g->P;
  h.pool = c->p.pool;
  h.table_hash = table_hash(*c->grp->g);
  h.seed = c->p.seed;
  h.sweep = c->sweep;
  h.beta0 = c->p.beta0;
  h.beta1 = c->p.beta1;
  h.beta2 = c->p.beta2;
  return h;
}

int dym_chain_checkpoint_save(dym_chain* c, const char* path) {
  if (!c || !path) return fail(DYM_EINVAL, "dym_chain_checkpoint_save: null argument");
  std::vector<uint16_t> links((size_t)c->dev.V * c->p.D);
  int rc = dym_links_get(c, links.data());
  if (rc) return rc;
  return checkpoint_write(path, chain_checkpoint_info(c), links.data());
}

int dym_chain_checkpoint_load(dym_chain* c, const char* path) {
  if (!c || !path) return fail(DYM_EINVAL, "dym_chain_checkpoint_load: null argument");
  dym_checkpoint_info h{};
  std::vector<uint16_t> links;
  int rc = checkpoint_read(path, &h, &links);
  if (rc) return rc;
  const dym_checkpoint_info me = chain_checkpoint_info(c);
  if (h.D != me.D || h.Nt != me.Nt || h.Nx != me.Nx)
    return fail(DYM_EINVAL, "dym_chain_checkpoint_load: the checkpoint is of a " + std::to_string(h.D) + "D " +
                                std::to_string(h.Nt) + "x" + std::to_string(h.Nx) + " lattice");
  if (h.order != me.order || h.table_hash != me.table_hash)
    return fail(DYM_EINVAL, "dym_chain_checkpoint_load: the checkpoint is of another group table");
  if (h.pool != me.pool) return fail(DYM_EINVAL, "dym_chain_checkpoint_load: the checkpoint uses another proposal pool");
  rc = dym_links_set(c, links.data());  // ids checked; a refused file leaves the chain as it was
  if (rc) return rc;
  c->p.seed = h.seed;
  c->sweep = h.sweep;
  c->p.beta0 = h.beta0;
  c->p.beta1 = h.beta1;
  c->p.beta2 = h.beta2;
  return DYM_OK;
}

int dym_checkpoint_read_info(const char* path, dym_checkpoint_info* out) {
  if (!path || !out) return fail(DYM_EINVAL, "dym_checkpoint_read_info: null argument");
  return checkpoint_read(path, out, nullptr);
}

int dym_group_table_hash(const dym_group* g, uint64_t* out) {
  if (!g || !out) return fail(DYM_EINVAL, "dym_group_table_hash: null argument");
  *out = table_hash(*g->g);
  return DYM_OK;
}

int dym_chain_get_schedule(const dym_chain* c, uint32_t* V, int32_t* nphase, int32_t* phase_dir,
                           uint32_t* phase_len, uint32_t* sites) {
  if (!c) return fail(DYM_EINVAL, "dym_chain_get_schedule: null chain");
  const Schedule& s = c->sched;
  if (V) *V = s.V;
  if (nphase) *nphase = (int32_t)s.phase_dir.size();
  if (phase_dir) for (size_t p = 0; p < s.phase_dir.size(); ++p) phase_dir[p] = s.phase_dir[p];
  if (phase_len) for (size_t p = 0; p < s.phase_len.size(); ++p) phase_len[p] = s.phase_len[p];
  if (sites) std::memcpy(sites, s.sites.data(), s.sites.size() * 4);
  return DYM_OK;
}

int dym_chain_staples(dym_chain* c, int32_t dir, const uint32_t* sites, int32_t n, uint16_t* out) {
  if (!c || (!sites && n) || (!out && n) || n < 0) return fail(DYM_EINVAL, "dym_chain_staples: bad argument");
  if (dir < 0 || dir >= c->p.D) return fail(DYM_EINVAL, "dym_chain_staples: bad direction");
  for (int32_t k = 0; k < n; ++k)
    if (sites[k] >= c->dev.V) return fail(DYM_EINVAL, "dym_chain_staples: site out of range");
  if (n == 0) return DYM_OK;
  DYM_CUDA(cudaSetDevice(c->p.device), "cudaSetDevice");
  const int ns = 8 * (c->p.D - 1);
  uint32_t* d_sites = nullptr;
  uint16_t* d_out = nullptr;
  DYM_CUDA(dmalloc(&d_sites, n), "cudaMalloc");
  cudaError_t e = dmalloc(&d_out, (size_t)n * ns);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_sites, sites, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = launch_staples(c->p.D, dir, sweep_args(c), d_sites, (uint32_t)n, d_out, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, d_out, (size_t)n * ns * 2, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d_sites);
  cudaFree(d_out);
  if (e != cudaSuccess) return cuda_fail(e, "staples");
  return DYM_OK;
}

int dym_probe_l2_gather(int32_t device, uint32_t table_bytes, double* sectors_per_s) {
  if (!sectors_per_s || table_bytes < 1024) return fail(DYM_EINVAL, "dym_probe_l2_gather: bad argument");
  DYM_CUDA(cudaSetDevice(device), "cudaSetDevice");
  DYM_CUDA(probe_l2_gather(table_bytes, sectors_per_s), "L2 gather probe");
  return DYM_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ batch --

struct dym_batch {
  int device = 0;
  int D = 0;
  std::vector<dym_chain*> chains;
  std::vector<dym::Group*> groups;
  std::vector<uint16_t*> d_group_sub;  // one sub-table per group (owned; packed when mixed)
  std::vector<int32_t*> d_group_cfix;  // fixed-point class values per group (mixed only)
  bool mixed = false;                  // every chain runs the mixed-precision visit
  dym::BatchGroups bg{};
  dym::BatchChainDev* d_chains = nullptr;
  dym::BatchTile* d_tiles = nullptr;
  uint32_t* d_sweeps = nullptr;
  unsigned long long* d_ctr = nullptr;
  std::vector<unsigned long long> h_ctr;
  std::vector<uint32_t> slot_off, slot_cnt;
  size_t smem = 0;
  uint64_t nlinks = 0;
  dym_batch_tuning tune{256, 256, 1, 1, 1};
  bool dirty = true;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_nhit = -1;
  int sms = 0;
};

namespace dym {

static void batch_release_device(dym_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  b->graph_nhit = -1;
  cudaFree(b->d_chains);
  cudaFree(b->d_tiles);
  cudaFree(b->d_sweeps);
  cudaFree(b->d_ctr);
  b->d_chains = nullptr;
  b->d_tiles = nullptr;
  b->d_sweeps = nullptr;
  b->d_ctr = nullptr;
  for (auto p : b->d_group_sub) cudaFree(p);
  b->d_group_sub.clear();
  for (auto p : b->d_group_cfix) cudaFree(p);
  b->d_group_cfix.clear();
}

// Lay out tables, descriptors and per-slot tile lists for the current chains.

// The batched mixed kernel packs 16-bit entries: it takes a chain whose own
// sweep uses the mixed kernel on a group of order <= 2048.
static bool batch_mixed_chain(const dym_chain* c) { return c->dev.mixed_ok && !c->dev.mixed_wide; }

static int batch_build(dym_batch* b) {
  batch_release_device(b);
  const size_t nc = b->chains.size();
  b->bg = BatchGroups{};
  b->bg.n = (int)b->groups.size();
  size_t off = 0;
  auto up16 = [](size_t x) { return (x + 15) / 16 * 16; };
  b->mixed = std::all_of(b->chains.begin(), b->chains.end(), batch_mixed_chain);
  if (!b->mixed && !std::all_of(b->chains.begin(), b->chains.end(), [](const dym_chain* c) { return c->dev.sub_ok; }))
    return fail(DYM_ENOTSUP, "a batch with FP64 shared-table chains cannot hold a chain whose table's ReTr is not "
                             "one double per class (create every chain with the mixed precision)");
  std::vector<int> shift(b->groups.size(), 0);
  for (size_t g = 0; g < b->groups.size(); ++g) {
    const Group& G = *b->groups[g];
    const auto& pool = G.pool_nearest;
    std::vector<uint16_t> sub(pool.size() * (size_t)G.P);
    for (size_t k = 0; k < pool.size(); ++k)
      for (uint32_t u = 0; u < G.P; ++u) {
        const uint16_t e = G.mult[(size_t)u * G.P + pool[k]];
        sub[k * G.P + u] = b->mixed ? (uint16_t)(e | (G.cls[e] << 11)) : e;
      }
    uint16_t* d = nullptr;
    DYM_CUDA(dmalloc(&d, sub.size()), "cudaMalloc(batch sub)");
    b->d_group_sub.push_back(d);
    DYM_CUDA(copy_sync(d, sub.data(), sub.size() * 2, cudaMemcpyHostToDevice, b->stream), "upload batch sub");
    BatchGroupDev& bd = b->bg.g[g];
    bd.mult = (const uint16_t*)G.d_mult;
    bd.inv = (const uint16_t*)G.d_inv;
    bd.retr = (const double*)G.d_retr;
    bd.sub = d;
    bd.P = G.P;
    bd.npool = (uint32_t)pool.size();
    bd.off_retr = (uint32_t)off;
    off = up16(off + (size_t)G.P * 8);
    bd.off_inv = (uint32_t)off;
    off = up16(off + (size_t)G.P * 2);
    bd.off_sub = (uint32_t)off;
    off = up16(off + sub.size() * 2);
    if (b->mixed) {
      shift[g] = fix_shift(G, b->D);
      std::vector<int32_t> cfix(kMixedMaxCls, 0);
      for (int k = 0; k < G.ncls; ++k) cfix[k] = (int32_t)std::llrint(std::ldexp(G.cls_val[k], shift[g]));
      int32_t* dc = nullptr;
      DYM_CUDA(dmalloc(&dc, (size_t)kMixedMaxCls), "cudaMalloc(batch cfix)");
      b->d_group_cfix.push_back(dc);
      DYM_CUDA(copy_sync(dc, cfix.data(), kMixedMaxCls * 4, cudaMemcpyHostToDevice, b->stream), "upload batch cfix");
      bd.cls8 = (const uint8_t*)G.d_cls;
      bd.cfix = dc;
      bd.dscale = std::ldexp(1.0f, -shift[g]);
      bd.off_cls8 = (uint32_t)off;
      off = up16(off + G.P);
      bd.off_cfix = (uint32_t)off;
      off = up16(off + kMixedMaxCls * 4);
    }
  }
  b->smem = off;
  int optin = 0;
  DYM_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device), "attribute");
  if (b->smem > (size_t)optin)
    return fail(DYM_ENOTSUP, "the batch's groups need " + std::to_string(b->smem) + " B of shared tables, more than " +
                                 std::to_string(optin));
  std::vector<BatchChainDev> cd(nc);
  DYM_CUDA(dmalloc(&b->d_ctr, 4 * nc), "cudaMalloc(batch counters)");
  b->nlinks = 0;
  size_t maxph = 0;
  for (size_t i = 0; i < nc; ++i) {
    dym_chain* c = b->chains[i];
    BatchChainDev& d = cd[i];
    d.links = c->dev.links;
    d.sites = c->dev.sites;
    d.V = c->dev.V;
    d.Nt = c->p.Nt;
    d.Nx = c->p.Nx;
    d.group = (int)(std::find(b->groups.begin(), b->groups.end(), c->grp->g) - b->groups.begin());
    if (d.group < 0 || d.group >= b->bg.n) return fail(DYM_ENOTSUP, "internal: chain's group missing from the batch");
    d.beta0 = c->p.beta0;
    d.beta1 = c->p.beta1;
    d.beta2 = c->p.beta2;
    d.seed = c->p.seed;
    d.ctr = b->d_ctr + 4 * i;
    d.xyz = c->dev.xyz;
    if (b->mixed) {
      d.b1f = (float)c->p.beta1;
      d.b2f = (float)c->p.beta2;
      d.dmargin = mixed_margin(*c->grp->g, b->D, shift[d.group], c->p.beta0, c->p.beta1, c->p.beta2);
    }
    b->nlinks += (uint64_t)c->dev.V * c->p.D;
    maxph = std::max(maxph, c->sched.phase_dir.size());
  }
  DYM_CUDA(dmalloc(&b->d_chains, nc), "cudaMalloc(batch chains)");
  DYM_CUDA(copy_sync(b->d_chains, cd.data(), nc * sizeof(BatchChainDev), cudaMemcpyHostToDevice, b->stream), "upload chains");
  DYM_CUDA(dmalloc(&b->d_sweeps, nc), "cudaMalloc(batch sweeps)");
  // Tiles: slot k holds phase k of every chain, split into pieces of `tile`
  // links; larger pieces first so the last blocks of a slot get small ones.
  std::vector<BatchTile> tiles;
  b->slot_off.assign(maxph, 0);
  b->slot_cnt.assign(maxph, 0);
  const uint32_t T = (uint32_t)std::max(32, b->tune.tile);
  for (size_t k = 0; k < maxph; ++k) {
    b->slot_off[k] = (uint32_t)tiles.size();
    std::vector<BatchTile> slot;
    for (size_t i = 0; i < nc; ++i) {
      const Schedule& s = b->chains[i]->sched;
      if (k >= s.phase_dir.size()) continue;
      for (uint32_t j = 0; j < s.phase_len[k]; j += T)
        slot.push_back(BatchTile{(uint32_t)i, s.phase_off[k] + j, std::min(T, s.phase_len[k] - j),
                                 (uint32_t)s.phase_dir[k]});
    }
    std::stable_sort(slot.begin(), slot.end(), [](const BatchTile& x, const BatchTile& y) { return x.count > y.count; });
    tiles.insert(tiles.end(), slot.begin(), slot.end());
    b->slot_cnt[k] = (uint32_t)slot.size();
  }
  DYM_CUDA(dmalloc(&b->d_tiles, std::max<size_t>(tiles.size(), 1)), "cudaMalloc(batch tiles)");
  DYM_CUDA(copy_sync(b->d_tiles, tiles.data(), tiles.size() * sizeof(BatchTile), cudaMemcpyHostToDevice, b->stream),
           "upload tiles");
  if (!batch_kernel_for(b->D, b->mixed, b->tune.hit_unroll)) return fail(DYM_ENOTSUP, "batch: unsupported D");
  b->dirty = false;
  return DYM_OK;
}

static int batch_grid(dym_batch* b, unsigned* grid) {
  int per_sm = 0;
  void* fn = batch_kernel_for(b->D, b->mixed, b->tune.hit_unroll);  // this tuning's instantiation
  if (!fn) return fail(DYM_ENOTSUP, "batch: unsupported D");
  DYM_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem), "smem attribute");
  DYM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, b->tune.threads, b->smem), "occupancy");
  *grid = (unsigned)std::max(1, b->sms * std::max(1, std::min(per_sm, b->tune.grid_per_sm)));
  return DYM_OK;
}

static int batch_enqueue_sweep(dym_batch* b, int nhit, unsigned grid) {
  for (size_t k = 0; k < b->slot_cnt.size(); ++k) {
    cudaError_t e = launch_batch_slot(b->D, b->mixed, b->tune.hit_unroll, b->d_tiles + b->slot_off[k], b->slot_cnt[k],
                                      b->d_chains, b->bg, b->d_sweeps, nhit, std::min<unsigned>(grid, b->slot_cnt[k]),
                                      (unsigned)b->tune.threads, b->smem, b->stream);
    if (e != cudaSuccess) return cuda_fail(e, "batch slot launch");
  }
  DYM_CUDA(launch_batch_advance(b->d_sweeps, (uint32_t)b->chains.size(), b->stream), "batch advance");
  return DYM_OK;
}

}  // namespace dym

extern "C" {

int dym_batch_create(int32_t device, dym_batch** out) {
  if (!out) return fail(DYM_EINVAL, "dym_batch_create: out is NULL");
  *out = nullptr;
  int ndev = 0;
  DYM_CUDA(cudaGetDeviceCount(&ndev), "cudaGetDeviceCount");
  if (device < 0 || device >= ndev) return fail(DYM_EINVAL, "bad device ordinal");
  DYM_CUDA(cudaSetDevice(device), "cudaSetDevice");
  std::unique_ptr<dym_batch> b(new dym_batch);
  b->device = device;
  DYM_CUDA(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, device), "attribute");
  DYM_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate");
  *out = b.release();
  return DYM_OK;
}

int dym_batch_add(dym_batch* b, dym_chain* c) {
  if (!b || !c) return fail(DYM_EINVAL, "dym_batch_add: null argument");
  if (c->p.device != b->device) return fail(DYM_EINVAL, "chain and batch are on different devices");
  if (!b->chains.empty() && c->p.D != b->D) return fail(DYM_EINVAL, "all chains of a batch must have the same D");
  if (!(c->dev.sub_ok || batch_mixed_chain(c)) || c->p.D != 4)
    return fail(DYM_ENOTSUP, "batch chains need D = 4 and the shared-table path (nearest pool, mixed)");
  if (std::find(b->chains.begin(), b->chains.end(), c) != b->chains.end())
    return fail(DYM_EINVAL, "chain already in the batch");
  Group* g = c->grp->g;
  if (std::find(b->groups.begin(), b->groups.end(), g) == b->groups.end()) {
    if ((int)b->groups.size() == kBatchMaxGroups) return fail(DYM_ENOTSUP, "a batch holds at most 4 groups");
    b->groups.push_back(g);
  }
  b->D = c->p.D;
  b->chains.push_back(c);
  b->dirty = true;
  return DYM_OK;
}

int dym_batch_size(const dym_batch* b, int32_t* nchains, uint64_t* nlinks, int32_t* nslots) {
  if (!b) return fail(DYM_EINVAL, "dym_batch_size: null batch");
  uint64_t links = 0;
  size_t maxph = 0;
  for (auto c : b->chains) {
    links += (uint64_t)c->dev.V * c->p.D;
    maxph = std::max(maxph, c->sched.phase_dir.size());
  }
  if (nchains) *nchains = (int32_t)b->chains.size();
  if (nlinks) *nlinks = links;
  if (nslots) *nslots = (int32_t)maxph;
  return DYM_OK;
}

int dym_batch_set_tuning(dym_batch* b, const dym_batch_tuning* t) {
  if (!b || !t) return fail(DYM_EINVAL, "dym_batch_set_tuning: null argument");
  if (t->tile < 32 || t->tile % 32 || (t->threads != 128 && t->threads != 256 && t->threads != 512) ||
      t->grid_per_sm < 1 || (t->hit_unroll != 0 && t->hit_unroll != 1 && t->hit_unroll != 2 && t->hit_unroll != 5 &&
                             t->hit_unroll != 10))
    return fail(DYM_EINVAL,
                "tuning: tile a multiple of 32, threads 128, 256 or 512, grid_per_sm >= 1, hit_unroll 1, 2, 5 or 10");
  if (t->threads == 512 && !b->mixed && !b->chains.empty() &&
      !std::all_of(b->chains.begin(), b->chains.end(), batch_mixed_chain))
    return fail(DYM_EINVAL, "tuning: 512 threads need the mixed-precision batch kernel");
  if (t->tile != b->tune.tile) b->dirty = true;
  b->tune = *t;
  if (b->tune.hit_unroll == 0) b->tune.hit_unroll = 1;
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  if (b->graph) {
    cudaGraphDestroy(b->graph);
    b->graph = nullptr;
  }
  b->graph_nhit = -1;
  return DYM_OK;
}

int dym_batch_get_tuning(const dym_batch* b, dym_batch_tuning* t) {
  if (!b || !t) return fail(DYM_EINVAL, "dym_batch_get_tuning: null argument");
  *t = b->tune;
  return DYM_OK;
}

int dym_batch_sweep(dym_batch* b, int32_t nsweeps, int32_t nhit, dym_stats* total) {
  NvtxRange nvtx("dym_batch_sweep");
  if (!b) return fail(DYM_EINVAL, "dym_batch_sweep: null batch");
  if (nsweeps < 0 || nhit < 0 || nhit > (1 << 20)) return fail(DYM_EINVAL, "dym_batch_sweep: bad nsweeps or nhit");
  DYM_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
  if (b->chains.empty()) return fail(DYM_EINVAL, "empty batch");
  if (b->dirty) {
    int rc = batch_build(b);
    if (rc) return rc;
  }
  const size_t nc = b->chains.size();
  std::vector<uint32_t> sw(nc);
  for (size_t i = 0; i < nc; ++i) sw[i] = b->chains[i]->sweep;
  DYM_CUDA(cudaMemcpyAsync(b->d_sweeps, sw.data(), nc * 4, cudaMemcpyHostToDevice, b->stream), "upload sweeps");
  DYM_CUDA(cudaMemsetAsync(b->d_ctr, 0, 4 * nc * sizeof(unsigned long long), b->stream), "reset counters");
  unsigned grid = 1;
  int grc = batch_grid(b, &grid);
  if (grc) return grc;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  DYM_CUDA(cudaEventCreate(&e0), "cudaEventCreate");
  DYM_CUDA(cudaEventCreate(&e1), "cudaEventCreate");
  if (b->tune.use_graph && (!b->exec || b->graph_nhit != nhit)) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    DYM_CUDA(cudaStreamSynchronize(b->stream), "pre-capture sync");
    DYM_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    int rc = batch_enqueue_sweep(b, nhit, grid);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    DYM_CUDA(ce, "end capture");
    b->graph = g;
    DYM_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0), "graph instantiate");
    b->graph_nhit = nhit;
  }
  DYM_CUDA(cudaEventRecord(e0, b->stream), "cudaEventRecord");
  for (int k = 0; k < nsweeps; ++k) {
    if (b->tune.use_graph) {
      DYM_CUDA(cudaGraphLaunch(b->exec, b->stream), "graph launch");
    } else {
      int rc = batch_enqueue_sweep(b, nhit, grid);
      if (rc) return rc;
    }
  }
  DYM_CUDA(cudaEventRecord(e1, b->stream), "cudaEventRecord");
  b->h_ctr.assign(4 * nc, 0);
  DYM_CUDA(cudaMemcpyAsync(b->h_ctr.data(), b->d_ctr, 4 * nc * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                           b->stream),
           "read counters");
  DYM_CUDA(cudaStreamSynchronize(b->stream), "batch sweep");
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (auto c : b->chains) c->sweep += (uint32_t)nsweeps;
  if (total) {
    std::memset(total, 0, sizeof *total);
    for (size_t i = 0; i < nc; ++i) {
      total->hits += b->h_ctr[4 * i];
      total->accepts += b->h_ctr[4 * i + 1];
      total->rechecks += b->h_ctr[4 * i + 2];
      float me;
      const uint32_t bits = (uint32_t)(b->h_ctr[4 * i + 3] & 0xFFFFFFFFull);
      std::memcpy(&me, &bits, 4);
      total->max_ds_err = std::max(total->max_ds_err, (double)me);
    }
    total->sweep = (uint32_t)nsweeps;
    total->launches = (uint32_t)(nsweeps * (b->slot_cnt.size() + 1));
    total->device_ms = ms;
  }
  return DYM_OK;
}

int dym_batch_chain_counters(const dym_batch* b, int32_t idx, uint64_t* hits, uint64_t* accepts) {
  if (!b || idx < 0 || (size_t)idx >= b->chains.size()) return fail(DYM_EINVAL, "dym_batch_chain_counters: bad index");
  if (b->h_ctr.size() != 4 * b->chains.size()) return fail(DYM_EINVAL, "no batch sweep yet");
  if (hits) *hits = b->h_ctr[4 * idx];
  if (accepts) *accepts = b->h_ctr[4 * idx + 1];
  return DYM_OK;
}

int dym_batch_autotune(dym_batch* b, int32_t nhit, int32_t nsweeps_per_trial, dym_batch_tuning* best) {
  NvtxRange nvtx("dym_batch_autotune");
  if (!b || nsweeps_per_trial < 1) return fail(DYM_EINVAL, "dym_batch_autotune: bad argument");
  if (b->chains.empty()) return fail(DYM_EINVAL, "empty batch");
  DYM_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
  // Save every chain's configuration and sweep counter.
  std::vector<uint16_t*> saved;
  std::vector<uint32_t> sw;
  for (auto c : b->chains) {
    uint16_t* p = nullptr;
    const size_t n = (size_t)c->dev.V * c->p.D;
    DYM_CUDA(dmalloc(&p, n), "cudaMalloc(autotune save)");
    DYM_CUDA(copy_sync(p, c->dev.links, n * 2, cudaMemcpyDeviceToDevice, b->stream), "save links");
    saved.push_back(p);
    sw.push_back(c->sweep);
  }
  const dym_batch_tuning start = b->tune;
  dym_batch_tuning win = start;
  float win_ms = 1e30f;
  int rc = DYM_OK;
  const bool all_mixed =
      std::all_of(b->chains.begin(), b->chains.end(), batch_mixed_chain);
  for (int threads : {128, 256, 512})
    for (int tile : {128, 256, 512, 1024})
      for (int gps : {1, 2})
        for (int hu : {1, 2}) {
          if (rc) break;
          if ((threads == 512 || hu > 1) && !all_mixed) continue;  // the FP64 batch kernel has neither
          dym_batch_tuning t{tile, threads, gps, 1, hu};
          rc = dym_batch_set_tuning(b, &t);
          dym_stats st;
          if (!rc) rc = dym_batch_sweep(b, 1, nhit, &st);  // warm-up, graph capture
          if (!rc) rc = dym_batch_sweep(b, nsweeps_per_trial, nhit, &st);
          if (!rc && st.device_ms < win_ms) {
            win_ms = st.device_ms;
            win = t;
          }
        }
  for (size_t i = 0; i < b->chains.size(); ++i) {
    dym_chain* c = b->chains[i];
    copy_sync(c->dev.links, saved[i], (size_t)c->dev.V * c->p.D * 2, cudaMemcpyDeviceToDevice, b->stream);
    cudaFree(saved[i]);
    c->sweep = sw[i];
  }
  if (rc) {
    dym_batch_set_tuning(b, &start);
    return rc;
  }
  rc = dym_batch_set_tuning(b, &win);
  b->h_ctr.clear();
  if (best) *best = win;
  return rc;
}

int dym_batch_free(dym_batch* b) {
  if (!b) return DYM_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  batch_release_device(b);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return DYM_OK;
}

}  // extern "C"
