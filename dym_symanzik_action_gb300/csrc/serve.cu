// LLR on the host side: per-chain state set-up, the work list that advances
// any set of chains by LLR sweeps, dym_llr_run (a work list of one chain), and
// the request server (continuous batching of LLR windows).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "batch.h"
#include "chain.h"
#include "util.h"

namespace dym {

namespace {

// A value in the fixed point of the LLR energies (times 2^kLlrFixShift, to
// the nearest integer).
long long fix_value(double x) { return std::llrint(std::ldexp(x, kLlrFixShift)); }

double class_sum_host(const long long* h, const std::vector<double>& v, int ncls) {
  double s = 0;
  for (int q = 0; q < ncls; ++q) s = s + (double)h[q] * v[q];
  return s;
}

// Element histograms of all plaquettes and oriented 1x2 rectangles of the
// chain's configuration, folded into ReTr classes (recompute_S1/S2,
// llr.cpp:46-55, 139-151).
int class_histograms(dym_chain* c, long long h[2][kLlrMaxCls]) {
  const Group& g = *c->grp->g;
  dym_meas_opts mo{-1, -1};
  dym_obs o;
  int rc = dym_measure(c, &mo, &o, nullptr);
  if (rc) return rc;
  for (int k = 0; k < 2; ++k)
    for (int q = 0; q < kLlrMaxCls; ++q) h[k][q] = 0;
  for (uint32_t n = 0; n < g.P; ++n) {
    h[0][g.cls[n]] += (long long)c->h_hist[n];
    h[1][g.cls[n]] += (long long)c->h_hist[g.P + n];
  }
  return DYM_OK;
}

int check_llr_group(const Group& g) {
  // The LLR's energies are exact sums of class values (one value per class,
  // that of its lowest-numbered element), so a table whose ReTr varies inside
  // a class by rounding noise is taken as its class values.
  if (g.ncls > kLlrMaxCls || !g.cls_conj_invariant || !g.assoc_ok)
    return fail(DYM_ENOTSUP, "LLR needs an associative group table whose ReTr classes are conjugation-invariant "
                             "(at most 32 classes)");
  return DYM_OK;
}

int check_llr_req(const dym_chain* c, const dym_llr_req* req) {
  if (req->axis != 1 && req->axis != 2) return fail(DYM_EINVAL, "axis must be 1 (S1 window) or 2 (S2 window)");
  if (req->K < 1 || req->NRM < 0 || req->NRM > DYM_LLR_MAX_NRM || req->nhit < 0 || !(req->hw > 0) ||
      req->drive_cap < 0)
    return fail(DYM_EINVAL, "LLR: bad K, NRM, nhit, hw or drive_cap");
  if (req->axis == 2 && (c->p.Nt < 3 || c->p.Nx < 3))
    return fail(DYM_ENOTSUP, "an S2 window needs every extent >= 3 (1x2 rectangles wrap otherwise)");
  if (c->p.pool != DYM_POOL_NEAREST) return fail(DYM_ENOTSUP, "LLR proposals use the nearest-element pool");
  if (c->p.D != 4) return fail(DYM_ENOTSUP, "LLR runs on four-dimensional lattices");
  return check_llr_group(*c->grp->g);
}

// A two-dimensional cell: S2 window and the initial a2 (a1 is req->a0).
struct Llr2dCell {
  double ewin2, hw2, a2;
};

// Allocate (once) and fill the chain's LLR state for window `req` (and, for a
// two-dimensional cell, its S2 window `cell`; req->axis is then 1).
int llr_init_state(dym_chain* c, const dym_llr_req* req, LlrState* st, const Llr2dCell* cell = nullptr) {
  const Group& g = *c->grp->g;
  DYM_CUDA(cudaSetDevice(c->p.device), "cudaSetDevice");
  if (!c->d_llr) {
    DYM_CUDA(dmalloc(&c->d_llr, 1), "cudaMalloc(llr)");
    uint32_t maxlen = 1;
    for (auto l : c->sched.phase_len) maxlen = std::max(maxlen, l);
    const size_t nrec = (maxlen + 31) / 32 * 32;  // whole 32-link tiles
    DYM_CUDA(dmalloc(&c->d_llr_rec, nrec), "cudaMalloc(llr link records)");
    DYM_CUDA(dmalloc(&c->d_llr_blk, nrec), "cudaMalloc(llr block records)");
    DYM_CUDA(dmalloc(&c->d_llr_bref, nrec), "cudaMalloc(llr block flags)");
  }
  std::memset(st, 0, sizeof(LlrState));
  long long h[2][kLlrMaxCls];
  int rc = class_histograms(c, h);
  if (rc) return rc;
  const double W = 2 * req->hw;
  st->a = req->a0;
  st->bg = req->bg;
  st->ewin = req->ewin;
  st->elo = req->ewin - req->hw;
  st->ehi = req->ewin + req->hw;
  st->emid = 0.5 * (st->elo + st->ehi);
  st->w2 = W * W;
  // Fixed-point class values, energies and window bounds (LlrState).
  for (int q = 0; q < g.ncls; ++q) st->vf[q] = fix_value(g.cls_val[q]);
  for (int t = 0; t < 2; ++t) {
    st->Ef[t] = 0;
    for (int q = 0; q < g.ncls; ++q) st->Ef[t] += h[t][q] * st->vf[q];
    st->E[t] = std::ldexp((double)st->Ef[t], -kLlrFixShift);
  }
  st->wlo[0] = fix_value(st->elo);
  st->whi[0] = fix_value(st->ehi);
  st->wmid[0] = fix_value(st->emid);
  st->axis = req->axis;
  st->K = req->K;
  st->NRM = req->NRM;
  st->drive_cap = req->drive_cap;
  st->sweep = c->sweep;
  const long long Ewf = st->Ef[req->axis - 1];
  st->mode = (Ewf >= st->wlo[0] && Ewf <= st->whi[0]) ? DYM_LLR_RM : DYM_LLR_DRIVE;
  st->dims = 1;
  if (cell) {
    st->dims = 2;
    st->bg = cell->a2;
    st->ewin2 = cell->ewin2;
    st->elo2 = cell->ewin2 - cell->hw2;
    st->ehi2 = cell->ewin2 + cell->hw2;
    st->emid2 = 0.5 * (st->elo2 + st->ehi2);
    st->w2b = (2 * cell->hw2) * (2 * cell->hw2);
    st->ihw[0] = 1.0 / req->hw;
    st->ihw[1] = 1.0 / cell->hw2;
    st->wlo[1] = fix_value(st->elo2);
    st->whi[1] = fix_value(st->ehi2);
    st->wmid[1] = fix_value(st->emid2);
    st->wsc[0] = std::ldexp(st->ihw[0], -kLlrFixShift);
    st->wsc[1] = std::ldexp(st->ihw[1], -kLlrFixShift);
    const bool in = st->Ef[0] >= st->wlo[0] && st->Ef[0] <= st->whi[0] && st->Ef[1] >= st->wlo[1] &&
                    st->Ef[1] <= st->whi[1];
    st->mode = in ? DYM_LLR_RM : DYM_LLR_DRIVE;
  }
  {
    const auto mm = std::minmax_element(g.retr.begin(), g.retr.end());
    st->blk = dym_llr_block_links(c->p.D, *mm.second - *mm.first, st->dims, st->axis, req->hw,
                                  cell ? cell->hw2 : 0.0);
  }
  if (req->NRM == 0 && st->mode == DYM_LLR_RM) st->mode = DYM_LLR_DONE;
  if (st->mode == DYM_LLR_DRIVE && req->drive_cap == 0) st->mode = DYM_LLR_UNREACHED;
  DYM_CUDA(copy_sync(c->d_llr, st, sizeof(LlrState), cudaMemcpyHostToDevice, c->stream), "upload llr state");
  return DYM_OK;
}

}  // namespace

// A set of chains advanced together by LLR sweeps: one propose/decide/commit
// triple per colour-phase slot.
struct LlrWork {
  int device = 0, D = 0;
  int sms = 0;
  std::vector<dym_chain*> chains;
  std::vector<Group*> groups;
  std::vector<uint16_t*> d_sub;
  std::vector<uint16_t*> d_cls16;
  std::vector<int32_t*> d_ev;
  BatchGroups bg{};
  size_t smem = 0;
  LlrChainDev* d_chains = nullptr;
  LlrTile* d_tiles = nullptr;
  LlrCommit* d_commits = nullptr;
  std::vector<uint32_t> tile_off, tile_cnt, commit_off, commit_cnt;
  unsigned grid = 1;
  bool dirty = true;
  cudaStream_t stream = nullptr;

  ~LlrWork() { release(); }

  void release_lists() {
    cudaFree(d_chains);
    cudaFree(d_tiles);
    cudaFree(d_commits);
    d_chains = nullptr;
    d_tiles = nullptr;
    d_commits = nullptr;
  }
  void release() {
    release_lists();
    for (auto p : d_sub) cudaFree(p);
    d_sub.clear();
    for (auto p : d_ev) cudaFree(p);
    d_ev.clear();
    groups.clear();
  }

  // Shared tables of a new group.
  int add_group(Group* g) {
    if (std::find(groups.begin(), groups.end(), g) != groups.end()) return DYM_OK;
    if ((int)groups.size() == kBatchMaxGroups) return fail(DYM_ENOTSUP, "at most 4 groups");
    // Packed sub-table sub[k][u] = e | class(e) << 11 with e = u * pool[k]
    // (32-bit entries, class << 16, for groups of order above 2048) and the
    // fixed-point value of every class (the hits' exact sums; LLR runs on
    // four-dimensional lattices only).
    const auto& pool = g->pool_nearest;
    const bool wide = g->P > kMixedMaxP;
    const size_t nent = pool.size() * (size_t)g->P;
    std::vector<uint16_t> sub(nent * (wide ? 2 : 1));
    for (size_t k = 0; k < pool.size(); ++k)
      for (uint32_t u = 0; u < g->P; ++u) {
        const uint32_t e = g->mult[(size_t)u * g->P + pool[k]];
        if (wide) {
          const uint32_t w = e | ((uint32_t)g->cls[e] << 16);
          std::memcpy(&sub[2 * (k * g->P + u)], &w, 4);
        } else {
          sub[k * g->P + u] = (uint16_t)(e | ((uint32_t)g->cls[e] << 11));
        }
      }
    uint16_t* d = nullptr;
    DYM_CUDA(dmalloc(&d, sub.size()), "cudaMalloc(llr sub)");
    DYM_CUDA(copy_sync(d, sub.data(), sub.size() * 2, cudaMemcpyHostToDevice, stream), "upload llr sub");
    d_sub.push_back(d);
    std::vector<int32_t> ev(kLlrMaxCls, 0);
    const int S = fix_shift(*g, 4);
    for (int c = 0; c < g->ncls; ++c) ev[c] = (int32_t)std::llrint(std::ldexp(g->cls_val[c], S));
    int32_t* dv = nullptr;
    DYM_CUDA(dmalloc(&dv, ev.size()), "cudaMalloc(llr values)");
    DYM_CUDA(copy_sync(dv, ev.data(), ev.size() * 4, cudaMemcpyHostToDevice, stream), "upload llr values");
    d_ev.push_back(dv);
    groups.push_back(g);
    // layout
    auto up16 = [](size_t x) { return (x + 15) / 16 * 16; };
    size_t off = 0;
    bg.n = (int)groups.size();
    for (size_t k = 0; k < groups.size(); ++k) {
      const Group& G = *groups[k];
      BatchGroupDev& b = bg.g[k];
      b.mult = (const uint16_t*)G.d_mult;
      b.inv = (const uint16_t*)G.d_inv;
      b.retr = (const double*)G.d_retr;
      b.sub = d_sub[k];
      b.cls16 = (const uint16_t*)G.d_cls16;
      b.ev = d_ev[k];
      b.evshift = fix_shift(G, 4);
      b.wide = G.P > kMixedMaxP ? 1 : 0;
      b.P = G.P;
      b.npool = (uint32_t)G.pool_nearest.size();
      b.off_retr = 0;
      b.off_ev = (uint32_t)off;
      off = up16(off + (size_t)kLlrMaxCls * 4);
      b.off_inv = (uint32_t)off;
      off = up16(off + (size_t)G.P * 2);
      b.off_cls = (uint32_t)off;
      off = up16(off + (size_t)G.P * 2);
      b.off_sub = (uint32_t)off;
      off = up16(off + (size_t)b.npool * G.P * (b.wide ? 4 : 2));
    }
    smem = off;
    int optin = 0;
    DYM_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device), "attribute");
    if (smem > (size_t)optin) return fail(DYM_ENOTSUP, "LLR tables do not fit shared memory");
    dirty = true;
    return DYM_OK;
  }

  int build() {
    release_lists();
    const size_t nc = chains.size();
    if (nc == 0) {
      dirty = false;
      return DYM_OK;
    }
    std::vector<LlrChainDev> cd(nc);
    size_t maxph = 0;
    for (size_t i = 0; i < nc; ++i) {
      dym_chain* c = chains[i];
      LlrChainDev& d = cd[i];
      d.links = c->dev.links;
      d.sites = c->dev.sites;
      d.V = c->dev.V;
      d.Nt = c->p.Nt;
      d.Nx = c->p.Nx;
      d.seed = c->p.seed;
      d.st = c->d_llr;
      d.rec = c->d_llr_rec;
      d.brec = c->d_llr_blk;
      d.bref = c->d_llr_bref;
      d.group = (int)(std::find(groups.begin(), groups.end(), c->grp->g) - groups.begin());
      if (d.group < 0 || d.group >= (int)groups.size() || d.group >= kBatchMaxGroups)
        return fail(DYM_ENOTSUP, "internal: chain's group missing from the work list's group table");
      maxph = std::max(maxph, c->sched.phase_dir.size());
    }
    std::vector<LlrTile> tiles;
    std::vector<LlrCommit> commits;
    tile_off.assign(maxph, 0);
    tile_cnt.assign(maxph, 0);
    commit_off.assign(maxph, 0);
    commit_cnt.assign(maxph, 0);
    const uint32_t T = kLlrTile;  // one warp's tile
    for (size_t k = 0; k < maxph; ++k) {
      tile_off[k] = (uint32_t)tiles.size();
      commit_off[k] = (uint32_t)commits.size();
      for (size_t i = 0; i < nc; ++i) {
        const Schedule& s = chains[i]->sched;
        if (k >= s.phase_dir.size()) continue;
        for (uint32_t j = 0; j < s.phase_len[k]; j += T)
          tiles.push_back(LlrTile{(uint32_t)i, s.phase_off[k] + j, std::min(T, s.phase_len[k] - j),
                                  (uint32_t)s.phase_dir[k], j});
        commits.push_back(LlrCommit{(uint32_t)i, k + 1 == s.phase_dir.size() ? 1u : 0u, s.phase_len[k],
                                    (uint32_t)s.phase_dir[k]});
      }
      tile_cnt[k] = (uint32_t)tiles.size() - tile_off[k];
      commit_cnt[k] = (uint32_t)commits.size() - commit_off[k];
    }
    DYM_CUDA(dmalloc(&d_chains, nc), "cudaMalloc(llr chains)");
    DYM_CUDA(dmalloc(&d_tiles, tiles.size()), "cudaMalloc(llr tiles)");
    DYM_CUDA(dmalloc(&d_commits, commits.size()), "cudaMalloc(llr commits)");
    DYM_CUDA(copy_sync(d_chains, cd.data(), nc * sizeof(LlrChainDev), cudaMemcpyHostToDevice, stream), "upload chains");
    DYM_CUDA(copy_sync(d_tiles, tiles.data(), tiles.size() * sizeof(LlrTile), cudaMemcpyHostToDevice, stream), "tiles");
    DYM_CUDA(copy_sync(d_commits, commits.data(), commits.size() * sizeof(LlrCommit), cudaMemcpyHostToDevice, stream),
             "commits");
    void* fn = llr_propose_kernel_for(D);
    if (!fn) return fail(DYM_ENOTSUP, "LLR: unsupported D");
    DYM_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "smem attribute");
    int per_sm = 0;
    DYM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kLlrWarps * 32, smem), "occupancy");
    grid = (unsigned)std::max(1, sms * std::max(1, per_sm));
    dirty = false;
    return DYM_OK;
  }

  int enqueue_sweeps(int nsweeps, int nhit) {
    if (dirty) {
      int rc = build();
      if (rc) return rc;
    }
    if (chains.empty()) return DYM_OK;
    for (int s = 0; s < nsweeps; ++s)
      for (size_t k = 0; k < tile_cnt.size(); ++k) {
        cudaError_t e = launch_llr_slot(D, d_tiles + tile_off[k], tile_cnt[k], d_commits + commit_off[k],
                                        commit_cnt[k], d_chains, bg, nhit, grid, smem, stream);
        if (e != cudaSuccess) return cuda_fail(e, "llr slot launch");
      }
    return DYM_OK;
  }
};

}  // namespace dym

using namespace dym;

extern "C" {

int dym_llr_energy(dym_chain* c, double* S1, double* S2) {
  if (!c) return fail(DYM_EINVAL, "dym_llr_energy: null chain");
  const Group& g = *c->grp->g;
  int rc = check_llr_group(g);
  if (rc) return rc;
  long long h[2][kLlrMaxCls];
  rc = class_histograms(c, h);
  if (rc) return rc;
  if (S1) *S1 = class_sum_host(h[0], g.cls_val, g.ncls);
  if (S2) *S2 = class_sum_host(h[1], g.cls_val, g.ncls);
  return DYM_OK;
}

}  // extern "C"

namespace dym {
namespace {

// Run the chain's LLR state machine to the end (or max_sweeps); st holds the
// initial state on entry and the final state on return.
int llr_run_state(dym_chain* c, LlrState* st, int nhit, long max_sweeps) {
  LlrWork w;
  w.device = c->p.device;
  w.D = c->p.D;
  w.stream = c->stream;
  DYM_CUDA(cudaDeviceGetAttribute(&w.sms, cudaDevAttrMultiProcessorCount, w.device), "attribute");
  int rc = w.add_group(c->grp->g);
  if (rc) return rc;
  w.chains.push_back(c);
  int mode = st->mode;
  long sweeps = 0;
  while (mode < DYM_LLR_DONE && sweeps < max_sweeps) {
    const int chunk = (int)std::min<long>(8, max_sweeps - sweeps);
    rc = w.enqueue_sweeps(chunk, nhit);
    if (rc) return rc;
    sweeps += chunk;
    DYM_CUDA(cudaMemcpyAsync(&st->mode, &c->d_llr->mode, sizeof(int), cudaMemcpyDeviceToHost, c->stream),
             "read llr mode");
    DYM_CUDA(cudaStreamSynchronize(c->stream), "llr sweeps");
    mode = st->mode;
  }
  DYM_CUDA(copy_sync(st, c->d_llr, sizeof(LlrState), cudaMemcpyDeviceToHost, c->stream), "read llr state");
  c->sweep = st->sweep;  // sweeps after the state machine finished did nothing
  return DYM_OK;
}

}  // namespace
}  // namespace dym

extern "C" {

int dym_llr_run(dym_chain* c, const dym_llr_req* req, dym_llr_result* out, double* a_hist) {
  NvtxRange nvtx("dym_llr_run");
  if (!c || !req || !out) return fail(DYM_EINVAL, "dym_llr_run: null argument");
  int rc = check_llr_req(c, req);
  if (rc) return rc;
  std::unique_ptr<LlrState> st(new LlrState());
  rc = llr_init_state(c, req, st.get());
  if (rc) return rc;
  rc = llr_run_state(c, st.get(), req->nhit, (long)req->drive_cap + (long)req->K * req->NRM + 2);
  if (rc) return rc;
  out->a = st->a;
  out->S1 = st->E[0];
  out->S2 = st->E[1];
  out->status = st->mode;
  out->drive_sweeps = st->drive_sweeps;
  out->sweeps = st->sweeps;
  out->hits = st->hits;
  out->accepts = st->accepts;
  out->phase_accepts = st->phase_acc;
  out->phase_rejects = st->phase_rej;
  if (a_hist)
    for (int m = 0; m < req->NRM; ++m) a_hist[m] = st->a_hist[m];
  return DYM_OK;
}

int dym_llr2d_run(dym_chain* c, const dym_llr2d_req* req, dym_llr2d_result* out, double* a_hist) {
  NvtxRange nvtx("dym_llr2d_run");
  if (!c || !req || !out) return fail(DYM_EINVAL, "dym_llr2d_run: null argument");
  dym_llr_req q{};
  q.axis = 1;
  q.bg = req->a2;
  q.ewin = req->E1;
  q.hw = req->hw1;
  q.a0 = req->a1;
  q.K = req->K;
  q.NRM = req->NRM;
  q.nhit = req->nhit;
  q.drive_cap = req->drive_cap;
  int rc = check_llr_req(c, &q);
  if (rc) return rc;
  if (!(req->hw2 > 0)) return fail(DYM_EINVAL, "dym_llr2d_run: hw2 must be positive");
  if (c->p.Nt < 3 || c->p.Nx < 3)
    return fail(DYM_ENOTSUP, "an S2 window needs every extent >= 3 (1x2 rectangles wrap otherwise)");
  const Llr2dCell cell{req->E2, req->hw2, req->a2};
  std::unique_ptr<LlrState> st(new LlrState());
  rc = llr_init_state(c, &q, st.get(), &cell);
  if (rc) return rc;
  rc = llr_run_state(c, st.get(), req->nhit, (long)req->drive_cap + (long)req->K * req->NRM + 2);
  if (rc) return rc;
  out->a1 = st->a;
  out->a2 = st->bg;
  out->S1 = st->E[0];
  out->S2 = st->E[1];
  out->status = st->mode;
  out->drive_sweeps = st->drive_sweeps;
  out->sweeps = st->sweeps;
  out->hits = st->hits;
  out->accepts = st->accepts;
  out->phase_accepts = st->phase_acc;
  out->phase_rejects = st->phase_rej;
  if (a_hist)
    for (int m = 0; m < req->NRM; ++m) {
      a_hist[2 * m] = st->a_hist[m];
      a_hist[2 * m + 1] = st->a2_hist[m];
    }
  return DYM_OK;
}

}  // extern "C"

// ----------------------------------------------------------------- server --

struct dym_server {
  dym_group* grp = nullptr;
  dym_server_params p{};
  struct Active {
    dym_llr_request req;
    dym_chain* chain;
    uint64_t bytes, links;
  };
  std::deque<dym_llr_request> queue;
  std::vector<Active> active;
  std::map<std::tuple<int, int, int>, std::vector<dym_chain*>> spare;  // finished chains by shape
  std::vector<dym_llr_response> done;
  dym::LlrWork work;
  uint64_t hbm_used = 0;
  uint64_t links_used = 0;
  uint64_t link_hits = 0;
  std::vector<int> h_modes;
};

namespace dym {
namespace {

uint64_t chain_bytes(int D, int Nt, int Nx, uint32_t P) {
  uint64_t V = (uint64_t)Nt;
  for (int d = 1; d < D; ++d) V *= (uint64_t)Nx;
  // links + site lists + link and block records of a phase (at most V links) +
  // LLR state + measurement histograms and pinned copies
  return V * D * 2 + V * D * 4 + (V + 31) / 32 * 32 * (sizeof(LlrLinkRec) + sizeof(LlrBlockRec) + 1) +
         sizeof(LlrState) + 2 * 3ull * P * 8;
}

dym_llr_response rejected(const dym_llr_request& r) {
  dym_llr_response resp{};
  resp.id = r.id;
  resp.status = DYM_LLR_REJECTED;
  resp.NRM = r.NRM;
  return resp;
}

// Response of resident chain i from its device state, with `status` (its own
// mode when finished, DYM_LLR_CANCELLED when withdrawn); the chain goes to the
// spare pool and its budget is returned.  The caller rebuilds the work list.
int retire_one(dym_server* s, size_t i, int status) {
  dym_server::Active& a = s->active[i];
  LlrState st;
  DYM_CUDA(copy_sync(&st, a.chain->d_llr, sizeof(LlrState), cudaMemcpyDeviceToHost, s->work.stream), "read llr state");
  dym_llr_response resp{};
  resp.id = a.req.id;
  resp.a = st.a;
  resp.S1 = st.E[0];
  resp.S2 = st.E[1];
  resp.status = status;
  resp.sweeps = st.sweeps;
  resp.drive_sweeps = st.drive_sweeps;
  resp.NRM = a.req.NRM;
  resp.hits = st.hits;
  resp.accepts = st.accepts;
  for (int m = 0; m < a.req.NRM && m < DYM_SERVE_MAX_NRM; ++m) resp.a_hist[m] = st.a_hist[m];
  s->done.push_back(resp);
  s->link_hits += st.hits;
  s->hbm_used -= a.bytes;
  s->links_used -= a.links;
  s->spare[std::make_tuple(a.req.D, a.req.Nt, a.req.Nx)].push_back(a.chain);
  return DYM_OK;
}

void rebuild_work(dym_server* s) {
  s->work.chains.clear();
  for (auto& a : s->active) s->work.chains.push_back(a.chain);
  s->work.dirty = true;
}

int server_admit(dym_server* s) {
  const Group& g = *s->grp->g;
  while (!s->queue.empty() && (int)s->active.size() < s->p.max_chains) {
    const dym_llr_request r = s->queue.front();
    const uint64_t bytes = chain_bytes(r.D, r.Nt, r.Nx, g.P);
    uint64_t links = (uint64_t)r.D * (uint64_t)r.Nt;
    for (int d = 1; d < r.D; ++d) links *= (uint64_t)r.Nx;
    if (!s->active.empty() && s->hbm_used + bytes > s->p.hbm_budget) break;
    if (!s->active.empty() && s->p.max_links && s->links_used + links > s->p.max_links) break;
    s->queue.pop_front();
    dym_chain* c = nullptr;
    auto key = std::make_tuple(r.D, r.Nt, r.Nx);
    auto it = s->spare.find(key);
    if (it != s->spare.end() && !it->second.empty()) {
      c = it->second.back();
      it->second.pop_back();
      int rc = chain_reset(c, r.seed, r.start);
      if (rc) {
        dym_chain_free(c);
        return rc;
      }
    } else {
      dym_chain_params cp{};
      cp.D = r.D;
      cp.Nt = r.Nt;
      cp.Nx = r.Nx;
      cp.seed = r.seed;
      cp.start = r.start;
      cp.pool = DYM_POOL_NEAREST;
      cp.precision = DYM_PREC_FP64;
      cp.device = s->p.device;
      int rc = dym_chain_create(s->grp, &cp, &c);
      if (rc && !s->active.empty()) {
        // Device memory may free up as resident chains retire: keep the
        // request at the head of the queue and admit nothing more this step.
        s->queue.push_front(r);
        break;
      }
      if (rc) {
        s->done.push_back(rejected(r));
        continue;
      }
    }
    dym_llr_req q{};
    q.axis = r.axis;
    q.bg = r.bg;
    q.ewin = r.ewin;
    q.hw = r.hw;
    q.a0 = r.a0;
    q.K = r.K;
    q.NRM = r.NRM;
    q.nhit = s->p.nhit;
    q.drive_cap = r.drive_cap;
    LlrState st;
    int rc = check_llr_req(c, &q);
    if (!rc) rc = llr_init_state(c, &q, &st);
    if (rc) {  // an invalid window or parameter set: answered, not fatal to the others
      dym_chain_free(c);
      s->done.push_back(rejected(r));
      continue;
    }
    s->active.push_back(dym_server::Active{r, c, bytes, links});
    s->hbm_used += bytes;
    s->links_used += links;
    s->work.chains.push_back(c);
    s->work.dirty = true;
  }
  return DYM_OK;
}

int server_retire(dym_server* s) {
  const size_t n = s->active.size();
  if (n == 0) return DYM_OK;
  s->h_modes.resize(n);
  for (size_t i = 0; i < n; ++i)
    DYM_CUDA(cudaMemcpyAsync(&s->h_modes[i], &s->active[i].chain->d_llr->mode, sizeof(int), cudaMemcpyDeviceToHost,
                             s->work.stream),
             "read modes");
  DYM_CUDA(cudaStreamSynchronize(s->work.stream), "read modes");
  std::vector<dym_server::Active> keep;
  bool changed = false;
  for (size_t i = 0; i < n; ++i) {
    dym_server::Active& a = s->active[i];
    if (s->h_modes[i] < DYM_LLR_DONE) {
      keep.push_back(a);
      continue;
    }
    int rc = retire_one(s, i, s->h_modes[i]);
    if (rc) return rc;
    changed = true;
  }
  if (changed) {
    s->active.swap(keep);
    rebuild_work(s);
  }
  return DYM_OK;
}

}  // namespace
}  // namespace dym

extern "C" {

int dym_server_create(const dym_group* g, const dym_server_params* p, dym_server** out) {
  if (!g || !p || !out) return fail(DYM_EINVAL, "dym_server_create: null argument");
  *out = nullptr;
  if (p->max_chains < 1 || p->nhit < 0) return fail(DYM_EINVAL, "dym_server_create: bad max_chains or nhit");
  int rc = check_llr_group(*g->g);
  if (rc) return rc;
  int ndev = 0;
  DYM_CUDA(cudaGetDeviceCount(&ndev), "cudaGetDeviceCount");
  if (p->device < 0 || p->device >= ndev) return fail(DYM_EINVAL, "bad device ordinal");
  DYM_CUDA(cudaSetDevice(p->device), "cudaSetDevice");
  rc = group_to_device(g->g);
  if (rc) return rc;
  std::unique_ptr<dym_server> s(new dym_server);
  s->grp = const_cast<dym_group*>(g);
  s->p = *p;
  s->work.device = p->device;
  DYM_CUDA(cudaDeviceGetAttribute(&s->work.sms, cudaDevAttrMultiProcessorCount, p->device), "attribute");
  DYM_CUDA(cudaStreamCreateWithFlags(&s->work.stream, cudaStreamNonBlocking), "cudaStreamCreate");
  rc = s->work.add_group(g->g);
  if (rc) return rc;
  *out = s.release();
  return DYM_OK;
}

int dym_server_submit(dym_server* s, const dym_llr_request* r) {
  if (!s || !r) return fail(DYM_EINVAL, "dym_server_submit: null argument");
  if (r->NRM < 0 || r->NRM > DYM_SERVE_MAX_NRM) return fail(DYM_EINVAL, "request NRM out of range");
  if (r->D != 4 || r->Nt < 1 || r->Nx < 1) return fail(DYM_EINVAL, "bad lattice shape (LLR runs on D = 4)");
  if (!s->active.empty() && r->D != s->work.D) return fail(DYM_ENOTSUP, "all requests of a server share D");
  const uint64_t bytes = chain_bytes(r->D, r->Nt, r->Nx, s->grp->g->P);
  if (bytes > s->p.hbm_budget)
    return fail(DYM_ERANGE, "dym_server_submit: the request's chain needs " + std::to_string(bytes) +
                                " bytes, more than the server's budget of " + std::to_string(s->p.hbm_budget));
  if (s->work.D == 0) s->work.D = r->D;
  s->queue.push_back(*r);
  return DYM_OK;
}

int dym_server_cancel(dym_server* s, uint64_t id) {
  if (!s) return fail(DYM_EINVAL, "dym_server_cancel: null server");
  for (auto q = s->queue.begin(); q != s->queue.end(); ++q)
    if (q->id == id) {
      dym_llr_response resp = rejected(*q);
      resp.status = DYM_LLR_CANCELLED;
      s->done.push_back(resp);
      s->queue.erase(q);
      return DYM_OK;
    }
  for (size_t i = 0; i < s->active.size(); ++i)
    if (s->active[i].req.id == id) {
      DYM_CUDA(cudaSetDevice(s->p.device), "cudaSetDevice");
      DYM_CUDA(cudaStreamSynchronize(s->work.stream), "cudaStreamSynchronize");
      int rc = retire_one(s, i, DYM_LLR_CANCELLED);
      if (rc) return rc;
      s->active.erase(s->active.begin() + (std::ptrdiff_t)i);
      rebuild_work(s);
      return DYM_OK;
    }
  return fail(DYM_EINVAL, "dym_server_cancel: no queued or resident request " + std::to_string(id));
}

int dym_server_step(dym_server* s, int32_t nsweeps) {
  NvtxRange nvtx("dym_server_step");
  if (!s || nsweeps < 0) return fail(DYM_EINVAL, "dym_server_step: bad argument");
  DYM_CUDA(cudaSetDevice(s->p.device), "cudaSetDevice");
  int rc = server_admit(s);
  if (rc) return rc;
  if (!s->active.empty()) {
    s->work.D = s->active.front().req.D;
    rc = s->work.enqueue_sweeps(nsweeps, s->p.nhit);
    if (rc) return rc;
  }
  return server_retire(s);
}

int dym_server_poll(dym_server* s, dym_llr_response* out, int32_t max, int32_t* n) {
  if (!s || (!out && max > 0) || !n || max < 0) return fail(DYM_EINVAL, "dym_server_poll: bad argument");
  const int32_t k = (int32_t)std::min<size_t>(s->done.size(), (size_t)max);
  for (int32_t i = 0; i < k; ++i) out[i] = s->done[i];
  s->done.erase(s->done.begin(), s->done.begin() + k);
  *n = k;
  return DYM_OK;
}

int dym_server_status(const dym_server* s, int32_t* active, int32_t* queued, uint64_t* hbm_used,
                      uint64_t* link_hits) {
  if (!s) return fail(DYM_EINVAL, "dym_server_status: null server");
  if (active) *active = (int32_t)s->active.size();
  if (queued) *queued = (int32_t)s->queue.size();
  if (hbm_used) *hbm_used = s->hbm_used;
  if (link_hits) *link_hits = s->link_hits;
  return DYM_OK;
}

int dym_server_free(dym_server* s) {
  if (!s) return DYM_OK;
  cudaSetDevice(s->p.device);
  if (s->work.stream) cudaStreamSynchronize(s->work.stream);
  for (auto& a : s->active) dym_chain_free(a.chain);
  for (auto& kv : s->spare)
    for (auto c : kv.second) dym_chain_free(c);
  s->work.release();
  if (s->work.stream) cudaStreamDestroy(s->work.stream);
  delete s;
  return DYM_OK;
}

}  // extern "C"
