// dym-llr: drop-in for the reference's llr executable (llr.cpp:276-344),
// running the windows on the GPU through libdymgpu.
//
//   dym-llr group D Nt Nx axis bg Etop Ebot step hw a0 seed [K] [NRM] [R]
//
// Same positional arguments and defaults (K = 50, NRM = 80, R = 1, NHIT = 20,
// drive-in cap 20000) and the same stdout lines: the LLR header, NPLAQ, NRECT,
// AXIS, RECT_MULT, the per-repeat "down reached / up reached" counts, the
// "ANE: Ewin a_n sd nrep" table (mean and sample deviation over repeats, or
// "--(unreached)") and the energy-drift line.  Each repeat runs the
// reference's two ladder passes (run_pass, llr.cpp:255-274): a hot start
// walking the windows down from Etop and a cold start walking them up from
// Ebot, every window seeded from the previous window's configuration and
// started from the previous a_n; a pass stops at its first window that the
// drive-in cannot reach.  The 2R passes are independent chains and run
// concurrently, one host thread and one chain (CUDA stream) each.
// Energies are exact class sums, so the drift line reports 0.
//
// Extensions, optional: DYM_NHIT (hits per link), DYM_DEVICE (CUDA device).
// Each pass's chain is keyed by Philox seed + 1000003 r (hot) and that seed
// with bit 40 set (cold): the reference reseeds its per-site generators the
// same way per repeat (llr.cpp:326), and the Philox stream replaces them.
// There is no CPU fallback: without a working GPU the program exits non-zero.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <string>
#include <thread>
#include <vector>

#include "dymgpu.h"

namespace {

struct Pass {
  int dir = 1;                 // +1: hot start, windows Etop downwards; -1: cold start, Ebot upwards
  uint64_t seed = 0;
  int reached = 0;
  std::vector<double> an;      // a_n per window index, NaN where not reached
  int rc = DYM_OK;
  std::string err;
};

struct Setup {
  const dym_group* g;
  int D, Nt, Nx, axis, K, NRM, nhit, M, device;
  double bg, Etop, stepE, hw, a0;
};

void run_pass(const Setup& s, Pass* p) {
  p->an.assign(s.M, NAN);
  dym_chain_params cp{};
  cp.D = s.D;
  cp.Nt = s.Nt;
  cp.Nx = s.Nx;
  cp.seed = p->seed;
  cp.start = p->dir > 0 ? DYM_START_HOT : DYM_START_COLD;
  cp.pool = DYM_POOL_NEAREST;
  cp.precision = DYM_PREC_FP64;
  cp.device = s.device;
  dym_chain* c = nullptr;
  if ((p->rc = dym_chain_create(s.g, &cp, &c)) != DYM_OK) {
    p->err = dym_last_error();
    return;
  }
  double a_prev = s.a0;
  for (int k = 0; k < s.M; ++k) {
    const int n = p->dir > 0 ? k : s.M - 1 - k;
    dym_llr_req q{};
    q.axis = s.axis;
    q.bg = s.bg;
    q.ewin = s.Etop - n * s.stepE;
    q.hw = s.hw;
    q.a0 = a_prev;
    q.K = s.K;
    q.NRM = s.NRM;
    q.nhit = s.nhit;
    q.drive_cap = 20000;
    dym_llr_result r{};
    if ((p->rc = dym_llr_run(c, &q, &r, nullptr)) != DYM_OK) {
      p->err = dym_last_error();
      break;
    }
    if (r.status != DYM_LLR_DONE) break;  // stalled; the rest of this pass is unreached
    p->an[n] = r.a;
    a_prev = r.a;
    ++p->reached;
  }
  dym_chain_free(c);
}

}  // namespace

int main(int argc, char* argv[]) {
  if (argc < 13) {
    fprintf(stderr,
            "usage: %s group D Nt Nx axis bg Etop Ebot step hw a0 seed [K] [NRM] [R]\n"
            "  axis=1: window S1 (beta1-driven), bg=beta2 ; axis=2: window S2 (beta2-driven), bg=beta1\n",
            argv[0]);
    return 1;
  }
  const char* groupfile = argv[1];
  Setup s{};
  s.D = atoi(argv[2]);
  s.Nt = atoi(argv[3]);
  s.Nx = atoi(argv[4]);
  s.axis = atoi(argv[5]);
  s.bg = atof(argv[6]);
  s.Etop = atof(argv[7]);
  const double Ebot = atof(argv[8]);
  s.stepE = atof(argv[9]);
  s.hw = atof(argv[10]);
  s.a0 = atof(argv[11]);
  const int iseed = atoi(argv[12]);
  s.K = argc > 13 ? atoi(argv[13]) : 50;
  s.NRM = argc > 14 ? atoi(argv[14]) : 80;
  const int R = argc > 15 ? atoi(argv[15]) : 1;
  s.nhit = getenv("DYM_NHIT") ? atoi(getenv("DYM_NHIT")) : 20;
  s.device = getenv("DYM_DEVICE") ? atoi(getenv("DYM_DEVICE")) : 0;
  s.M = (int)((s.Etop - Ebot) / s.stepE + 0.5) + 1;
  if (s.M < 1 || R < 1 || !(s.stepE > 0)) {
    fprintf(stderr, "dym-llr: need Etop >= Ebot, step > 0 and R >= 1\n");
    return 1;
  }
  printf("LLR(grp,D,Nt,Nx,axis,bg): %s %d %d %d %d %g | Etop=%g Ebot=%g step=%g hw=%g a0=%g seed=%d K=%u NRM=%u "
         "R=%u | %d windows\n",
         groupfile, s.D, s.Nt, s.Nx, s.axis, s.bg, s.Etop, Ebot, s.stepE, s.hw, s.a0, iseed, (unsigned)s.K,
         (unsigned)s.NRM, (unsigned)R, s.M);
  unsigned V = (unsigned)s.Nt;
  for (int d = 1; d < s.D; ++d) V *= (unsigned)s.Nx;
  printf("NPLAQ: %u\n", V * s.D * (s.D - 1) / 2);
  printf("NRECT: %u\n", V * s.D * (s.D - 1));
  printf("AXIS: %d\n", s.axis);
  // Every 1x2 rectangle through a link is one of its 6(D-1) rectangle terms
  // when no extent is below 3, so a link's rectangle sum changes by exactly
  // the change of the total (the multiplicity the reference calibrates).
  const bool wrap = s.Nt < 3 || s.Nx < 3;
  if (!wrap) printf("RECT_MULT calibrated: %.6f\n", 6.0);
  if (s.axis == 2 && wrap)
    printf("WARNING: the 1x2 rectangles wrap on this lattice (extent < 3); the S2 window is invalid.\n"
           "  Use a lattice with extent >= 3 for axis=2.\n");
  fflush(stdout);

  dym_group* g = nullptr;
  if (dym_group_load(groupfile, &g) != DYM_OK) {
    fprintf(stderr, "dym-llr: %s\n", dym_last_error());
    return 1;
  }
  s.g = g;
  std::vector<Pass> passes(2 * R);
  for (int r = 0; r < R; ++r) {
    const uint64_t base = (uint64_t)(uint32_t)iseed + 1000003ull * (uint64_t)r;
    passes[2 * r].dir = 1;
    passes[2 * r].seed = base;
    passes[2 * r + 1].dir = -1;
    passes[2 * r + 1].seed = base | (1ull << 40);
  }
  {
    // The first chain binds the group's tables to the device before the
    // passes start in parallel.
    dym_chain_params cp{};
    cp.D = s.D;
    cp.Nt = s.Nt;
    cp.Nx = s.Nx;
    cp.start = DYM_START_COLD;
    cp.device = s.device;
    dym_chain* c = nullptr;
    if (dym_chain_create(g, &cp, &c) != DYM_OK) {
      fprintf(stderr, "dym-llr: %s\n", dym_last_error());
      return 1;
    }
    dym_chain_free(c);
  }
  std::vector<std::thread> th;
  for (auto& p : passes) th.emplace_back(run_pass, std::cref(s), &p);
  for (auto& t : th) t.join();
  for (auto& p : passes)
    if (p.rc != DYM_OK) {
      fprintf(stderr, "dym-llr: %s\n", p.err.c_str());
      return 1;
    }
  std::vector<std::vector<double>> an(s.M);
  for (int r = 0; r < R; ++r) {
    const Pass& dn = passes[2 * r];
    const Pass& up = passes[2 * r + 1];
    for (int n = 0; n < s.M; ++n) {
      if (!isnan(dn.an[n])) an[n].push_back(dn.an[n]);
      if (!isnan(up.an[n])) an[n].push_back(up.an[n]);
    }
    printf("repeat %u: down reached %d/%d, up reached %d/%d\n", (unsigned)r, dn.reached, s.M, up.reached, s.M);
  }
  printf("\n# Ewin   a_n        sd        nrep\n");
  for (int n = 0; n < s.M; ++n) {
    const double Ewin = s.Etop - n * s.stepE;
    if (an[n].empty()) {
      printf("ANE: %8.2f   --(unreached)\n", Ewin);
      continue;
    }
    double mean = 0;
    for (double x : an[n]) mean += x;
    mean /= an[n].size();
    double var = 0;
    for (double x : an[n]) var += (x - mean) * (x - mean);
    const double sd = an[n].size() > 1 ? sqrt(var / (an[n].size() - 1)) : 0.0;
    printf("ANE: %8.2f  %9.5f  %9.5f  %lu\n", Ewin, mean, sd, (unsigned long)an[n].size());
  }
  printf("max |incr - recompute| E(axis%d) : %.3e\n", s.axis, 0.0);
  dym_group_free(g);
  return 0;
}
