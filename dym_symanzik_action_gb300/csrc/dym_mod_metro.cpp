// dym-mod-metro: drop-in for the reference executable of the same name
// (dym-mod-metro.cpp:199-337), running on the GPU through libdymgpu.
//
//   dym-mod-metro group D Nt Nx beta0 beta1 beta2 seed [K] [N] [Ntherm] [hot|cold] [NHIT]
//
// Same positional arguments, defaults (K = N = 1000, Ntherm = 0, hot start,
// NHIT = 20) and stdout lines (PARAMS, RUN, START, GMES, RMES, ACC, TM_BEGIN,
// TM_END) as the reference.  Extensions, all optional:
//   argv[13] or DYM_NHIT      hits per link (the reference fixes NHIT at compile time)
//   DYM_POOL=nearest|all      proposal pool (default nearest, as the reference)
//   DYM_PRECISION=mixed|shared|fp64  accept arithmetic (default mixed; decisions identical)
//   DYM_WLOOP_MAX=KxL         Wilson grid 1..K by 1..L (default the full Nx x Nt grid)
//   DYM_DEVICE=n              CUDA device
//   DYM_PERF=1                add PERF lines (link-hits/s and sweeps/s per block)
//   DYM_CHECKPOINT=path       resume from `path` when it exists (links, seed, sweeps done;
//                             the command line's couplings then apply, so a checkpoint of
//                             a neighbouring beta is a warm start) and write it at the end
// There is no CPU fallback: without a working GPU the program exits non-zero.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#include <string>
#include <vector>

#include "dymgpu.h"

namespace {

double now() {
  timeval tv;
  gettimeofday(&tv, nullptr);
  return tv.tv_sec + tv.tv_usec * 1e-6;
}

// The reference's timer lines (timer.cpp:10-34).
struct Timer {
  std::string msg;
  double t0 = 0, elapsed = 0;
  void start(const char* m) {
    msg = m;
    printf("TM_BEGIN: %-40s ...\n", msg.c_str());
    t0 = now();
  }
  void stop() {
    elapsed = now() - t0;
    printf("TM_END:   %-20s %-20s... done in %.3e sec.\n", msg.c_str(), "", elapsed);
    fflush(stdout);
  }
};

int die(const char* what) {
  fprintf(stderr, "dym-mod-metro: %s: %s\n", what, dym_last_error());
  return 1;
}

}  // namespace

int main(int argc, char* argv[]) {
  if (argc < 9) {
    fprintf(stderr, "usage: %s group D Nt Nx beta0 beta1 beta2 seed [K] [N] [Ntherm]\n", argv[0]);
    return 1;
  }
  const char* groupfilename = argv[1];
  const int D = atoi(argv[2]);
  const int Nt = atoi(argv[3]);
  const int Nx = atoi(argv[4]);
  const double beta0 = atof(argv[5]);
  const double beta1 = atof(argv[6]);
  const double beta2 = atof(argv[7]);
  const int iseed = atoi(argv[8]);
  const unsigned K = (argc > 9) ? (unsigned)atoi(argv[9]) : 1000;
  const unsigned N = (argc > 10) ? (unsigned)atoi(argv[10]) : 1000;
  const unsigned NTHERM = (argc > 11) ? (unsigned)atoi(argv[11]) : 0;
  const char* startkind = (argc > 12) ? argv[12] : "hot";
  int nhit = 20;
  if (getenv("DYM_NHIT")) nhit = atoi(getenv("DYM_NHIT"));
  if (argc > 13) nhit = atoi(argv[13]);
  const char* pool_s = getenv("DYM_POOL");
  const char* prec_s = getenv("DYM_PRECISION");
  const char* wl_s = getenv("DYM_WLOOP_MAX");
  const bool perf = getenv("DYM_PERF") && atoi(getenv("DYM_PERF"));
  int wl_nx = 0, wl_nt = 0;
  if (wl_s && sscanf(wl_s, "%dx%d", &wl_nx, &wl_nt) != 2) {
    fprintf(stderr, "DYM_WLOOP_MAX must look like 8x8\n");
    return 1;
  }

  printf("PARAMS(grp,D,Nt,Nx,beta0,beta1,beta2,seed): %s %d %d %d %e %e %e %d\n", groupfilename, D, Nt, Nx, beta0,
         beta1, beta2, iseed);
  printf("RUN(K,N,Ntherm,NHIT): %u %u %u %d\n", K, N, NTHERM, nhit);

  dym_group* g = nullptr;
  if (dym_group_load(groupfilename, &g) != DYM_OK) return die("cannot load group");
  dym_group_info gi;
  dym_group_get_info(g, &gi);
  std::vector<int32_t> mult((size_t)gi.order * gi.order);
  dym_group_get_tables(g, mult.data(), nullptr, nullptr, nullptr, nullptr);
  printf("read the group\n");
  fflush(stdout);
  printf("id: %i\n", (int)gi.identity);
  if (gi.order > 3) {
    auto m = [&](int a, int b) { return mult[(size_t)a * gi.order + b]; };
    printf("check stuff: (a*b)*c: %d a*(b*c): %d\n", m(m(1, 2), 3), m(1, m(2, 3)));
  }
  printf("min_retr: %e nn_retr: %e \n", gi.min_retr, gi.nn_retr);
  const bool pool_all = pool_s && strcmp(pool_s, "all") == 0;
  printf("small group size: %lu\n", (unsigned long)gi.pool_nearest);

  const bool coldstart = (startkind[0] == 'c' || startkind[0] == 'C');
  printf("START: %s\n", coldstart ? "cold" : "hot");

  dym_chain_params p;
  memset(&p, 0, sizeof p);
  p.D = D;
  p.Nt = Nt;
  p.Nx = Nx;
  p.beta0 = beta0;
  p.beta1 = beta1;
  p.beta2 = beta2;
  p.seed = (uint64_t)(int64_t)iseed;
  p.start = coldstart ? DYM_START_COLD : DYM_START_HOT;
  p.pool = pool_all ? DYM_POOL_ALL : DYM_POOL_NEAREST;
  p.precision = DYM_PREC_MIXED;
  if (prec_s && strcmp(prec_s, "fp64") == 0) p.precision = DYM_PREC_FP64;
  if (prec_s && strcmp(prec_s, "shared") == 0) p.precision = DYM_PREC_SHARED;
  p.device = getenv("DYM_DEVICE") ? atoi(getenv("DYM_DEVICE")) : 0;
  printf("Initializing nearest neighbours [%d:%d]... \n", Nt, Nx);
  dym_chain* c = nullptr;
  if (dym_chain_create(g, &p, &c) != DYM_OK) return die("cannot create chain");
  const char* ckpt = getenv("DYM_CHECKPOINT");
  if (ckpt && *ckpt) {
    dym_checkpoint_info ci;
    if (FILE* f = fopen(ckpt, "rb")) {
      fclose(f);
      if (dym_checkpoint_read_info(ckpt, &ci) != DYM_OK || dym_chain_checkpoint_load(c, ckpt) != DYM_OK ||
          dym_chain_set_beta(c, beta0, beta1, beta2) != DYM_OK)
        return die("cannot resume from DYM_CHECKPOINT");
      fprintf(stderr, "dym-mod-metro: resumed from %s after %u sweeps\n", ckpt, ci.sweep);
    }
  }
  printf("init done\n");
  fflush(stdout);

  unsigned long long hit = 0, acc = 0;
  dym_stats st;
  if (NTHERM) {
    if (dym_sweep(c, (int32_t)NTHERM, nhit, &st) != DYM_OK) return die("sweep failed");
    hit += st.hits;
    acc += st.accepts;
  }
  printf("thermo done\n");
  fflush(stdout);

  uint32_t V = 0;
  dym_chain_get_schedule(c, &V, nullptr, nullptr, nullptr, nullptr);
  dym_meas_opts mo{wl_nx, wl_nt};
  std::vector<double> wloop((size_t)(wl_nx > 0 ? wl_nx : Nx) * (wl_nt > 0 ? wl_nt : Nt));
  for (unsigned n = 0; n < N; n++) {
    Timer tm;
    tm.start("update");
    if (K) {
      if (dym_sweep(c, (int32_t)K, nhit, &st) != DYM_OK) return die("sweep failed");
      hit += st.hits;
      acc += st.accepts;
    }
    tm.stop();
    if (perf && tm.elapsed > 0)
      printf("PERF: link-hits/s %e sweeps/s %e\n", (double)V * D * nhit * K / tm.elapsed, K / tm.elapsed);

    tm.start("meas");
    dym_obs o;
    if (dym_measure(c, &mo, &o, wloop.data()) != DYM_OK) return die("measurement failed");
    printf("GMES: %e %e %e %e", 999.0, o.poly_re, o.poly_im, o.plaq);
    for (int k = 0; k < o.wl_nx; ++k)
      for (int l = 0; l < o.wl_nt; ++l) printf(" %e", wloop[(size_t)k * o.wl_nt + l]);
    printf("\n");
    printf("RMES: %e %e\n", o.plaq, o.rect);
    fflush(stdout);
    printf("ACC: %f\n", ((double)acc) / hit);
    tm.stop();
  }
  if (ckpt && *ckpt && dym_chain_checkpoint_save(c, ckpt) != DYM_OK) return die("cannot write DYM_CHECKPOINT");
  dym_chain_free(c);
  dym_group_free(g);
  return 0;
}
