// dym-mod-metro-savecfg: drop-in for the reference executable of the same name
// (dym-mod-metro-savecfg.cpp:218-324): the Metropolis run of dym-mod-metro on
// the GPU, writing the configuration after every K sweeps as SU(3) matrices in
// the Kentucky/NERSC layout the reference writes (savekyconfig, :55-86).
//
//   dym-mod-metro-savecfg group D Nt Nx beta0 beta1 beta2 seed [outprefix] [K] [N] [Ntherm]
//
// Same arguments and defaults (outprefix "./", K = 200, N = 1000, Ntherm = 0,
// NHIT = 20, hot start), the same stdout lines (PARAMS, RUN, "saving configs
// to", GMES with the Polyakov loop and plaquette, ACC, TM_BEGIN/TM_END) and
// the same files: <outprefix>lat-beta1%.3f-beta2%.3f-nt%02d-nx%02d-num%04d,
// V*4*18 big-endian doubles, element (x, y, z, t, part, row, col, dir) at
// x + Nx*(y + Nx*(z + Nx*(t + Nt*(part + 2*(row + 3*(col + 3*dir))))))
// with dir = (d + 3) mod 4, i.e. the spatial directions first.  The matrix of
// every element is read from the group file after the Cayley table (18 doubles
// per element, Re/Im of U[0][0], U[0][1], ..., U[2][2]), as the reference does;
// a file without them is refused.  D must be 4.  Extensions: DYM_NHIT,
// DYM_PRECISION, DYM_DEVICE as for dym-mod-metro.
// There is no CPU fallback: without a working GPU the program exits non-zero.
#include <errno.h>
#include <stdint.h>
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

struct Timer {  // the reference's timer lines (timer.cpp:10-34)
  std::string msg;
  double t0 = 0;
  void start(const char* m) {
    msg = m;
    printf("TM_BEGIN: %-40s ...\n", msg.c_str());
    t0 = now();
  }
  void stop() {
    printf("TM_END:   %-20s %-20s... done in %.3e sec.\n", msg.c_str(), "", now() - t0);
    fflush(stdout);
  }
};

int die(const char* what) {
  fprintf(stderr, "dym-mod-metro-savecfg: %s: %s\n", what, dym_last_error());
  return 1;
}

// The 18 doubles per element appended after the group file's 1 + 2P + P^2 tokens.
bool read_matrices(const char* path, uint32_t P, std::vector<double>* mats) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  std::string text;
  char buf[1 << 16];
  size_t n;
  while ((n = fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, n);
  fclose(f);
  const char* s = text.c_str();
  const char* end = s + text.size();
  auto skip_ws = [&] {
    while (s < end && (*s == ' ' || *s == '\n' || *s == '\t' || *s == '\r')) ++s;
  };
  const uint64_t skip = 1 + 2ull * P + (uint64_t)P * P;
  for (uint64_t k = 0; k < skip; ++k) {
    skip_ws();
    if (s >= end) return false;
    while (s < end && !(*s == ' ' || *s == '\n' || *s == '\t' || *s == '\r')) ++s;
  }
  mats->resize((size_t)P * 18);
  for (size_t k = 0; k < mats->size(); ++k) {
    skip_ws();
    if (s >= end) return false;
    char* e = nullptr;
    errno = 0;
    (*mats)[k] = strtod(s, &e);
    if (e == s || errno) return false;
    s = e;
  }
  return true;
}

void put_be(double v, unsigned char* out) {
  uint64_t b;
  memcpy(&b, &v, 8);
  for (int k = 7; k >= 0; --k, b >>= 8) out[k] = (unsigned char)(b & 0xFF);
}

}  // namespace

int main(int argc, char* argv[]) {
  if (argc < 9) {
    fprintf(stderr, "usage: %s group D Nt Nx beta0 beta1 beta2 seed [outprefix] [K] [N] [Ntherm]\n", argv[0]);
    return 1;
  }
  const char* groupfilename = argv[1];
  const int D = atoi(argv[2]);
  const int Nt = atoi(argv[3]);
  const int Nx = atoi(argv[4]);
  const double beta0 = atof(argv[5]), beta1 = atof(argv[6]), beta2 = atof(argv[7]);
  const int iseed = atoi(argv[8]);
  const char* outprefix = argc >= 10 ? argv[9] : "./";
  const unsigned K = argc > 10 ? (unsigned)atoi(argv[10]) : 200;
  const unsigned N = argc > 11 ? (unsigned)atoi(argv[11]) : 1000;
  const unsigned NTHERM = argc > 12 ? (unsigned)atoi(argv[12]) : 0;
  const int nhit = getenv("DYM_NHIT") ? atoi(getenv("DYM_NHIT")) : 20;
  const char* prec_s = getenv("DYM_PRECISION");
  if (D != 4) {
    fprintf(stderr, "dym-mod-metro-savecfg: the configuration format is four-dimensional (D = 4)\n");
    return 1;
  }
  printf("PARAMS(grp,D,Nt,Nx,beta0,beta1,beta2,seed): %s %d %d %d %e %e %e %d\n", groupfilename, D, Nt, Nx, beta0,
         beta1, beta2, iseed);
  printf("RUN(K,N,Ntherm,NHIT): %u %u %u %d\n", K, N, NTHERM, nhit);
  printf("saving configs to: %s\n", outprefix);

  dym_group* g = nullptr;
  if (dym_group_load(groupfilename, &g) != DYM_OK) return die("cannot load group");
  dym_group_info gi;
  dym_group_get_info(g, &gi);
  std::vector<double> mats;
  if (!read_matrices(groupfilename, gi.order, &mats)) {
    fprintf(stderr, "group file '%s' has no appended SU(3) matrices; cannot save configurations\n", groupfilename);
    return 1;
  }
  printf("read the group\n");
  printf("id: %i\n", (int)gi.identity);
  std::vector<int32_t> mult((size_t)gi.order * gi.order);
  dym_group_get_tables(g, mult.data(), nullptr, nullptr, nullptr, nullptr);
  if (gi.order > 3) {
    auto m = [&](int a, int b) { return mult[(size_t)a * gi.order + b]; };
    printf("check stuff: (a*b)*c: %d a*(b*c): %d\n", m(m(1, 2), 3), m(1, m(2, 3)));
  }
  printf("small group size: %lu\n", (unsigned long)gi.pool_nearest);
  fflush(stdout);

  dym_chain_params p{};
  p.D = D;
  p.Nt = Nt;
  p.Nx = Nx;
  p.beta0 = beta0;
  p.beta1 = beta1;
  p.beta2 = beta2;
  p.seed = (uint64_t)(int64_t)iseed;
  p.start = DYM_START_HOT;
  p.pool = DYM_POOL_NEAREST;
  p.precision = DYM_PREC_MIXED;
  if (prec_s && strcmp(prec_s, "fp64") == 0) p.precision = DYM_PREC_FP64;
  if (prec_s && strcmp(prec_s, "shared") == 0) p.precision = DYM_PREC_SHARED;
  p.device = getenv("DYM_DEVICE") ? atoi(getenv("DYM_DEVICE")) : 0;
  dym_chain* c = nullptr;
  if (dym_chain_create(g, &p, &c) != DYM_OK) return die("cannot create chain");
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
  std::vector<uint16_t> links((size_t)V * D);
  std::vector<unsigned char> out((size_t)V * 4 * 18 * 8);
  dym_meas_opts mo{-1, -1};  // no Wilson grid: the reference prints the Polyakov loop and plaquette only
  for (unsigned n = 0; n < N; n++) {
    Timer tm;
    tm.start("update");
    if (K) {
      if (dym_sweep(c, (int32_t)K, nhit, &st) != DYM_OK) return die("sweep failed");
      hit += st.hits;
      acc += st.accepts;
    }
    tm.stop();
    tm.start("meas");
    dym_obs o;
    if (dym_measure(c, &mo, &o, nullptr) != DYM_OK) return die("measurement failed");
    printf("GMES: %e %e %e %e\n", 999.0, o.poly_re, o.poly_im, o.plaq);
    fflush(stdout);
    printf("ACC: %f\n", ((double)acc) / hit);
    if (dym_links_get(c, links.data()) != DYM_OK) return die("cannot read the configuration");
    for (uint32_t i = 0; i < V; ++i) {
      const uint32_t t = i % (uint32_t)Nt, x = (i / Nt) % Nx, y = (i / Nt / Nx) % Nx, z = i / Nt / Nx / Nx;
      for (int d = 0; d < D; ++d) {
        const double* m = &mats[(size_t)links[(size_t)d * V + i] * 18];
        const int dd = (d + 3) % D;
        for (int part = 0; part < 2; ++part)
          for (int col = 0; col < 3; ++col)
            for (int row = 0; row < 3; ++row) {
              const size_t k = x + (size_t)Nx * (y + (size_t)Nx * (z + (size_t)Nx * (t + (size_t)Nt *
                                                 (part + 2 * (row + 3 * (col + 3 * (size_t)dd))))));
              put_be(m[part + 2 * (col + 3 * row)], &out[k * 8]);
            }
      }
    }
    char name[1024];
    snprintf(name, sizeof(name), "%slat-beta1%.3f-beta2%.3f-nt%02d-nx%02d-num%04d", outprefix, beta1, beta2, Nt, Nx,
             n);
    FILE* f = fopen(name, "wb");
    if (!f || fwrite(out.data(), 1, out.size(), f) != out.size()) {
      fprintf(stderr, "cannot write %s\n", name);
      if (f) fclose(f);
      return 1;
    }
    fclose(f);
    tm.stop();
  }
  dym_chain_free(c);
  dym_group_free(g);
  return 0;
}
