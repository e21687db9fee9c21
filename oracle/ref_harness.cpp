// ORACLE (test infrastructure only): a driver around the reference's own
// code, linked with group.c, lattice.c and dym-mod-metro.cpp compiled from
// the reference sources by oracle/build_ref.sh (its main() renamed).  Used only
// by tests/golden/make_golden.py to pin the oracle restatement
// (oracle/dym_oracle.c) and the CUDA engine to the reference.
//
// The staples, plaquettes, rectangles, Polyakov loops and Wilson loops below
// are the reference's functions themselves (get_staples, get_rect_loops,
// plaquette, wilson, getpoly).  The hit loop repeats dym-mod-metro.cpp:161-192
// with two substitutions that the engine under test also makes: links are
// visited in the caller's race-free colour phases, and rand01(rnd[i]) is
// replaced by the Philox stream of dym_core.h.
extern "C" {
#include "group.h"
#include "lattice.h"
extern unsigned int* nn;
}
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "dym_core.h"

void get_staples(unsigned int i, unsigned int d, group_t* st);
void get_rect_loops(unsigned int i, unsigned int d, group_t* st);
extern std::vector<group_t> smallgroup;

static std::string g_loaded;

extern "C" int refh_init(const char* groupfile, int D_, int Nt_, int Nx_) {
  if (g_loaded != groupfile) {
    load_group(groupfile);
    g_loaded = groupfile;
    // proposal pool as in dym-mod-metro.cpp:239-245
    smallgroup.clear();
    double min_retr = 0, nn_retr = 10;
    for (unsigned i = 0; i < P; ++i) if (ReTr[i] < min_retr) min_retr = ReTr[i];
    for (unsigned i = 0; i < P; ++i) if (ReTr[i] > min_retr && ReTr[i] < nn_retr) nn_retr = ReTr[i];
    for (unsigned i = 0; i < P; ++i) if (ReTr[i] < nn_retr + 1e-6 && ReTr[i] > min_retr) smallgroup.push_back(i);
  }
  D = (unsigned)D_;
  Nt = (unsigned)Nt_;
  Nx = (unsigned)Nx_;
  V = Nt;
  for (unsigned d = 1; d < D; ++d) V *= Nx;
  free(a);
  a = (group_t*)malloc(sizeof(group_t) * V * D);
  for (unsigned k = 0; k < V * D; ++k) a[k] = id;
  free(nn);
  nn = NULL;
  step(0, 0, 1);
  return (int)smallgroup.size();
}

extern "C" void refh_set_links(const uint16_t* dm) {
  for (unsigned d = 0; d < D; ++d)
    for (unsigned i = 0; i < V; ++i) a[i * D + d] = dm[(size_t)d * V + i];
}

extern "C" void refh_get_links(uint16_t* dm) {
  for (unsigned d = 0; d < D; ++d)
    for (unsigned i = 0; i < V; ++i) dm[(size_t)d * V + i] = (uint16_t)a[i * D + d];
}

extern "C" void refh_staples(unsigned i, unsigned d, int* st, int* re) {
  get_staples(i, d, st);
  get_rect_loops(i, d, re);
}

extern "C" void refh_sweep(const int* phase_dir, const uint32_t* phase_len, const uint32_t* sites, int nphase,
                           double b0, double b1, double b2, uint64_t seed, uint32_t first_sweep, int nsweeps,
                           int nhit, int pool_all, uint64_t* counters) {
  beta0 = b0;
  beta1 = b1;
  beta2 = b2;
  const int nstaple = 2 * (D - 1);
  const int nrect = 6 * (D - 1);
  for (int s = 0; s < nsweeps; ++s) {
    size_t off = 0;
    for (int p = 0; p < nphase; ++p) {
      const unsigned d = (unsigned)phase_dir[p];
      for (uint32_t k = 0; k < phase_len[p]; ++k) {
        const unsigned i = sites[off + k];
        std::vector<group_t> staples(nstaple), rect(nrect);
        get_staples(i, d, staples.data());
        get_rect_loops(i, d, rect.data());
        group_t b = a[i * D + d];
        double r1 = 0, m1 = 0;
        for (int j = 0; j < nstaple; ++j) r1 += ReTr[mult[b][staples[j]]];
        for (int j = 0; j < nrect; ++j) m1 += ReTr[mult[b][rect[j]]];
        for (int h = 0; h < nhit; ++h) {
          dym_u32x4 r = dym_hit_random(seed, first_sweep + (uint32_t)s, i, d, (uint32_t)h, DYM_TAG_METRO);
          const double u1 = (double)r.v[0] * 0x1p-32;
          group_t g = pool_all ? (group_t)(P * u1) : smallgroup[smallgroup.size() * u1];
          group_t bnew = mult[b][g];
          double r1new = 0, m1new = 0;
          for (int j = 0; j < nstaple; ++j) r1new += ReTr[mult[bnew][staples[j]]];
          for (int j = 0; j < nrect; ++j) m1new += ReTr[mult[bnew][rect[j]]];
          double oldact = beta0 + beta1 * r1 + beta2 * m1;
          double newact = beta0 + beta1 * r1new + beta2 * m1new;
          double probrat = (newact <= oldact) ? 1.0 : dym_exp(-(newact - oldact));
          counters[0]++;
          if (probrat > dym_u53(r.v[1], r.v[2])) {
            a[i * D + d] = bnew;
            b = bnew;
            r1 = r1new;
            m1 = m1new;
            counters[1]++;
          }
        }
      }
      off += phase_len[p];
    }
  }
}

// Observables by the reference's own loop functions and summation order
// (dym-mod-metro.cpp:282-318, single-threaded): out[0..3] = ReP, ImP, plaq,
// rect; out[4 + k*wl_nt + l] = Wilson loop (k+1)x(l+1).
extern "C" void refh_measure(int wl_nx, int wl_nt, double* out) {
  double rep, imp;
  getpoly(&rep, &imp);
  double simpleplaq = 0;
  for (unsigned i = 0; i < V; ++i)
    for (unsigned d1 = 0; d1 < D; ++d1)
      for (unsigned d2 = d1 + 1; d2 < D; ++d2) simpleplaq += ReTr[plaquette(i, d1, d2)];
  simpleplaq /= V * D * (D - 1) / 2;
  double simplerect = 0;
  for (unsigned i = 0; i < V; ++i)
    for (unsigned d1 = 0; d1 < D; ++d1)
      for (unsigned d2 = 0; d2 < D; ++d2)
        if (d1 != d2) simplerect += ReTr[wilson(i, d1, d2, 2, 1)];
  simplerect /= V * D * (D - 1);
  out[0] = rep;
  out[1] = imp;
  out[2] = simpleplaq;
  out[3] = simplerect;
  for (int k = 0; k < wl_nx; ++k)
    for (int l = 0; l < wl_nt; ++l) {
      double lw = 0;
      for (unsigned i = 0; i < V; ++i)
        for (unsigned d1 = 1; d1 < D; ++d1) lw += ReTr[wilson(i, d1, 0, k + 1, l + 1)];
      out[4 + k * wl_nt + l] = lw / (V * (D - 1));
    }
}
