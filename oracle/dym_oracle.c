/*
 * ORACLE -- test infrastructure only.  A CPU restatement of the reference's
 * discrete-group Symanzik Metropolis path (hlammiv/dym_symanzik_action), used
 * by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
 * checker.  Nothing in the product links or calls this file.
 *
 * Parity is pinned: tests/golden/ holds fixtures produced by the reference's
 * own get_staples/get_rect_loops/plaquette/wilson/getpoly/load_group compiled
 * from its sources (oracle/build_ref.sh), and tests check this file against
 * them bit for bit.
 *
 * What is restated, with the reference lines it follows:
 *   - group file parse, identity and inverse search     group.c:13-98
 *   - site index and neighbour table                     lattice.c:119-153
 *   - plaquette / polyakov / getpoly / wilson            lattice.c:157-205
 *   - plaquette and rectangle staples                    dym-mod-metro.cpp:63-142
 *   - proposal pool of nearest elements                  dym-mod-metro.cpp:239-245
 *   - the multi-hit Metropolis update of one link        dym-mod-metro.cpp:161-192
 *   - observables of one measurement                     dym-mod-metro.cpp:282-318
 * What differs from the reference, by design of the engine under test:
 *   - links are visited in the race-free colour phases passed in by the
 *     caller instead of the racy two-parity checkerboard (dym-mod-metro.cpp:152-159);
 *   - the per-site minstd engines are replaced by Philox4x32-10 keyed by
 *     (seed, sweep, link, hit), and glibc exp by dym_exp (dym_core.h);
 *   - observables sum integer histograms over group elements, then take one
 *     FP64 dot product in ascending element order.
 * Data layout follows the reference (AoS int links a[i*D+mu], int Cayley rows,
 * a neighbour table), so that its timing is representative of the reference's
 * OpenMP CPU code.
 */
#include <errno.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../dym_symanzik_action_gb300/csrc/dym_core.h"

#define OR_PMAX 5040

typedef struct {
  unsigned P;
  double* ReTr;
  double* ImTr;
  int* block;
  int** mult;
  int* inv;
  int id;
  int* pool;  /* nearest-to-identity proposal pool */
  int npool;
} or_group;

typedef struct {
  const or_group* g;
  unsigned D, Nt, Nx, V;
  int* a;          /* a[i*D + mu] */
  unsigned* nn;    /* nn[i*2D + 2d + (s>0)] */
} or_lattice;

/* ------------------------------------------- shared arithmetic (dym_core.h) */

void or_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
  dym_u32x4 c = {{ctr[0], ctr[1], ctr[2], ctr[3]}};
  dym_u32x4 r = dym_philox4x32_10(c, key[0], key[1]);
  memcpy(out, r.v, sizeof r.v);
}
double or_exp(double x) { return dym_exp(x); }
uint32_t or_pick(uint32_t r0, uint32_t n) { return dym_pick(r0, n); }

/* ------------------------------------------------------------------ group */

void or_group_free(or_group* g) {
  if (!g) return;
  free(g->ReTr); free(g->ImTr); free(g->block); free(g->mult); free(g->inv); free(g->pool);
  free(g);
}

/* 0 ok; -2 cannot open; -3 malformed (truncated, out of range, no identity or
 * inverse); -8 order above OR_PMAX. */
int or_group_load(const char* fn, or_group** out) {
  *out = NULL;
  FILE* f = fopen(fn, "r");
  if (!f) return -2;
  int P = 0;
  if (fscanf(f, "%d", &P) != 1 || P <= 0) { fclose(f); return -3; }
  if (P > OR_PMAX) { fclose(f); return -8; }
  or_group* g = (or_group*)calloc(1, sizeof *g);
  g->P = (unsigned)P;
  g->ReTr = (double*)malloc(sizeof(double) * P);
  g->ImTr = (double*)malloc(sizeof(double) * P);
  g->block = (int*)malloc(sizeof(int) * (size_t)P * P);
  g->mult = (int**)malloc(sizeof(int*) * P);
  g->inv = (int*)malloc(sizeof(int) * P);
  for (int n = 0; n < P; ++n) g->mult[n] = g->block + (size_t)n * P;
  int bad = 0;
  for (int n = 0; n < P && !bad; ++n) bad = fscanf(f, "%lf", &g->ReTr[n]) != 1;
  for (int n = 0; n < P && !bad; ++n) bad = fscanf(f, "%lf", &g->ImTr[n]) != 1;
  for (size_t k = 0; k < (size_t)P * P && !bad; ++k) {
    bad = fscanf(f, "%d", &g->block[k]) != 1;
    if (!bad && (g->block[k] < 0 || g->block[k] >= P)) bad = 1;
  }
  fclose(f);
  if (bad) { or_group_free(g); return -3; }
  /* identity: first n whose row and column are the identity map */
  g->id = -1;
  for (int n = 0; n < P && g->id < 0; ++n) {
    int ok = 1;
    for (int m = 0; m < P && ok; ++m) ok = g->mult[n][m] == m && g->mult[m][n] == m;
    if (ok) g->id = n;
  }
  if (g->id < 0) { or_group_free(g); return -3; }
  for (int n = 0; n < P; ++n) {
    int found = -1;
    for (int m = 0; m < P && found < 0; ++m)
      if (g->mult[n][m] == g->id && g->mult[m][n] == g->id) found = m;
    if (found < 0) { or_group_free(g); return -3; }
    g->inv[n] = found;
  }
  /* proposal pool: elements at the second-smallest ReTr; min starts at 0
   * and the runner-up at 10, as in the reference */
  double lo = 0, next = 10;
  for (int n = 0; n < P; ++n) if (g->ReTr[n] < lo) lo = g->ReTr[n];
  for (int n = 0; n < P; ++n) if (g->ReTr[n] > lo && g->ReTr[n] < next) next = g->ReTr[n];
  g->pool = (int*)malloc(sizeof(int) * P);
  g->npool = 0;
  for (int n = 0; n < P; ++n)
    if (g->ReTr[n] < next + 1e-6 && g->ReTr[n] > lo) g->pool[g->npool++] = n;
  *out = g;
  return 0;
}

int or_group_order(const or_group* g) { return (int)g->P; }
int or_group_identity(const or_group* g) { return g->id; }
int or_group_pool(const or_group* g, int* pool) {
  if (pool) memcpy(pool, g->pool, sizeof(int) * g->npool);
  return g->npool;
}
void or_group_tables(const or_group* g, int* mult, int* inv, double* retr, double* imtr) {
  if (mult) memcpy(mult, g->block, sizeof(int) * (size_t)g->P * g->P);
  if (inv) memcpy(inv, g->inv, sizeof(int) * g->P);
  if (retr) memcpy(retr, g->ReTr, sizeof(double) * g->P);
  if (imtr) memcpy(imtr, g->ImTr, sizeof(double) * g->P);
}

/* ---------------------------------------------------------------- lattice */

static void coords_of(const or_lattice* L, unsigned idx, int* pos) {
  pos[0] = (int)(idx % L->Nt);
  idx /= L->Nt;
  for (unsigned d = 1; d < L->D; ++d) { pos[d] = (int)(idx % L->Nx); idx /= L->Nx; }
}

static unsigned index_of(const or_lattice* L, const int* pos) {
  long idx = 0;
  for (int d = (int)L->D - 1; d > 0; --d) idx = ((pos[d] + (long)L->Nx) % L->Nx) + (long)L->Nx * idx;
  return (unsigned)(((pos[0] + (long)L->Nt) % L->Nt) + (long)L->Nt * idx);
}

void or_lattice_free(or_lattice* L) {
  if (!L) return;
  free(L->a); free(L->nn); free(L);
}

int or_lattice_create(const or_group* g, int D, int Nt, int Nx, or_lattice** out) {
  *out = NULL;
  if (D < 2 || D > 8 || Nt < 1 || Nx < 1) return -1;
  or_lattice* L = (or_lattice*)calloc(1, sizeof *L);
  L->g = g; L->D = (unsigned)D; L->Nt = (unsigned)Nt; L->Nx = (unsigned)Nx;
  L->V = (unsigned)Nt;
  for (int d = 1; d < D; ++d) L->V *= (unsigned)Nx;
  L->a = (int*)malloc(sizeof(int) * (size_t)L->V * D);
  L->nn = (unsigned*)malloc(sizeof(unsigned) * (size_t)L->V * 2 * D);
  int pos[8];
  for (unsigned i = 0; i < L->V; ++i) {
    coords_of(L, i, pos);
    for (int d = 0; d < D; ++d) {
      pos[d] -= 1; L->nn[2 * D * i + 2 * d + 0] = index_of(L, pos);
      pos[d] += 2; L->nn[2 * D * i + 2 * d + 1] = index_of(L, pos);
      pos[d] -= 1;
    }
  }
  for (size_t k = 0; k < (size_t)L->V * D; ++k) L->a[k] = g->id;
  *out = L;
  return 0;
}

unsigned or_lattice_volume(const or_lattice* L) { return L->V; }

static inline unsigned stp(const or_lattice* L, unsigned i, unsigned d, int s) {
  return L->nn[i * 2 * L->D + d * 2 + (s > 0)];
}

/* Links in the engine's host layout: dm[d*V + site]. */
void or_set_links(or_lattice* L, const uint16_t* dm) {
  for (unsigned d = 0; d < L->D; ++d)
    for (unsigned i = 0; i < L->V; ++i) L->a[i * L->D + d] = dm[(size_t)d * L->V + i];
}
void or_get_links(const or_lattice* L, uint16_t* dm) {
  for (unsigned d = 0; d < L->D; ++d)
    for (unsigned i = 0; i < L->V; ++i) dm[(size_t)d * L->V + i] = (uint16_t)L->a[i * L->D + d];
}

/* Hot start: link (i, d) = floor(P * u), u from Philox counter (i, 0, d, HOT). */
void or_hot_start(or_lattice* L, uint64_t seed) {
  for (unsigned d = 0; d < L->D; ++d)
    for (unsigned i = 0; i < L->V; ++i) {
      dym_u32x4 c = {{i, 0u, d, DYM_TAG_HOT}};
      dym_u32x4 r = dym_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
      L->a[i * L->D + d] = (int)dym_pick(r.v[0], L->g->P);
    }
}

/* ---------------------------------------------------------------- staples */

/* A link term of a staple: the link at x + de*e_d + df*e_d1 in direction d
 * (DIR_D) or d1 (DIR_F), used inverted or not.  The eight staples of one
 * (d, d1) plane, in the reference's order: the two plaquette staples of
 * get_staples (dym-mod-metro.cpp:68-76), then the six rectangle staples of
 * get_rect_loops (dym-mod-metro.cpp:88-140). */
enum { DIR_D = 0, DIR_F = 1 };
typedef struct { int de, df, dir, inv; } term;
static const term PLAQ[2][3] = {
  {{1, 0, DIR_F, 0}, {0, 1, DIR_D, 1}, {0, 0, DIR_F, 1}},
  {{1, -1, DIR_F, 1}, {0, -1, DIR_D, 1}, {0, -1, DIR_F, 0}},
};
static const term RECT[6][5] = {
  {{1, 0, DIR_F, 0}, {1, 1, DIR_F, 0}, {0, 2, DIR_D, 1}, {0, 1, DIR_F, 1}, {0, 0, DIR_F, 1}},
  {{1, 0, DIR_D, 0}, {2, 0, DIR_F, 0}, {1, 1, DIR_D, 1}, {0, 1, DIR_D, 1}, {0, 0, DIR_F, 1}},
  {{1, 0, DIR_F, 0}, {0, 1, DIR_D, 1}, {-1, 1, DIR_D, 1}, {-1, 0, DIR_F, 1}, {-1, 0, DIR_D, 0}},
  {{1, -1, DIR_F, 1}, {1, -2, DIR_F, 1}, {0, -2, DIR_D, 1}, {0, -2, DIR_F, 0}, {0, -1, DIR_F, 0}},
  {{1, 0, DIR_D, 0}, {2, -1, DIR_F, 1}, {1, -1, DIR_D, 1}, {0, -1, DIR_D, 1}, {0, -1, DIR_F, 0}},
  {{1, -1, DIR_F, 1}, {0, -1, DIR_D, 1}, {-1, -1, DIR_D, 1}, {-1, -1, DIR_F, 0}, {-1, 0, DIR_D, 0}},
};

static unsigned walk(const or_lattice* L, unsigned i, unsigned d, unsigned d1, int de, int df) {
  for (; de > 0; --de) i = stp(L, i, d, 1);
  for (; de < 0; ++de) i = stp(L, i, d, -1);
  for (; df > 0; --df) i = stp(L, i, d1, 1);
  for (; df < 0; ++df) i = stp(L, i, d1, -1);
  return i;
}

static int fold(const or_lattice* L, unsigned i, unsigned d, unsigned d1, const term* t, int n) {
  const or_group* g = L->g;
  int acc = g->id;
  for (int k = 0; k < n; ++k) {
    unsigned s = walk(L, i, d, d1, t[k].de, t[k].df);
    int x = L->a[s * L->D + (t[k].dir == DIR_D ? d : d1)];
    if (t[k].inv) x = g->inv[x];
    acc = g->mult[acc][x];
  }
  return acc;
}

/* st: 2(D-1) plaquette staples; re: 6(D-1) rectangle staples. */
void or_staples(const or_lattice* L, unsigned i, unsigned d, int* st, int* re) {
  int k = 0, kr = 0;
  for (unsigned d1 = 0; d1 < L->D; ++d1) {
    if (d1 == d) continue;
    for (int p = 0; p < 2; ++p) st[k++] = fold(L, i, d, d1, PLAQ[p], 3);
    for (int r = 0; r < 6; ++r) re[kr++] = fold(L, i, d, d1, RECT[r], 5);
  }
}

/* Links (site, dir) read by the staples of link (i, d): out[2*k], out[2*k+1];
 * returns the count, 16*(D-1)*... terms with repeats. */
static int read_set(const or_lattice* L, unsigned i, unsigned d, unsigned* out) {
  int n = 0;
  for (unsigned d1 = 0; d1 < L->D; ++d1) {
    if (d1 == d) continue;
    for (int p = 0; p < 2; ++p)
      for (int k = 0; k < 3; ++k) {
        out[n++] = walk(L, i, d, d1, PLAQ[p][k].de, PLAQ[p][k].df);
        out[n++] = PLAQ[p][k].dir == DIR_D ? d : d1;
      }
    for (int r = 0; r < 6; ++r)
      for (int k = 0; k < 5; ++k) {
        out[n++] = walk(L, i, d, d1, RECT[r][k].de, RECT[r][k].df);
        out[n++] = RECT[r][k].dir == DIR_D ? d : d1;
      }
  }
  return n / 2;
}

/* Pairs (x, y) in one phase where updating x reads the link updated at y
 * (y != x), from the staple read sets above; 0 proves the schedule race-free.
 * Also counts links not visited exactly once per sweep. */
uint64_t or_schedule_conflicts(const or_lattice* L, const int* phase_dir, const uint32_t* phase_len,
                               const uint32_t* sites, int nphase) {
  const unsigned D = L->D, V = L->V;
  int* ph = (int*)malloc(sizeof(int) * V * D);
  int* seen = (int*)calloc((size_t)V * D, sizeof(int));
  for (size_t k = 0; k < (size_t)V * D; ++k) ph[k] = -1;
  size_t off = 0;
  for (int p = 0; p < nphase; ++p) {
    for (uint32_t k = 0; k < phase_len[p]; ++k) {
      ph[sites[off + k] * D + phase_dir[p]] = p;
      seen[sites[off + k] * D + phase_dir[p]]++;
    }
    off += phase_len[p];
  }
  uint64_t bad = 0;
  unsigned rs[2 * 8 * 40];
  off = 0;
  for (int p = 0; p < nphase; ++p) {
    const unsigned d = (unsigned)phase_dir[p];
    for (uint32_t k = 0; k < phase_len[p]; ++k) {
      const unsigned i = sites[off + k];
      int n = read_set(L, i, d, rs);
      for (int t = 0; t < n; ++t) {
        unsigned s = rs[2 * t], dd = rs[2 * t + 1];
        if (!(s == i && dd == d) && ph[s * D + dd] == p) ++bad;
      }
    }
    off += phase_len[p];
  }
  for (size_t k = 0; k < (size_t)V * D; ++k) if (seen[k] != 1) ++bad;
  free(ph); free(seen);
  return bad;
}

/* ------------------------------------------------------------------ sweep */

/* One multi-hit Metropolis visit of link (i, d) (dym-mod-metro.cpp:161-192).
 * pool == NULL: proposals uniform over the group. */
static void visit(or_lattice* L, unsigned i, unsigned d, double b0, double b1, double b2, uint64_t seed,
                  uint32_t sweep, int nhit, const int* pool, int npool, long* hit, long* acc) {
  const or_group* g = L->g;
  const int ns = 2 * ((int)L->D - 1), nr = 6 * ((int)L->D - 1);
  int st[2 * 7], re[6 * 7];
  or_staples(L, i, d, st, re);
  int b = L->a[i * L->D + d];
  double r1 = 0, m1 = 0;
  for (int j = 0; j < ns; ++j) r1 += g->ReTr[g->mult[b][st[j]]];
  for (int k = 0; k < nr; ++k) m1 += g->ReTr[g->mult[b][re[k]]];
  for (int h = 0; h < nhit; ++h) {
    dym_u32x4 r = dym_hit_random(seed, sweep, i, d, (uint32_t)h, DYM_TAG_METRO);
    /* reference: smallgroup[ smallgroup.size() * rand01 ] with truncation */
    const double u1 = (double)r.v[0] * 0x1p-32;
    const int gi = pool ? pool[(size_t)(npool * u1)] : (int)(size_t)(g->P * u1);
    const int bnew = g->mult[b][gi];
    double r1new = 0, m1new = 0;
    for (int j = 0; j < ns; ++j) r1new += g->ReTr[g->mult[bnew][st[j]]];
    for (int k = 0; k < nr; ++k) m1new += g->ReTr[g->mult[bnew][re[k]]];
    double oldact = b0 + b1 * r1 + b2 * m1;
    double newact = b0 + b1 * r1new + b2 * m1new;
    double probrat = (newact <= oldact) ? 1.0 : dym_exp(-(newact - oldact));
    ++*hit;
    if (probrat > dym_u53(r.v[1], r.v[2])) {
      L->a[i * L->D + d] = bnew;
      b = bnew; r1 = r1new; m1 = m1new;
      ++*acc;
    }
  }
}

/* nsweeps sweeps over the colour phases, sweep counters first_sweep, +1, ...
 * pool_all != 0: proposals uniform over the group.  nthreads <= 0: OpenMP
 * default.  counters[0] += hits, counters[1] += accepts. */
void or_sweep(or_lattice* L, const int* phase_dir, const uint32_t* phase_len, const uint32_t* sites, int nphase,
              double b0, double b1, double b2, uint64_t seed, uint32_t first_sweep, int nsweeps, int nhit,
              int pool_all, uint64_t* counters, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  const int* pool = pool_all ? NULL : L->g->pool;
  const int npool = L->g->npool;
  for (int s = 0; s < nsweeps; ++s) {
    size_t off = 0;
    for (int p = 0; p < nphase; ++p) {
      const unsigned d = (unsigned)phase_dir[p];
      const uint32_t* ps = sites + off;
      const long n = (long)phase_len[p];
      long lhit = 0, lacc = 0;
#pragma omp parallel for schedule(static) reduction(+ : lhit, lacc)
      for (long k = 0; k < n; ++k)
        visit(L, ps[k], d, b0, b1, b2, seed, first_sweep + (uint32_t)s, nhit, pool, npool, &lhit, &lacc);
      counters[0] += (uint64_t)lhit;
      counters[1] += (uint64_t)lacc;
      off += phase_len[p];
    }
  }
}

/* ------------------------------------------------------------ observables */

static int plaq_elem(const or_lattice* L, unsigned i, unsigned d1, unsigned d2) {
  const or_group* g = L->g;
  int x = g->mult[g->id][L->a[i * L->D + d1]];
  x = g->mult[x][L->a[stp(L, i, d1, 1) * L->D + d2]];
  x = g->mult[x][g->inv[L->a[stp(L, i, d2, 1) * L->D + d1]]];
  return g->mult[x][g->inv[L->a[i * L->D + d2]]];
}

static int wilson_elem(const or_lattice* L, unsigned i, unsigned d1, unsigned d2, int n1, int n2) {
  const or_group* g = L->g;
  int x = g->id;
  for (int j = 0; j < n1; ++j) { x = g->mult[x][L->a[i * L->D + d1]]; i = stp(L, i, d1, 1); }
  for (int j = 0; j < n2; ++j) { x = g->mult[x][L->a[i * L->D + d2]]; i = stp(L, i, d2, 1); }
  for (int j = 0; j < n1; ++j) { i = stp(L, i, d1, -1); x = g->mult[x][g->inv[L->a[i * L->D + d1]]]; }
  for (int j = 0; j < n2; ++j) { i = stp(L, i, d2, -1); x = g->mult[x][g->inv[L->a[i * L->D + d2]]]; }
  return x;
}

static double dot(const uint64_t* h, const double* w, unsigned P) {
  double s = 0;
  for (unsigned n = 0; n < P; ++n) s += (double)h[n] * w[n];
  return s;
}

/* out[0..3] = poly_re, poly_im, plaq, rect; out[4 + k*wl_nt + l] = Wilson
 * loop (k+1) x (l+1) for k < wl_nx, l < wl_nt.  hist (may be NULL) receives
 * the (3 + wl_nx*wl_nt) x P element histograms. */
void or_measure(const or_lattice* L, int wl_nx, int wl_nt, double* out, uint64_t* hist) {
  const or_group* g = L->g;
  const unsigned P = g->P, D = L->D, V = L->V;
  const size_t slots = 3 + (size_t)(wl_nx > 0 ? wl_nx : 0) * (wl_nt > 0 ? wl_nt : 0);
  uint64_t* h = (uint64_t*)calloc(slots * P, sizeof(uint64_t));
  int pos[8];
  for (unsigned i = 0; i < V; ++i) {
    for (unsigned d1 = 0; d1 < D; ++d1)
      for (unsigned d2 = d1 + 1; d2 < D; ++d2) h[plaq_elem(L, i, d1, d2)]++;
    for (unsigned d1 = 0; d1 < D; ++d1)
      for (unsigned d2 = 0; d2 < D; ++d2)
        if (d1 != d2) h[P + wilson_elem(L, i, d1, d2, 2, 1)]++;
    coords_of(L, i, pos);
    if (pos[0] == 0) {
      int r = g->id;
      unsigned s = i;
      do { r = g->mult[r][L->a[s * D + 0]]; s = stp(L, s, 0, 1); } while (s != i);
      h[2 * P + r]++;
    }
    for (int k = 0; k < wl_nx; ++k)
      for (int l = 0; l < wl_nt; ++l)
        for (unsigned d1 = 1; d1 < D; ++d1)
          h[(3 + (size_t)k * wl_nt + l) * P + wilson_elem(L, i, d1, 0, k + 1, l + 1)]++;
  }
  out[2] = dot(h, g->ReTr, P) / (double)(V * D * (D - 1) / 2);
  out[3] = dot(h + P, g->ReTr, P) / (double)(V * D * (D - 1));
  out[0] = dot(h + 2 * P, g->ReTr, P) / (double)(V / L->Nt);
  out[1] = dot(h + 2 * P, g->ImTr, P) / (double)(V / L->Nt);
  for (int k = 0; k < wl_nx; ++k)
    for (int l = 0; l < wl_nt; ++l)
      out[4 + k * wl_nt + l] = dot(h + (3 + (size_t)k * wl_nt + l) * P, g->ReTr, P) / (double)(V * (D - 1));
  if (hist) memcpy(hist, h, slots * P * sizeof(uint64_t));
  free(h);
}

/* -------------------------------------------------------------------- LLR */
/* Restatement of the engine's colour-parallel LLR (test oracle), following
 * llr.cpp:178-250 of the reference for the per-hit rule, the drive-in rule
 * and the Robbins-Monro step.  The reference tests the window after every
 * hit, one link at a time.  The engine lets every link of a colour class run
 * its hits at once (the links of a class share no plaquette or rectangle;
 * each hit weighs the exact integer sums of its terms' class values at scale
 * 2^dym_fix_shift, drive-in hits compare fixed-point energies) and
 * then scans the class in site-list order in blocks of dym_llr_block_links
 * links: a block's moves are kept iff the running energy plus their change
 * stays in the window (outside the window: iff it comes closer to the
 * centre), else its links get their old values back.  Each step of the scan
 * leaves the window-restricted distribution invariant, as the reference's
 * per-hit test does, and a block's change is at most a quarter of the window
 * width, so a block can always move away from a wall.  Energies
 * are exact 64-bit fixed-point sums of the plaquette and rectangle class
 * values (each value times 2^32, rounded): a kept link adds its exact integer
 * change, so the tracked energy never drifts from the configuration's, and
 * the FP64 energy the Robbins-Monro step averages is that sum times 2^-32. */

#define OR_MAXCLS 32
#define OR_FIX_S 32

/* ReTr value classes: elements sorted by ReTr, a new class whenever a value
 * exceeds the first value of the current class by more than 1e-9; the class
 * value is the ReTr of the class's lowest-numbered element. */
static int or_classes(const or_group* g, int* cls, double* val) {
  const unsigned P = g->P;
  int* ord = (int*)malloc(sizeof(int) * P);
  for (unsigned i = 0; i < P; ++i) ord[i] = (int)i;
  for (unsigned i = 1; i < P; ++i) { /* stable insertion sort by ReTr */
    int x = ord[i];
    int j = (int)i - 1;
    while (j >= 0 && g->ReTr[ord[j]] > g->ReTr[x]) { ord[j + 1] = ord[j]; --j; }
    ord[j + 1] = x;
  }
  int n = 0;
  double first = 0;
  for (unsigned k = 0; k < P; ++k) {
    int i = ord[k];
    if (k == 0 || g->ReTr[i] - first > 1e-9) { first = g->ReTr[i]; ++n; }
    cls[i] = n - 1;
  }
  free(ord);
  if (n > OR_MAXCLS) return -1;
  for (int c = 0; c < n; ++c) {
    for (unsigned i = 0; i < P; ++i)
      if (cls[i] == c) { val[c] = g->ReTr[i]; break; }
  }
  return n;
}

static long long or_class_fix(const long long* h, const long long* vf, int n) {
  long long s = 0;
  for (int c = 0; c < n; ++c) s += h[c] * vf[c];
  return s;
}

static long long or_fix(double x) { return llrint(ldexp(x, OR_FIX_S)); }

enum { OR_DRIVE = 0, OR_SETTLE = 1, OR_RM = 2, OR_DONE = 3, OR_UNREACHED = 4 };

/* The window tests of the scan on fixed-point energies (e1, e2): in the
 * window (box), and closer to the centre than (p1, p2). */
typedef struct {
  int dims, w;
  long long lo[2], hi[2], mid[2];
  double sc[2]; /* 2^-32 / half-width per axis (two-dimensional drive-in) */
} or_win;

static int or_in(const or_win* W, long long e1, long long e2) {
  if (W->dims == 2) return e1 >= W->lo[0] && e1 <= W->hi[0] && e2 >= W->lo[1] && e2 <= W->hi[1];
  const long long e = W->w == 0 ? e1 : e2;
  return e >= W->lo[0] && e <= W->hi[0];
}

static double or_nsq(const or_win* W, long long e1, long long e2) {
  const double x = (double)(e1 - W->mid[0]) * W->sc[0], y = (double)(e2 - W->mid[1]) * W->sc[1];
  return x * x + y * y;
}

static int or_closer(const or_win* W, long long e1, long long e2, long long p1, long long p2) {
  if (W->dims == 2) return or_nsq(W, e1, e2) < or_nsq(W, p1, p2);
  const long long e = W->w == 0 ? e1 : e2, p = W->w == 0 ? p1 : p2;
  return llabs(e - W->mid[0]) < llabs(p - W->mid[0]);
}

/* out[0..3] = a, S1, S2, mode; iout[0..5] = drive_sweeps, sweeps, hits,
 * accepts, links kept by the scan, links refused; a_hist[NRM]. */
/* dims == 2: a two-dimensional cell (llr2d.cpp:178-259), axis 1, S2 window
 * [ewin2 - hw2, ewin2 + hw2], bg is a2 and is Robbins-Monro updated too, a2_hist
 * receives it; drive-in compares squared normalised distances to the centre. */
static int llr_impl(or_lattice* L, const int* phase_dir, const uint32_t* phase_len, const uint32_t* sites,
                    int nphase, int axis, double bg, double ewin, double hw, double a0, int K, int NRM, int nhit,
                    int drive_cap, uint64_t seed, uint32_t first_sweep, double* out, int64_t* iout, double* a_hist,
                    int dims, double ewin2, double hw2, double* a2_hist) {
  const or_group* g = L->g;
  const unsigned D = L->D, V = L->V;
  int* cls = (int*)malloc(sizeof(int) * g->P);
  double v[OR_MAXCLS];
  long long vf[OR_MAXCLS];
  const int ncls = or_classes(g, cls, v);
  if (ncls < 0) { free(cls); return -6; }
  for (int c = 0; c < ncls; ++c) vf[c] = or_fix(v[c]);
  long long h[2][OR_MAXCLS] = {{0}};
  for (unsigned i = 0; i < V; ++i) {
    for (unsigned d1 = 0; d1 < D; ++d1)
      for (unsigned d2 = d1 + 1; d2 < D; ++d2) h[0][cls[plaq_elem(L, i, d1, d2)]]++;
    for (unsigned d1 = 0; d1 < D; ++d1)
      for (unsigned d2 = 0; d2 < D; ++d2)
        if (d1 != d2) h[1][cls[wilson_elem(L, i, d1, d2, 2, 1)]]++;
  }
  long long Ef[2] = {or_class_fix(h[0], vf, ncls), or_class_fix(h[1], vf, ncls)};
  double E[2] = {ldexp((double)Ef[0], -OR_FIX_S), ldexp((double)Ef[1], -OR_FIX_S)};
  const double W = 2 * hw, elo = ewin - hw, ehi = ewin + hw;
  const double emid = 0.5 * (elo + ehi), w2 = W * W;
  const double elo2 = ewin2 - hw2, ehi2 = ewin2 + hw2, emid2 = 0.5 * (elo2 + ehi2), w2b = (2 * hw2) * (2 * hw2);
  const double ihw0 = dims == 2 ? 1.0 / hw : 0, ihw1 = dims == 2 ? 1.0 / hw2 : 0;
  or_win win;
  win.dims = dims;
  win.w = axis - 1;
  win.lo[0] = or_fix(elo); win.hi[0] = or_fix(ehi); win.mid[0] = or_fix(emid);
  win.lo[1] = or_fix(elo2); win.hi[1] = or_fix(ehi2); win.mid[1] = or_fix(emid2);
  win.sc[0] = ldexp(ihw0, -OR_FIX_S); win.sc[1] = ldexp(ihw1, -OR_FIX_S);
  const int w = axis - 1;
  double a = a0, sumE = 0, sumE2 = 0;
  int mode = or_in(&win, Ef[0], Ef[1]) ? OR_RM : OR_DRIVE;
  if (NRM == 0 && mode == OR_RM) mode = OR_DONE;
  if (mode == OR_DRIVE && drive_cap == 0) mode = OR_UNREACHED;
  int k = 0, m = 0, drive_sweeps = 0;
  long long hits = 0, accs = 0, pacc = 0, prej = 0;
  const long max_sweeps = (long)drive_cap + (long)K * NRM + 2;
  long sweeps = 0;
  const int ns = 2 * ((int)D - 1), nr = 6 * ((int)D - 1), nt = ns + nr;
  double rmin = g->ReTr[0], rmax = g->ReTr[0];
  for (unsigned e = 1; e < g->P; ++e) {
    if (g->ReTr[e] < rmin) rmin = g->ReTr[e];
    if (g->ReTr[e] > rmax) rmax = g->ReTr[e];
  }
  const int blk = dym_llr_block_links((int)D, rmax - rmin, dims, axis, hw, hw2);
  /* The hits compare exact integer sums of class values at the scale 2^S of
   * the mixed-precision sweep (dym_fix_shift); vS per class. */
  const int S = dym_fix_shift(fabs(rmax) > fabs(rmin) ? fabs(rmax) : fabs(rmin), (int)D);
  const int up = OR_FIX_S - S;
  long long vS[OR_MAXCLS];
  for (int c = 0; c < ncls; ++c) vS[c] = llrint(ldexp(v[c], S));
  /* Changed links of one phase: position in the phase, site, old value,
   * fixed-point energy changes. */
  uint32_t* rp = (uint32_t*)malloc(sizeof(uint32_t) * V);
  uint32_t* rs = (uint32_t*)malloc(sizeof(uint32_t) * V);
  int* rb0 = (int*)malloc(sizeof(int) * V);
  long long* rde = (long long*)malloc(sizeof(long long) * 2 * V);
  while (mode < OR_DONE && sweeps < max_sweeps) {
    const uint32_t sweep = first_sweep + (uint32_t)sweeps;
    size_t off = 0;
    for (int p = 0; p < nphase && mode < OR_DONE; ++p) {
      const unsigned dir = (unsigned)phase_dir[p];
      int nchg = 0;
      const int drive = (mode == OR_DRIVE);
      for (uint32_t kk = 0; kk < phase_len[p]; ++kk) {
        const unsigned i = sites[off + kk];
        int st[2 * 7], re[6 * 7];
        or_staples(L, i, dir, st, re);
        const int b0 = L->a[i * D + dir];
        int b = b0;
        long long R = 0, M = 0;
        for (int j = 0; j < ns; ++j) R += vS[cls[g->mult[b][st[j]]]];
        for (int j = 0; j < nr; ++j) M += vS[cls[g->mult[b][re[j]]]];
        long long cum1 = 0, cum2 = 0; /* drive-in: the link's moves so far, scale 2^32 */
        for (int hh = 0; hh < nhit; ++hh) {
          dym_u32x4 r = dym_hit_random(seed, sweep, i, dir, (uint32_t)hh, DYM_TAG_LLR);
          const double u1 = (double)r.v[0] * 0x1p-32;
          const int bnew = g->mult[b][g->pool[(size_t)(g->npool * u1)]];
          long long Rn = 0, Mn = 0;
          for (int j = 0; j < ns; ++j) Rn += vS[cls[g->mult[bnew][st[j]]]];
          for (int j = 0; j < nr; ++j) Mn += vS[cls[g->mult[bnew][re[j]]]];
          const long long d1 = Rn - R, d2 = Mn - M;
          int acc;
          long long n1 = 0, n2 = 0;
          if (drive) {
            n1 = cum1 + d1 * (1ll << up);
            n2 = cum2 + d2 * (1ll << up);
            acc = or_closer(&win, Ef[0] + n1, Ef[1] + n2, Ef[0] + cum1, Ef[1] + cum2);
          } else {
            const double dS1 = ldexp((double)d1, -S), dS2 = ldexp((double)d2, -S);
            const double dEw = axis == 1 ? dS1 : dS2, dEbg = axis == 1 ? dS2 : dS1;
            acc = dym_weight_accept(-a * dEw - bg * dEbg, dym_u53(r.v[1], r.v[2]));
          }
          ++hits;
          if (acc) { b = bnew; R = Rn; M = Mn; cum1 = n1; cum2 = n2; ++accs; }
        }
        if (b != b0) {
          L->a[i * D + dir] = b;
          long long de1 = 0, de2 = 0;
          for (int j = 0; j < nt; ++j) {
            const int s = j < ns ? st[j] : re[j - ns];
            const long long dv = vf[cls[g->mult[b][s]]] - vf[cls[g->mult[b0][s]]];
            if (j < ns) de1 += dv;
            else de2 += dv;
          }
          rp[nchg] = kk;
          rs[nchg] = i;
          rb0[nchg] = b0;
          rde[2 * nchg] = de1;
          rde[2 * nchg + 1] = de2;
          ++nchg;
        }
      }
      off += phase_len[p];
      /* The scan, block by block in site-list order. */
      long long R1 = Ef[0], R2 = Ef[1];
      for (int c2 = 0; c2 < nchg;) {
        const uint32_t b = rp[c2] / (uint32_t)blk;
        int e2 = c2;
        long long s1 = 0, s2 = 0;
        while (e2 < nchg && rp[e2] / (uint32_t)blk == b) { s1 += rde[2 * e2]; s2 += rde[2 * e2 + 1]; ++e2; }
        const long long n1 = R1 + s1, n2 = R2 + s2;
        const int keep = drive ? or_closer(&win, n1, n2, R1, R2) : or_in(&win, n1, n2);
        if (keep) {
          R1 = n1;
          R2 = n2;
          pacc += e2 - c2;
        } else {
          for (int x = c2; x < e2; ++x) L->a[rs[x] * D + dir] = rb0[x];
          prej += e2 - c2;
        }
        c2 = e2;
      }
      Ef[0] = R1;
      Ef[1] = R2;
      E[0] = ldexp((double)Ef[0], -OR_FIX_S);
      E[1] = ldexp((double)Ef[1], -OR_FIX_S);
      if (mode == OR_DRIVE && or_in(&win, Ef[0], Ef[1])) mode = OR_SETTLE;
      if (p == nphase - 1) {
        if (mode == OR_DRIVE) {
          if (++drive_sweeps >= drive_cap) mode = OR_UNREACHED;
        } else if (mode == OR_SETTLE) {
          mode = NRM > 0 ? OR_RM : OR_DONE; k = 0; m = 0; sumE = 0; sumE2 = 0;
        } else if (mode == OR_RM) {
          sumE = sumE + E[w];
          if (dims == 2) sumE2 = sumE2 + E[1];
          if (++k == K) {
            const double gg = sumE / (double)K - ewin;
            const double step = 12.0 / (w2 * (double)(m + 1));
            a = a + step * gg;
            if (a_hist) a_hist[m] = a;
            if (dims == 2) {
              const double g2 = sumE2 / (double)K - ewin2;
              const double step2 = 12.0 / (w2b * (double)(m + 1));
              bg = bg + step2 * g2;
              if (a2_hist) a2_hist[m] = bg;
            }
            ++m; k = 0; sumE = 0; sumE2 = 0;
            if (m >= NRM) mode = OR_DONE;
          }
        }
      }
    }
    ++sweeps;
  }
  out[0] = a; out[1] = E[0]; out[2] = E[1]; out[3] = mode;
  iout[0] = drive_sweeps; iout[1] = sweeps; iout[2] = hits; iout[3] = accs; iout[4] = pacc; iout[5] = prej;
  free(cls); free(rp); free(rs); free(rb0); free(rde);
  if (dims == 2) out[4] = bg;
  return 0;
}

int or_llr_run(or_lattice* L, const int* phase_dir, const uint32_t* phase_len, const uint32_t* sites, int nphase,
               int axis, double bg, double ewin, double hw, double a0, int K, int NRM, int nhit, int drive_cap,
               uint64_t seed, uint32_t first_sweep, double* out, int64_t* iout, double* a_hist) {
  return llr_impl(L, phase_dir, phase_len, sites, nphase, axis, bg, ewin, hw, a0, K, NRM, nhit, drive_cap, seed,
                  first_sweep, out, iout, a_hist, 1, 0.0, 1.0, NULL);
}

/* Two-dimensional cell; out[0] a1, out[4] a2 (llr2d.cpp:178-259 with the
 * colour-parallel rule of or_llr_run). */
int or_llr2d_run(or_lattice* L, const int* phase_dir, const uint32_t* phase_len, const uint32_t* sites, int nphase,
                 double E1, double hw1, double E2, double hw2, double a1, double a2, int K, int NRM, int nhit,
                 int drive_cap, uint64_t seed, uint32_t first_sweep, double* out, int64_t* iout, double* a1_hist,
                 double* a2_hist) {
  return llr_impl(L, phase_dir, phase_len, sites, nphase, 1, a2, E1, hw1, a1, K, NRM, nhit, drive_cap, seed,
                  first_sweep, out, iout, a1_hist, 2, E2, hw2, a2_hist);
}

/* S1, S2 of the current configuration by the reference's loops (serial). */
void or_energies(const or_lattice* L, double* S1, double* S2) {
  const unsigned D = L->D, V = L->V;
  double s1 = 0, s2 = 0;
  for (unsigned i = 0; i < V; ++i) {
    for (unsigned d1 = 0; d1 < D; ++d1)
      for (unsigned d2 = d1 + 1; d2 < D; ++d2) s1 += L->g->ReTr[plaq_elem(L, i, d1, d2)];
    for (unsigned d1 = 0; d1 < D; ++d1)
      for (unsigned d2 = 0; d2 < D; ++d2)
        if (d1 != d2) s2 += L->g->ReTr[wilson_elem(L, i, d1, d2, 2, 1)];
  }
  *S1 = s1;
  *S2 = s2;
}
