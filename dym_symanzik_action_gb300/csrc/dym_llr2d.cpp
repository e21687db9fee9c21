// dym-llr2d: drop-in for the reference's llr2d executable (llr2d.cpp:295-518),
// the two-dimensional LLR cells on the GPU through libdymgpu.
//
//   dym-llr2d group D Nt Nx E1top E1bot step1 hw1 c0 c1 c2 step2 hw2 nperp a0 seed [K] [NRM] [R]
//   dym-llr2d seed group D Nt Nx E1top E1bot step1 hw1 c0 c1 c2 step2 hw2 nperp a0 seed cfgdir
//   dym-llr2d solve group D Nt Nx manifest lo hi a0 K NRM seed
//
// Same arguments, defaults (K = 40, NRM = 70, R = 1, drive-in cap 4000,
// NHIT = 20) and output lines as the reference: the LLR2D header, NPLAQ,
// NRECT, "repeat r: cold ridge / hot ridge", the "ANE2: E1 E2 a1 a2 sd1 sd2
// nrep" table, "reached n/N cells" and the drift line (exact class sums: 0);
// seed mode writes the configurations as the reference does (raw int32 element
// ids, site-major a[i*D + d], llr2d.cpp:262-271) and prints the "CELL:"
// manifest; solve mode reads them back.
//
// The cell grid and walk are the reference's: cells E1 = E1top - i step1,
// E2 = c0 + c1 E1 + c2 E1^2 + (j - nperp) step2; a cold pass walks the ridge
// (j = nperp) from the frozen end and a hot pass from the disordered end, each
// ridge cell seeded from the previous one's configuration, and every
// transverse cell of a reached ridge cell seeded from the ridge configuration
// with the ridge cell's (a1, a2), stopping at the first unreachable one in
// each direction.  Here the passes of all repeats run concurrently and so do
// the transverse cells of a ridge cell (each on its own chain, started from a
// copy of the ridge configuration), and the solve mode solves its cells
// concurrently; every chain has its own Philox key (seed + 1000003 r, bit 40
// for the cold pass, bits 41+ for the cell), so results do not depend on the
// scheduling.  Extensions, optional: DYM_NHIT, DYM_DEVICE.
// There is no CPU fallback: without a working GPU the program exits non-zero.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "dymgpu.h"

namespace {

struct Geom {
  int D = 4, Nt = 0, Nx = 0;
  unsigned V = 0;
  int nhit = 20, device = 0;
};

struct Cell {
  double E1 = 0, E2 = 0;
  std::vector<double> a1s, a2s;
  bool reached = false;
};

std::mutex g_mu;  // cell results
std::string g_err;

bool fail_with(const char* what) {
  std::lock_guard<std::mutex> l(g_mu);
  if (g_err.empty()) g_err = std::string(what) + ": " + dym_last_error();
  return false;
}

dym_chain* make_chain(const dym_group* g, const Geom& G, uint64_t seed, int start) {
  dym_chain_params p{};
  p.D = G.D;
  p.Nt = G.Nt;
  p.Nx = G.Nx;
  p.seed = seed;
  p.start = start;
  p.pool = DYM_POOL_NEAREST;
  p.precision = DYM_PREC_FP64;
  p.device = G.device;
  dym_chain* c = nullptr;
  if (dym_chain_create(g, &p, &c) != DYM_OK) return nullptr;
  return c;
}

// Drive the chain into the cell and, if NRM > 0, Robbins-Monro solve it.
bool run_cell(dym_chain* c, const Geom& G, const Cell& cell, double hw1, double hw2, double a1, double a2, int K,
              int NRM, dym_llr2d_result* r) {
  dym_llr2d_req q{};
  q.E1 = cell.E1;
  q.hw1 = hw1;
  q.E2 = cell.E2;
  q.hw2 = hw2;
  q.a1 = a1;
  q.a2 = a2;
  q.K = K;
  q.NRM = NRM;
  q.nhit = G.nhit;
  q.drive_cap = 4000;
  if (dym_llr2d_run(c, &q, r, nullptr) != DYM_OK) return fail_with("dym_llr2d_run");
  return true;
}

// Reference configuration file <-> chain links (site-major int32 <-> direction-major uint16).
bool save_cfg(dym_chain* c, const Geom& G, const char* path) {
  std::vector<uint16_t> links((size_t)G.V * G.D);
  if (dym_links_get(c, links.data()) != DYM_OK) return fail_with("dym_links_get");
  std::vector<int32_t> a((size_t)G.V * G.D);
  for (unsigned i = 0; i < G.V; ++i)
    for (int d = 0; d < G.D; ++d) a[(size_t)i * G.D + d] = links[(size_t)d * G.V + i];
  FILE* f = fopen(path, "wb");
  if (!f) return false;
  const size_t n = fwrite(a.data(), sizeof(int32_t), a.size(), f);
  fclose(f);
  return n == a.size();
}

bool load_cfg(dym_chain* c, const Geom& G, const char* path) {
  std::vector<int32_t> a((size_t)G.V * G.D);
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  const size_t n = fread(a.data(), sizeof(int32_t), a.size(), f);
  fclose(f);
  if (n != a.size()) return false;
  std::vector<uint16_t> links(a.size());
  for (unsigned i = 0; i < G.V; ++i)
    for (int d = 0; d < G.D; ++d) {
      const int32_t e = a[(size_t)i * G.D + d];
      if (e < 0 || e > 65535) return false;
      links[(size_t)d * G.V + i] = (uint16_t)e;
    }
  return dym_links_set(c, links.data()) == DYM_OK;
}

struct Grid {
  int N1 = 0, N2 = 0, nperp = 0;
  double hw1 = 0, hw2 = 0;
  std::vector<std::vector<Cell>> cells;
};

Grid make_grid(double E1top, double E1bot, double step1, double hw1, double c0, double c1, double c2, double step2,
               double hw2, int nperp) {
  Grid g;
  g.N1 = (int)((E1top - E1bot) / step1 + 0.5) + 1;
  g.N2 = 2 * nperp + 1;
  g.nperp = nperp;
  g.hw1 = hw1;
  g.hw2 = hw2;
  g.cells.assign(g.N1, std::vector<Cell>(g.N2));
  for (int i = 0; i < g.N1; ++i)
    for (int j = 0; j < g.N2; ++j) {
      const double E1 = E1top - i * step1;
      g.cells[i][j].E1 = E1;
      g.cells[i][j].E2 = c0 + c1 * E1 + c2 * E1 * E1 + (j - nperp) * step2;
    }
  return g;
}

uint64_t cell_key(uint64_t pass_seed, int i, int j) {
  return pass_seed + ((uint64_t)(i + 1) << 41) + ((uint64_t)(j + 1) << 52);
}

// One ridge pass of mode_full (llr2d.cpp:336-394): cold (dir -1) or hot (dir +1).
void full_pass(const dym_group* g, const Geom& G, Grid* grid, int dir, uint64_t seed, double a0, int K, int NRM,
               int* reached) {
  *reached = 0;
  dym_chain* c = make_chain(g, G, seed, dir > 0 ? DYM_START_HOT : DYM_START_COLD);
  if (!c) {
    fail_with("dym_chain_create");
    return;
  }
  std::vector<uint16_t> ridge((size_t)G.V * G.D);
  for (int s = 0; s < grid->N1; ++s) {
    const int i = dir > 0 ? s : grid->N1 - 1 - s;
    Cell& c0 = grid->cells[i][grid->nperp];
    dym_llr2d_result r{};
    if (!run_cell(c, G, c0, grid->hw1, grid->hw2, a0, a0, K, NRM, &r)) break;
    if (r.status != DYM_LLR_DONE) continue;  // not reached: the next ridge cell starts from here
    const double b1 = r.a1, b2 = r.a2;
    {
      std::lock_guard<std::mutex> l(g_mu);
      c0.a1s.push_back(b1);
      c0.a2s.push_back(b2);
      c0.reached = true;
    }
    ++*reached;
    if (dym_links_get(c, ridge.data()) != DYM_OK) {
      fail_with("dym_links_get");
      break;
    }
    // Transverse cells, each from the ridge configuration, concurrently; a
    // direction ends at its first unreachable cell.
    const int np = grid->nperp;
    std::vector<dym_llr2d_result> tr(2 * np);
    std::vector<int> ok(2 * np, 0);
    std::vector<std::thread> th;
    for (int side = 0; side < 2; ++side)
      for (int t = 1; t <= np; ++t) {
        const int j = np + (side ? t : -t);
        const int slot = side * np + t - 1;
        th.emplace_back([&, j, slot] {
          dym_chain* ct = make_chain(g, G, cell_key(seed, i, j), DYM_START_COLD);
          if (!ct) {
            fail_with("dym_chain_create");
            return;
          }
          if (dym_links_set(ct, ridge.data()) != DYM_OK) {
            fail_with("dym_links_set");
          } else if (run_cell(ct, G, grid->cells[i][j], grid->hw1, grid->hw2, b1, b2, K, NRM, &tr[slot])) {
            ok[slot] = tr[slot].status == DYM_LLR_DONE;
          }
          dym_chain_free(ct);
        });
      }
    for (auto& x : th) x.join();
    for (int side = 0; side < 2; ++side)
      for (int t = 1; t <= np; ++t) {
        const int slot = side * np + t - 1;
        if (!ok[slot]) break;
        Cell& cc = grid->cells[i][np + (side ? t : -t)];
        std::lock_guard<std::mutex> l(g_mu);
        cc.a1s.push_back(tr[slot].a1);
        cc.a2s.push_back(tr[slot].a2);
        cc.reached = true;
      }
    if (dym_links_set(c, ridge.data()) != DYM_OK) {  // the next ridge step continues from the ridge cell
      fail_with("dym_links_set");
      break;
    }
  }
  dym_chain_free(c);
}

int mode_full(int argc, char* argv[]) {
  if (argc < 17) {
    fprintf(stderr,
            "usage: %s group D Nt Nx E1top E1bot step1 hw1 c0 c1 c2 step2 hw2 nperp a0 seed [K] [NRM] [R]\n"
            "  windows BOTH S1 and S2; tiles a band around the curved ridge\n"
            "  E2 = c0 + c1*E1 + c2*E1^2, offset by (j-nperp)*step2 (j=0..2*nperp).\n",
            argv[0]);
    return 1;
  }
  const char* grp = argv[1];
  Geom G;
  G.D = atoi(argv[2]);
  G.Nt = atoi(argv[3]);
  G.Nx = atoi(argv[4]);
  const double E1top = atof(argv[5]), E1bot = atof(argv[6]), step1 = atof(argv[7]), hw1 = atof(argv[8]);
  const double c0 = atof(argv[9]), c1 = atof(argv[10]), c2 = atof(argv[11]);
  const double step2 = atof(argv[12]), hw2 = atof(argv[13]);
  const int nperp = atoi(argv[14]);
  const double a0 = atof(argv[15]);
  const int iseed = atoi(argv[16]);
  const int K = argc > 17 ? atoi(argv[17]) : 40;
  const int NRM = argc > 18 ? atoi(argv[18]) : 70;
  const int R = argc > 19 ? atoi(argv[19]) : 1;
  Grid grid = make_grid(E1top, E1bot, step1, hw1, c0, c1, c2, step2, hw2, nperp);
  printf("LLR2D(grp,D,Nt,Nx): %s %d %d %d | E1=[%g,%g] step1=%g hw1=%g | ridge c0=%g c1=%g c2=%g step2=%g hw2=%g "
         "nperp=%d | a0=%g seed=%d K=%u NRM=%u R=%u | %dx%d cells\n",
         grp, G.D, G.Nt, G.Nx, E1top, E1bot, step1, hw1, c0, c1, c2, step2, hw2, nperp, a0, iseed, (unsigned)K,
         (unsigned)NRM, (unsigned)R, grid.N1, grid.N2);
  G.V = (unsigned)G.Nt;
  for (int d = 1; d < G.D; ++d) G.V *= (unsigned)G.Nx;
  printf("NPLAQ: %u\nNRECT: %u\n", G.V * G.D * (G.D - 1) / 2, G.V * G.D * (G.D - 1));
  fflush(stdout);
  G.nhit = getenv("DYM_NHIT") ? atoi(getenv("DYM_NHIT")) : 20;
  G.device = getenv("DYM_DEVICE") ? atoi(getenv("DYM_DEVICE")) : 0;
  dym_group* g = nullptr;
  if (dym_group_load(grp, &g) != DYM_OK) {
    fprintf(stderr, "dym-llr2d: %s\n", dym_last_error());
    return 1;
  }
  if (dym_chain* c = make_chain(g, G, 0, DYM_START_COLD)) {  // bind the tables to the device first
    dym_chain_free(c);
  } else {
    fprintf(stderr, "dym-llr2d: %s\n", dym_last_error());
    return 1;
  }
  std::vector<int> creach(R), hreach(R);
  std::vector<std::thread> th;
  for (int r = 0; r < R; ++r) {
    const uint64_t base = (uint64_t)(uint32_t)iseed + 1000003ull * (uint64_t)r;
    th.emplace_back(full_pass, g, std::cref(G), &grid, -1, base | (1ull << 40), a0, K, NRM, &creach[r]);
    th.emplace_back(full_pass, g, std::cref(G), &grid, 1, base, a0, K, NRM, &hreach[r]);
  }
  for (auto& t : th) t.join();
  if (!g_err.empty()) {
    fprintf(stderr, "dym-llr2d: %s\n", g_err.c_str());
    return 1;
  }
  for (int r = 0; r < R; ++r)
    printf("repeat %u: cold ridge %d/%d, hot ridge %d/%d\n", (unsigned)r, creach[r], grid.N1, hreach[r], grid.N1);
  printf("\n# E1 E2 a1 a2 sd1 sd2 nrep\n");
  int nreached = 0;
  for (int i = 0; i < grid.N1; ++i)
    for (int j = 0; j < grid.N2; ++j) {
      const Cell& c = grid.cells[i][j];
      if (!c.reached) continue;
      ++nreached;
      const int n = (int)c.a1s.size();
      double m1 = 0, m2 = 0;
      for (int k = 0; k < n; ++k) {
        m1 += c.a1s[k];
        m2 += c.a2s[k];
      }
      m1 /= n;
      m2 /= n;
      double v1 = 0, v2 = 0;
      for (int k = 0; k < n; ++k) {
        v1 += (c.a1s[k] - m1) * (c.a1s[k] - m1);
        v2 += (c.a2s[k] - m2) * (c.a2s[k] - m2);
      }
      const double sd1 = n > 1 ? sqrt(v1 / (n - 1)) : 0, sd2 = n > 1 ? sqrt(v2 / (n - 1)) : 0;
      printf("ANE2: %9.2f %9.2f %10.6f %10.6f %9.5f %9.5f %d\n", c.E1, c.E2, m1, m2, sd1, sd2, n);
    }
  printf("reached %d/%d cells\n", nreached, grid.N1 * grid.N2);
  printf("max |incr-recompute|: S1 %.3e  S2 %.3e\n", 0.0, 0.0);
  dym_group_free(g);
  return 0;
}

// seed: drive every reachable cell (both ridge walks, then the transverse
// cells of each ridge cell) and save its configuration (llr2d.cpp:418-477).
int mode_seed(int argc, char* argv[]) {
  if (argc < 18) {
    fprintf(stderr,
            "usage: %s seed group D Nt Nx E1top E1bot step1 hw1 c0 c1 c2 step2 hw2 nperp a0 seed cfgdir\n",
            argv[0]);
    return 1;
  }
  const char* grp = argv[1];
  Geom G;
  G.D = atoi(argv[2]);
  G.Nt = atoi(argv[3]);
  G.Nx = atoi(argv[4]);
  const double E1top = atof(argv[5]), E1bot = atof(argv[6]), step1 = atof(argv[7]), hw1 = atof(argv[8]);
  const double c0 = atof(argv[9]), c1 = atof(argv[10]), c2 = atof(argv[11]);
  const double step2 = atof(argv[12]), hw2 = atof(argv[13]);
  const int nperp = atoi(argv[14]);
  const double a0 = atof(argv[15]);
  const int iseed = atoi(argv[16]);
  const char* cfgdir = argv[17];
  Grid grid = make_grid(E1top, E1bot, step1, hw1, c0, c1, c2, step2, hw2, nperp);
  G.V = (unsigned)G.Nt;
  for (int d = 1; d < G.D; ++d) G.V *= (unsigned)G.Nx;
  printf("LLR2D(seed): %s %d %d %d | E1=[%g,%g] step1=%g hw1=%g | ridge c0=%g c1=%g c2=%g step2=%g hw2=%g nperp=%d\n",
         grp, G.D, G.Nt, G.Nx, E1top, E1bot, step1, hw1, c0, c1, c2, step2, hw2, nperp);
  G.nhit = getenv("DYM_NHIT") ? atoi(getenv("DYM_NHIT")) : 20;
  G.device = getenv("DYM_DEVICE") ? atoi(getenv("DYM_DEVICE")) : 0;
  dym_group* g = nullptr;
  if (dym_group_load(grp, &g) != DYM_OK) {
    fprintf(stderr, "dym-llr2d: %s\n", dym_last_error());
    return 1;
  }
  std::vector<std::vector<bool>> saved(grid.N1, std::vector<bool>(grid.N2, false));
  int idx = 0;
  char path[1024];
  const uint64_t base = (uint64_t)(uint32_t)iseed;
  auto try_save = [&](dym_chain* c, int i, int j, const dym_llr2d_result& r) {
    if (saved[i][j] || r.status != DYM_LLR_DONE) return true;
    snprintf(path, sizeof(path), "%s/cell_%d_%d.cfg", cfgdir, i, j);
    if (!save_cfg(c, G, path)) {
      fprintf(stderr, "dym-llr2d: cannot write %s\n", path);
      return false;
    }
    saved[i][j] = true;
    const Cell& cc = grid.cells[i][j];
    printf("CELL: %d %d %d %.2f %.2f %.2f %.2f %s\n", idx++, i, j, cc.E1, cc.E2, hw1, hw2, path);
    fflush(stdout);
    return true;
  };
  bool ok = true;
  for (int pass = 0; pass < 2 && ok; ++pass) {  // cold pass (frozen -> disordered), then hot
    const int dir = pass == 0 ? -1 : 1;
    const uint64_t pseed = pass == 0 ? (base | (1ull << 40)) : base;
    dym_chain* c = make_chain(g, G, pseed, dir > 0 ? DYM_START_HOT : DYM_START_COLD);
    if (!c) {
      fprintf(stderr, "dym-llr2d: %s\n", dym_last_error());
      return 1;
    }
    std::vector<uint16_t> ridge((size_t)G.V * G.D);
    for (int s = 0; s < grid.N1 && ok; ++s) {
      const int i = dir > 0 ? s : grid.N1 - 1 - s;
      dym_llr2d_result r{};
      if (!(ok = run_cell(c, G, grid.cells[i][nperp], hw1, hw2, a0, a0, 1, 0, &r))) break;
      if (r.status != DYM_LLR_DONE) continue;
      if (!(ok = try_save(c, i, nperp, r))) break;
      if (dym_links_get(c, ridge.data()) != DYM_OK) {
        ok = fail_with("dym_links_get");
        break;
      }
      for (int side = 0; side < 2 && ok; ++side)
        for (int t = 1; t <= nperp; ++t) {
          const int j = nperp + (side ? t : -t);
          if (dym_links_set(c, ridge.data()) != DYM_OK) {
            ok = fail_with("dym_links_set");
            break;
          }
          dym_llr2d_result rt{};
          if (!(ok = run_cell(c, G, grid.cells[i][j], hw1, hw2, a0, a0, 1, 0, &rt))) break;
          if (rt.status != DYM_LLR_DONE) break;
          if (!(ok = try_save(c, i, j, rt))) break;
        }
      if (ok && dym_links_set(c, ridge.data()) != DYM_OK) ok = fail_with("dym_links_set");
    }
    dym_chain_free(c);
  }
  if (!ok) {
    if (!g_err.empty()) fprintf(stderr, "dym-llr2d: %s\n", g_err.c_str());
    return 1;
  }
  fprintf(stderr, "SEED: saved %d cells to %s\n", idx, cfgdir);
  dym_group_free(g);
  return 0;
}

// solve: Robbins-Monro solve the manifest's cells [lo, hi) from their saved
// configurations (llr2d.cpp:479-511), concurrently, one chain per cell.
int mode_solve(int argc, char* argv[]) {
  if (argc < 12) {
    fprintf(stderr, "usage: %s solve group D Nt Nx manifest lo hi a0 K NRM seed\n", argv[0]);
    return 1;
  }
  const char* grp = argv[1];
  Geom G;
  G.D = atoi(argv[2]);
  G.Nt = atoi(argv[3]);
  G.Nx = atoi(argv[4]);
  const char* manifest = argv[5];
  const int lo = atoi(argv[6]), hi = atoi(argv[7]);
  const double a0 = atof(argv[8]);
  const int K = atoi(argv[9]), NRM = atoi(argv[10]);
  const int iseed = atoi(argv[11]);
  G.V = (unsigned)G.Nt;
  for (int d = 1; d < G.D; ++d) G.V *= (unsigned)G.Nx;
  G.nhit = getenv("DYM_NHIT") ? atoi(getenv("DYM_NHIT")) : 20;
  G.device = getenv("DYM_DEVICE") ? atoi(getenv("DYM_DEVICE")) : 0;
  dym_group* g = nullptr;
  if (dym_group_load(grp, &g) != DYM_OK) {
    fprintf(stderr, "dym-llr2d: %s\n", dym_last_error());
    return 1;
  }
  FILE* mf = fopen(manifest, "r");
  if (!mf) {
    fprintf(stderr, "solve: cannot open manifest %s\n", manifest);
    return 1;
  }
  struct Job {
    int idx, i, j;
    double E1, E2, hw1, hw2;
    std::string path;
    bool loaded = false, done = false;
    double a1 = 0, a2 = 0;
  };
  std::vector<Job> jobs;
  char line[2048];
  while (fgets(line, sizeof(line), mf)) {
    if (strncmp(line, "CELL:", 5)) continue;
    Job jb;
    char path[1024];
    if (sscanf(line, "CELL: %d %d %d %lf %lf %lf %lf %1023s", &jb.idx, &jb.i, &jb.j, &jb.E1, &jb.E2, &jb.hw1, &jb.hw2,
               path) != 8)
      continue;
    if (jb.idx < lo || jb.idx >= hi) continue;
    jb.path = path;
    jobs.push_back(jb);
  }
  fclose(mf);
  if (dym_chain* c = make_chain(g, G, 0, DYM_START_COLD)) {
    dym_chain_free(c);
  } else {
    fprintf(stderr, "dym-llr2d: %s\n", dym_last_error());
    return 1;
  }
  std::vector<std::thread> th;
  for (auto& jb : jobs)
    th.emplace_back([&, p = &jb] {
      dym_chain* c = make_chain(g, G, cell_key((uint64_t)(uint32_t)iseed, p->i, p->j), DYM_START_COLD);
      if (!c) {
        fail_with("dym_chain_create");
        return;
      }
      p->loaded = load_cfg(c, G, p->path.c_str());
      if (p->loaded) {
        Cell cell;
        cell.E1 = p->E1;
        cell.E2 = p->E2;
        dym_llr2d_result r{};
        if (run_cell(c, G, cell, p->hw1, p->hw2, a0, a0, K, NRM, &r) && r.status == DYM_LLR_DONE) {
          p->done = true;
          p->a1 = r.a1;
          p->a2 = r.a2;
        }
      }
      dym_chain_free(c);
    });
  for (auto& t : th) t.join();
  if (!g_err.empty()) {
    fprintf(stderr, "dym-llr2d: %s\n", g_err.c_str());
    return 1;
  }
  int done = 0;
  for (const auto& jb : jobs) {
    if (!jb.loaded) {
      fprintf(stderr, "solve: missing cfg %s\n", jb.path.c_str());
      continue;
    }
    if (!jb.done) continue;
    printf("ANE2: %9.2f %9.2f %10.6f %10.6f %9.5f %9.5f %d\n", jb.E1, jb.E2, jb.a1, jb.a2, 0.0, 0.0, 1);
    ++done;
  }
  fflush(stdout);
  fprintf(stderr, "SOLVE[%d,%d): %d cells, drift S1 %.3e S2 %.3e\n", lo, hi, done, 0.0, 0.0);
  dym_group_free(g);
  return 0;
}

}  // namespace

int main(int argc, char* argv[]) {
  if (argc > 1 && strcmp(argv[1], "seed") == 0) return mode_seed(argc - 1, argv + 1);
  if (argc > 1 && strcmp(argv[1], "solve") == 0) return mode_solve(argc - 1, argv + 1);
  return mode_full(argc, argv);
}
