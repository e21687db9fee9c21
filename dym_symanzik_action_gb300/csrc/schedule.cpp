// Race-free colour schedule for the checkerboard Metropolis sweep.
//
// The reference updates all links of direction d on sites of one parity at
// once (dym-mod-metro.cpp:152-159) and states that this is race-free
// (dym-mod-metro.cpp:21-23).  It is not: the rectangle staples of
// get_rect_loops (dym-mod-metro.cpp:83-142) read same-direction links at
// x +- 2 e_a and x +- e_d +- e_a, which have the parity of x.  This file builds
// a schedule whose phases are independent sets of the real read graph:
//
//   for link (x, d), same-direction links read are x + delta with
//   delta in {+-e_a, +-2e_a : a != d} u {+-e_d} u {+-e_d +- e_a : a != d}.
//
// Colouring: colour(x) = (sum_b w_b x_b) mod m with the smallest m and weights
// such that every delta that names another site (after periodic wrap) changes
// the colour, and N_b w_b = 0 mod m so the colouring is periodic.  For extents
// that are multiples of 4 this gives m = 4 (w_d = 2, w_a = 1): 4 phases per
// direction, which is optimal (x, x+e_d, x+e_a, x+e_d+e_a are pairwise
// conflicting).  Shapes with no linear colouring up to m = 24 fall back to a
// greedy colouring.  Every schedule is checked by brute force.
#include <algorithm>
#include <numeric>

#include "engine.h"

namespace dym {

namespace {

struct Shape {
  int D, Nt, Nx;
  int ext(int b) const { return b == 0 ? Nt : Nx; }
};

std::vector<std::vector<int>> conflict_offsets(int D, int d) {
  std::vector<std::vector<int>> out;
  auto add = [&](std::vector<int> v) { out.push_back(v); };
  for (int s = -1; s <= 1; s += 2) {
    std::vector<int> v(D, 0);
    v[d] = s;
    add(v);
  }
  for (int a = 0; a < D; ++a) {
    if (a == d) continue;
    for (int s : {-2, -1, 1, 2}) {
      std::vector<int> v(D, 0);
      v[a] = s;
      add(v);
    }
    for (int sd = -1; sd <= 1; sd += 2)
      for (int sa = -1; sa <= 1; sa += 2) {
        std::vector<int> v(D, 0);
        v[d] = sd;
        v[a] = sa;
        add(v);
      }
  }
  return out;
}

// An offset names the site itself when each component is 0 mod its extent.
bool is_self(const Shape& sh, const std::vector<int>& v) {
  for (int b = 0; b < sh.D; ++b)
    if (((v[b] % sh.ext(b)) + sh.ext(b)) % sh.ext(b) != 0) return false;
  return true;
}

bool try_linear(const Shape& sh, int d, int m, std::vector<int>* wout) {
  const int D = sh.D;
  auto offs = conflict_offsets(D, d);
  std::vector<std::vector<int>> need;
  for (auto& v : offs) if (!is_self(sh, v)) need.push_back(v);
  // Candidate weights per axis: periodic (N_b w_b = 0 mod m).
  std::vector<std::vector<int>> cand(D);
  for (int b = 0; b < D; ++b)
    for (int w = 0; w < m; ++w)
      if ((sh.ext(b) * w) % m == 0) cand[b].push_back(w);
  std::vector<int> w(D, 0), idx(D, 0);
  for (int b = 0; b < D; ++b) if (cand[b].empty()) return false;
  while (true) {
    for (int b = 0; b < D; ++b) w[b] = cand[b][idx[b]];
    bool ok = true;
    for (auto& v : need) {
      long s = 0;
      for (int b = 0; b < D; ++b) s += (long)w[b] * v[b];
      if (((s % m) + m) % m == 0) { ok = false; break; }
    }
    if (ok) { *wout = w; return true; }
    int b = 0;
    while (b < D && ++idx[b] == (int)cand[b].size()) { idx[b] = 0; ++b; }
    if (b == D) return false;
  }
}

// Greedy colouring of direction d's conflict graph, sites in index order.
int greedy(const Shape& sh, int d, uint32_t V, std::vector<int>* colour) {
  auto offs = conflict_offsets(sh.D, d);
  colour->assign(V, -1);
  int ncol = 0;
  std::vector<int> x(sh.D), y(sh.D);
  std::vector<char> used;
  for (uint32_t i = 0; i < V; ++i) {
    site_coords(i, sh.D, sh.Nt, sh.Nx, x.data());
    used.assign(ncol + 1, 0);
    for (auto& v : offs) {
      for (int b = 0; b < sh.D; ++b) y[b] = x[b] + v[b];
      uint32_t j = site_index(y.data(), sh.D, sh.Nt, sh.Nx);
      if (j != i && (*colour)[j] >= 0) used[(*colour)[j]] = 1;
    }
    int c = 0;
    while (used[c]) ++c;
    (*colour)[i] = c;
    ncol = std::max(ncol, c + 1);
  }
  return ncol;
}

}  // namespace

int schedule_build(int D, int Nt, int Nx, Schedule* s) {
  if (D < 2 || D > 4) return fail(DYM_ENOTSUP, "lattice dimension D must be 2, 3 or 4");
  if (Nt < 1 || Nx < 1) return fail(DYM_EINVAL, "lattice extents must be positive");
  uint64_t V64 = (uint64_t)Nt;
  for (int d = 1; d < D; ++d) V64 *= (uint64_t)Nx;
  if (V64 > (1ull << 31) / 8) return fail(DYM_ERANGE, "lattice volume too large");
  const uint32_t V = (uint32_t)V64;
  Shape sh{D, Nt, Nx};
  *s = Schedule();
  s->D = D; s->Nt = Nt; s->Nx = Nx; s->V = V;
  s->modulus.assign(D, 0);
  s->weights.assign(D, std::vector<int>(D, 0));
  std::vector<int> x(D);
  for (int d = 0; d < D; ++d) {
    std::vector<int> colour(V);
    int ncol = 0;
    std::vector<int> w;
    for (int m = 2; m <= 24; ++m) {
      if (try_linear(sh, d, m, &w)) { ncol = m; break; }
    }
    if (ncol) {
      s->modulus[d] = ncol;
      s->weights[d] = w;
      for (uint32_t i = 0; i < V; ++i) {
        site_coords(i, D, Nt, Nx, x.data());
        long c = 0;
        for (int b = 0; b < D; ++b) c += (long)w[b] * x[b];
        colour[i] = (int)(c % ncol);
      }
    } else {
      ncol = greedy(sh, d, V, &colour);
    }
    std::vector<std::vector<uint32_t>> lists(ncol);
    for (uint32_t i = 0; i < V; ++i) lists[colour[i]].push_back(i);
    for (int c = 0; c < ncol; ++c) {
      if (lists[c].empty()) continue;
      s->phase_dir.push_back(d);
      s->phase_off.push_back((uint32_t)s->sites.size());
      s->phase_len.push_back((uint32_t)lists[c].size());
      s->sites.insert(s->sites.end(), lists[c].begin(), lists[c].end());
    }
  }
  if (schedule_conflicts(*s) != 0) return fail(DYM_ENOTSUP, "internal: colour schedule has conflicts");
  return DYM_OK;
}

uint64_t schedule_conflicts(const Schedule& s) {
  const int D = s.D;
  std::vector<int> phase_of(s.V);
  std::vector<int> x(D), y(D);
  uint64_t bad = 0;
  for (size_t p = 0; p < s.phase_dir.size(); ++p) {
    const int d = s.phase_dir[p];
    for (uint32_t k = 0; k < s.phase_len[p]; ++k) phase_of[s.sites[s.phase_off[p] + k]] = (int)p;
  }
  for (size_t p = 0; p < s.phase_dir.size(); ++p) {
    const int d = s.phase_dir[p];
    auto offs = conflict_offsets(D, d);
    for (uint32_t k = 0; k < s.phase_len[p]; ++k) {
      uint32_t i = s.sites[s.phase_off[p] + k];
      site_coords(i, D, s.Nt, s.Nx, x.data());
      for (auto& v : offs) {
        for (int b = 0; b < D; ++b) y[b] = x[b] + v[b];
        uint32_t j = site_index(y.data(), D, s.Nt, s.Nx);
        if (j != i && phase_of[j] == (int)p) ++bad;
      }
    }
  }
  // Every (site, dir) must appear exactly once per sweep.
  std::vector<uint32_t> seen((size_t)s.V * D, 0);
  for (size_t p = 0; p < s.phase_dir.size(); ++p)
    for (uint32_t k = 0; k < s.phase_len[p]; ++k) ++seen[(size_t)s.phase_dir[p] * s.V + s.sites[s.phase_off[p] + k]];
  for (auto c : seen) if (c != 1) ++bad;
  return bad;
}

}  // namespace dym
