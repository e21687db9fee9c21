// Group-table loader and the per-group facts the kernels need.
//
// File format and parse order follow the reference loader (group.c:13-65):
// the order P, P values of ReTr, P of ImTr, then the P*P Cayley table; any
// trailing tokens are ignored.  The identity is the first n whose row and column
// are the identity permutation, and inv[n] the first m with n*m = m*n = id
// (group.c:67-98).  Where the reference aborts (no identity, no inverse, P >
// PMAX) this loader returns an error code instead; it also rejects truncated
// files and out-of-range entries, which the reference reads as garbage.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>

#include "engine.h"

namespace dym {

namespace {

struct Tokenizer {
  const char* p;
  const char* end;
  void skip() {
    while (p < end && (*p == ' ' || *p == '\n' || *p == '\t' || *p == '\r' || *p == '\f' || *p == '\v')) ++p;
  }
  bool next_long(long* v) {
    skip();
    if (p >= end) return false;
    char* e = nullptr;
    errno = 0;
    long x = strtol(p, &e, 10);
    if (e == p || errno) return false;
    // The reference reads with %d, which stops at the first non-digit; a token
    // such as "3.0" would desynchronise its parse.  Require a clean token.
    if (e < end && !(*e == ' ' || *e == '\n' || *e == '\t' || *e == '\r' || *e == '\f' || *e == '\v'))
      return false;
    p = e;
    *v = x;
    return true;
  }
  bool next_double(double* v) {
    skip();
    if (p >= end) return false;
    char* e = nullptr;
    double x = strtod(p, &e);
    if (e == p) return false;
    p = e;
    *v = x;
    return true;
  }
};

bool read_file(const char* path, std::string* buf) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  char tmp[1 << 16];
  size_t n;
  while ((n = fread(tmp, 1, sizeof tmp, f)) > 0) buf->append(tmp, n);
  bool ok = !ferror(f);
  fclose(f);
  return ok;
}

// Subgroup generated by `gens` (BFS by right multiplication).
size_t closure_size(const Group& g, const std::vector<uint16_t>& gens, std::vector<uint8_t>* seen) {
  seen->assign(g.P, 0);
  std::vector<uint32_t> q{g.id};
  (*seen)[g.id] = 1;
  for (size_t h = 0; h < q.size(); ++h) {
    for (uint16_t s : gens) {
      uint32_t x = g.mult[(size_t)q[h] * g.P + s];
      if (!(*seen)[x]) { (*seen)[x] = 1; q.push_back(x); }
    }
  }
  return q.size();
}

void analyse(Group& g) {
  const uint32_t P = g.P;
  // Proposal pool "nearest the identity", exactly as dym-mod-metro.cpp:239-243
  // (including the initial values 0 and 10 of min_retr and nn_retr).
  double min_retr = 0, nn_retr = 10;
  for (uint32_t i = 0; i < P; ++i) if (g.retr[i] < min_retr) min_retr = g.retr[i];
  for (uint32_t i = 0; i < P; ++i) if (g.retr[i] > min_retr && g.retr[i] < nn_retr) nn_retr = g.retr[i];
  g.pool_nearest.clear();
  for (uint32_t i = 0; i < P; ++i)
    if (g.retr[i] < nn_retr + 1e-6 && g.retr[i] > min_retr) g.pool_nearest.push_back((uint16_t)i);
  g.min_retr = min_retr;
  g.nn_retr = nn_retr;

  // ReTr value clusters.
  std::vector<uint32_t> order(P);
  for (uint32_t i = 0; i < P; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return g.retr[a] < g.retr[b]; });
  g.cls.assign(P, 0);
  g.cls_val.clear();
  double last = 0;
  for (uint32_t k = 0; k < P; ++k) {
    uint32_t i = order[k];
    if (k == 0 || g.retr[i] - last > 1e-9) {
      g.cls_val.push_back(g.retr[i]);
      last = g.retr[i];
    }
    g.cls[i] = (uint8_t)std::min<size_t>(g.cls_val.size() - 1, 255);
  }
  g.ncls = (int)g.cls_val.size();
  // Representative value: the ReTr of the lowest-numbered element of the class.
  std::vector<int> rep(g.ncls, -1);
  for (uint32_t i = 0; i < P; ++i) if (rep[g.cls[i]] < 0) rep[g.cls[i]] = (int)i;
  for (int c = 0; c < g.ncls; ++c) g.cls_val[c] = g.retr[rep[c]];
  g.cls_spread = 0;
  g.cls_exact = true;
  g.max_abs_retr = 0;
  for (uint32_t i = 0; i < P; ++i) {
    double dv = std::fabs(g.retr[i] - g.cls_val[g.cls[i]]);
    g.cls_spread = std::max(g.cls_spread, dv);
    if (std::memcmp(&g.retr[i], &g.cls_val[g.cls[i]], sizeof(double)) != 0) g.cls_exact = false;
    g.max_abs_retr = std::max(g.max_abs_retr, std::fabs(g.retr[i]));
  }
  if (g.ncls > 255) g.cls_exact = false;

  // Greedy generating set.
  g.gens.clear();
  std::vector<uint8_t> seen;
  size_t have = closure_size(g, g.gens, &seen);
  for (uint32_t x = 0; x < P && have < P; ++x) {
    if (seen[x]) continue;
    g.gens.push_back((uint16_t)x);
    have = closure_size(g, g.gens, &seen);
  }
  // Cluster label invariant under conjugation by the generators => invariant
  // under the whole group (labels are exact integers, so nothing accumulates).
  g.cls_conj_invariant = (g.ncls <= 255);
  for (uint16_t h : g.gens) {
    uint32_t hi = g.inv[h];
    for (uint32_t x = 0; x < P && g.cls_conj_invariant; ++x) {
      uint32_t y = g.mult[(size_t)g.mult[(size_t)hi * P + x] * P + h];
      if (g.cls[y] != g.cls[x]) g.cls_conj_invariant = false;
    }
  }
  // Sampled associativity (xorshift64, as in the reference's verify_group).
  g.assoc_ok = true;
  uint64_t s = 88172645463325252ull;
  const uint64_t nchk = std::min<uint64_t>((uint64_t)P * P * P, 300000);
  for (uint64_t t = 0; t < nchk; ++t) {
    uint32_t v[3];
    for (int r = 0; r < 3; ++r) {
      s ^= s << 13; s ^= s >> 7; s ^= s << 17;
      v[r] = (uint32_t)((s >> 3) % P);
    }
    uint32_t l = g.mult[(size_t)g.mult[(size_t)v[0] * P + v[1]] * P + v[2]];
    uint32_t r = g.mult[(size_t)v[0] * P + g.mult[(size_t)v[1] * P + v[2]]];
    if (l != r) { g.assoc_ok = false; break; }
  }
}

}  // namespace

int group_load(const char* path, Group** out) {
  if (!path || !out) return fail(DYM_EINVAL, "dym_group_load: null argument");
  *out = nullptr;
  std::string buf;
  if (!read_file(path, &buf)) return fail(DYM_EIO, std::string("cannot read group file ") + path);
  Tokenizer tk{buf.data(), buf.data() + buf.size()};
  long P = 0;
  if (!tk.next_long(&P) || P <= 0) return fail(DYM_EFORMAT, "group file: bad order token");
  if (P > DYM_PMAX)
    return fail(DYM_ERANGE, "Order of group too large: " + std::to_string(P) + " > " + std::to_string(DYM_PMAX));
  std::unique_ptr<Group> g(new Group);
  g->path = path;
  g->P = (uint32_t)P;
  g->retr.resize(P);
  g->imtr.resize(P);
  for (long n = 0; n < P; ++n)
    if (!tk.next_double(&g->retr[n])) return fail(DYM_EFORMAT, "group file: truncated ReTr row");
  for (long n = 0; n < P; ++n)
    if (!tk.next_double(&g->imtr[n])) return fail(DYM_EFORMAT, "group file: truncated ImTr row");
  g->mult.resize((size_t)P * P);
  for (size_t k = 0; k < (size_t)P * P; ++k) {
    long v;
    if (!tk.next_long(&v)) return fail(DYM_EFORMAT, "group file: truncated or non-integer Cayley table");
    if (v < 0 || v >= P)
      return fail(DYM_EFORMAT, "group file: mult[" + std::to_string(k / P) + "][" + std::to_string(k % P) +
                                   "]=" + std::to_string(v) + " out of range");
    g->mult[k] = (uint16_t)v;
  }
  // Identity (group.c:67-83).
  bool found = false;
  for (uint32_t n = 0; n < (uint32_t)P && !found; ++n) {
    bool is_id = true;
    for (uint32_t m = 0; m < (uint32_t)P; ++m)
      if (g->mult[(size_t)n * P + m] != m || g->mult[(size_t)m * P + n] != m) { is_id = false; break; }
    if (is_id) { g->id = n; found = true; }
  }
  if (!found) return fail(DYM_EFORMAT, "Group does not have identity element");
  // Inverses (group.c:85-98).
  g->inv.resize(P);
  for (uint32_t n = 0; n < (uint32_t)P; ++n) {
    bool ok = false;
    for (uint32_t m = 0; m < (uint32_t)P; ++m)
      if (g->mult[(size_t)n * P + m] == g->id && g->mult[(size_t)m * P + n] == g->id) {
        g->inv[n] = (uint16_t)m;
        ok = true;
        break;
      }
    if (!ok) return fail(DYM_EFORMAT, "Group does not have inverses");
  }
  analyse(*g);
  *out = g.release();
  return DYM_OK;
}

}  // namespace dym
