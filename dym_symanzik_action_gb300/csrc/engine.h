// Internal C++ interfaces of libdymgpu.  The public C ABI is include/dymgpu.h.
#pragma once
#include <stdint.h>
#include <stddef.h>
#include <string>
#include <vector>

#include "dymgpu.h"

namespace dym {

// Thread-local message behind dym_last_error().
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);

// ------------------------------------------------------------------ group --
// Host copy of a finite group loaded from a Cayley-table file, plus what the
// kernels derive from it.  Mirrors the globals of the reference's group.h:8-16
// (P, ReTr, ImTr, mult, inv, id) without the PMAX-sized static arrays.
struct Group {
  std::string path;
  uint32_t P = 0;
  uint32_t id = 0;
  std::vector<double> retr, imtr;
  std::vector<uint16_t> mult;  // row-major P*P, mult[n*P+m] = n*m
  std::vector<uint16_t> inv;
  // Proposal pools (dym-mod-metro.cpp:239-245 and "uniform over the group").
  std::vector<uint16_t> pool_nearest;
  double min_retr = 0, nn_retr = 0;
  // ReTr value clusters (tolerance 1e-9), sorted by value.  cls[n] is the
  // cluster of element n; cls_val[c] the ReTr of the cluster's first element.
  std::vector<uint8_t> cls;
  std::vector<double> cls_val;
  int ncls = 0;
  double cls_spread = 0;      // max |ReTr[n] - cls_val[cls[n]]|
  bool cls_exact = false;     // every cluster holds one bit pattern
  bool cls_conj_invariant = false;  // cluster label invariant under conjugation
  bool assoc_ok = false;      // sampled associativity check passed
  double max_abs_retr = 0;
  std::vector<uint16_t> gens;  // a small generating set
  // Device copies (owned; freed with the group).
  void* d_mult = nullptr;
  void* d_inv = nullptr;
  void* d_retr = nullptr;
  void* d_imtr = nullptr;
  void* d_cls = nullptr;
  void* d_cls16 = nullptr;     // the same classes as uint16
  void* d_clsval = nullptr;
  int device = -1;
};

int group_load(const char* path, Group** out);
int group_to_device(Group* g);
void group_free(Group* g);

// Chain checkpoint files (checkpoint.cpp): FNV-1a 64 of the Cayley table, and
// the file's writer and validating reader (links may be null: header only).
uint64_t table_hash(const Group& g);
int checkpoint_write(const char* path, const dym_checkpoint_info& h, const uint16_t* links);
int checkpoint_read(const char* path, dym_checkpoint_info* h, std::vector<uint16_t>* links);

// --------------------------------------------------------------- schedule --
// Race-free update order.  A link (x, d) update reads same-direction links at
// x +- e_a, x +- 2 e_a (a != d), x +- e_d and x +- e_d +- e_a (from the staple
// index sets of dym-mod-metro.cpp:63-142).  Phase p holds the sites of one
// direction whose links can be updated at once: no two of them read each other.
struct Schedule {
  int D = 0, Nt = 0, Nx = 0;
  uint32_t V = 0;
  std::vector<int> phase_dir;        // direction of phase p
  std::vector<uint32_t> phase_off;   // offset of phase p in `sites`
  std::vector<uint32_t> phase_len;
  std::vector<uint32_t> sites;       // concatenated site lists, ascending in a phase
  // Linear colouring per direction: colour = (sum_b w_b x_b) mod m, or m = 0
  // when the greedy fallback was used.
  std::vector<int> modulus;
  std::vector<std::vector<int>> weights;
};

int schedule_build(int D, int Nt, int Nx, Schedule* s);
// Number of same-phase pairs where one site's update reads the other's link;
// zero proves the schedule race-free.
uint64_t schedule_conflicts(const Schedule& s);

// Site index t + Nt*(x1 + Nx*(x2 + ...)) (lattice.c getidx/getpos).
inline void site_coords(uint32_t i, int D, int Nt, int Nx, int* x) {
  x[0] = (int)(i % (uint32_t)Nt);
  i /= (uint32_t)Nt;
  for (int d = 1; d < D; ++d) { x[d] = (int)(i % (uint32_t)Nx); i /= (uint32_t)Nx; }
}
inline uint32_t site_index(const int* x, int D, int Nt, int Nx) {
  uint32_t idx = 0;
  for (int d = D - 1; d > 0; --d) idx = (uint32_t)(((x[d] % Nx) + Nx) % Nx) + (uint32_t)Nx * idx;
  return (uint32_t)(((x[0] % Nt) + Nt) % Nt) + (uint32_t)Nt * idx;
}

}  // namespace dym
