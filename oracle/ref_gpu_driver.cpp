// The reference's own dym-mod-metro driver with its sweeps served by this
// engine: oracle/build_ref.sh streams dym-mod-metro.cpp through sed so that
// its two sweep loops (`for (k < NTHERM) update();`, dym-mod-metro.cpp:271, and
// `for (k < K) update();`, :278) become calls of dym_ref_sweeps below, and
// links the result with the reference's group.o, lattice.o, timer.o and
// libdymgpu.  Everything else -- argument parsing, table loading, the hot or
// cold start into its link array `a`, its measurements, its output lines and
// its timer -- is the reference's code, unchanged.  This is the binding a
// maintainer of the reference would add, built and tested.
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "dymgpu.h"
#include "lattice.h"  // the reference's globals: D, Nt, Nx, V, beta0..2 and the link array a

extern unsigned long hit, acc;  // the reference's running counters (dym-mod-metro.cpp:60)

// nsweeps sweeps of NHIT hits applied to the reference's link array `a` in
// place (dym_sweep_refarray), counters added to the reference's hit and acc.
// The chain (and the group tables on the device) are created on the first
// call from the reference's own arguments.
void dym_ref_sweeps(const char* groupfile, int iseed, unsigned nsweeps, int nhit) {
  static dym_group* g = nullptr;
  static dym_chain* c = nullptr;
  if (!c) {
    if (dym_group_load(groupfile, &g) != DYM_OK) {
      std::fprintf(stderr, "dym_group_load: %s\n", dym_last_error());
      std::exit(1);
    }
    dym_chain_params p{};
    p.D = (int32_t)D;
    p.Nt = (int32_t)Nt;
    p.Nx = (int32_t)Nx;
    p.beta0 = beta0;
    p.beta1 = beta1;
    p.beta2 = beta2;
    p.seed = (uint64_t)(uint32_t)iseed;
    p.start = DYM_START_COLD;  // replaced by `a` on every call
    p.pool = DYM_POOL_NEAREST;
    p.precision = DYM_PREC_MIXED;
    p.device = 0;
    if (dym_chain_create(g, &p, &c) != DYM_OK) {
      std::fprintf(stderr, "dym_chain_create: %s\n", dym_last_error());
      std::exit(1);
    }
  }
  dym_stats st;
  if (dym_sweep_refarray(c, reinterpret_cast<int32_t*>(a), (int32_t)nsweeps, nhit, &st) != DYM_OK) {
    std::fprintf(stderr, "dym_sweep_refarray: %s\n", dym_last_error());
    std::exit(1);
  }
  hit += st.hits;
  acc += st.accepts;
}
