// Host check of the sweep kernels' neighbour offsets (staples.cuh): the
// compare-and-select form site_geo_fast against the plain periodic wrap
// site_geo_xyz, every coordinate of every extent 1..40 (time) x 1..12
// (space, every fifth x3) and every extent up to 256 on one axis.  The
// header's device qualifiers are defined away; built and run by
// tests/test_site_geometry.py.
#include <cstdio>
#include <cstdint>
#define __device__
#define __host__
#define __forceinline__ inline
template <class T> T __ldg(const T* p) { return *p; }
#include "staples.cuh"
using namespace dym;
int main() {
  long bad = 0, n = 0;
  for (int Nt = 1; Nt <= 40; ++Nt) for (int Nx = 1; Nx <= 12; ++Nx) {
    for (int x0 = 0; x0 < Nt; ++x0) for (int x1 = 0; x1 < Nx; ++x1) for (int x2 = 0; x2 < Nx; x2 += 1) for (int x3 = 0; x3 < Nx; x3 += 5) {
      int x[4] = {x0, x1, x2, x3};
      uint32_t xyz = x0 | (x1 << 8) | (x2 << 16) | (x3 << 24);
      SiteGeo<4> a, b;
      site_geo_xyz<4>(x, Nt, Nx, a);
      site_geo_fast<4>(xyz, Nt, Nx, b);
      for (int d = 0; d < 4; ++d) for (int k = 0; k < 5; ++k) { ++n; if (a.off[d][k] != b.off[d][k]) { if (bad < 5) printf("Nt %d Nx %d x %d %d %d %d d %d k %d: %d vs %d\n", Nt, Nx, x0, x1, x2, x3, d, k, a.off[d][k], b.off[d][k]); ++bad; } }
    }
  }
  for (int N = 1; N <= 256; ++N) for (int x = 0; x < N; ++x) {  // one axis, all extents up to 256
    int xs[4] = {x, 0, 0, 0};
    SiteGeo<4> a, b;
    site_geo_xyz<4>(xs, N, 1, a);
    site_geo_fast<4>((uint32_t)x, N, 1, b);
    for (int k = 0; k < 5; ++k) { ++n; if (a.off[0][k] != b.off[0][k]) ++bad; }
  }
  printf("checked %ld offsets, %ld differ\n", n, bad);
  return bad != 0;
}
