/* Host check of dym_metro_hit (dym_core.h): the Metropolis hit draws with the
 * per-link half of the first two Philox rounds precomputed and the round keys
 * from dym_philox_round_keys equal dym_hit_random for 2,000,000 pseudo-random
 * (seed, sweep, site, dir, hit, tag) tuples, including hit indices at and
 * beyond the 20-bit field.  Built and run by tests/test_philox_split.py. */
#include <stdint.h>
#include <stdio.h>

#include "dym_core.h"

static uint64_t sm64(uint64_t* s) {  /* splitmix64 */
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

int main(void) {
  uint64_t st = 12345;
  long bad = 0, n = 0;
  const uint32_t tags[3] = {DYM_TAG_METRO, DYM_TAG_LLR, DYM_TAG_HOT};
  for (int t = 0; t < 20000; ++t) {
    const uint64_t seed = sm64(&st);
    uint32_t rk[20];
    dym_philox_round_keys(seed, rk);
    const uint32_t sweep = (uint32_t)sm64(&st), site = (uint32_t)sm64(&st), dir = (uint32_t)(sm64(&st) % 4);
    const uint32_t tag = tags[t % 3];
    const dym_metro_link L = dym_metro_link_init(rk, sweep, site, dir, tag);
    for (int h = 0; h < 100; ++h) {
      const uint32_t hit = h < 50 ? (uint32_t)h : (uint32_t)sm64(&st);
      const dym_u32x4 a = dym_hit_random(seed, sweep, site, dir, hit, tag);
      const dym_u32x4 b = dym_metro_hit(rk, L, hit);
      ++n;
      if (a.v[0] != b.v[0] || a.v[1] != b.v[1] || a.v[2] != b.v[2] || a.v[3] != b.v[3]) ++bad;
    }
  }
  printf("checked %ld draws, %ld differ\n", n, bad);
  return bad != 0;
}
