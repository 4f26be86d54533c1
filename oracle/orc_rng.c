/*
 * Oracle (test infrastructure only): random number generators.
 *
 * MT19937: Matsumoto & Nishimura (1998) with the 2002 `init_genrand` seeding,
 * which is what GSL's gsl_rng_mt19937 uses; GSL maps seed 0 to 4357 and
 * gsl_rng_uniform returns the 32-bit output divided by 2^32.  The reference
 * draws through src/common.c:133-164 (init_rng, rng_01, rng_delta_gauss).
 *
 * Philox4x32-10: Salmon, Moraes, Dror & Shaw, "Parallel random numbers: as
 * easy as 1, 2, 3" (SC'11).  Used by the production (counter-based) modes.
 */
#include "orc.h"

void orc_mt_seed(orc_mt *s, uint32_t seed)
{
  if (seed == 0) seed = 4357;
  s->mt[0] = seed;
  for (int i = 1; i < 624; i++)
    s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i;
  s->mti = 624;
}

uint32_t orc_mt_next(orc_mt *s)
{
  if (s->mti >= 624) {
    for (int k = 0; k < 624; k++) {
      uint32_t y = (s->mt[k] & 0x80000000u) | (s->mt[(k + 1) % 624] & 0x7fffffffu);
      s->mt[k] = s->mt[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    s->mti = 0;
  }
  uint32_t y = s->mt[s->mti++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

double orc_mt_uniform(orc_mt *s) { return orc_mt_next(s) / 4294967296.0; }

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
