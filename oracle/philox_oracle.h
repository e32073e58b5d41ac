/* Oracle (test infrastructure only): Philox4x32-10 counter-based RNG and the
   draw contract that replaces RandomPark in the parity oracle.

   Philox4x32-10 is the published algorithm of Salmon, Moraes, Dror and Shaw,
   "Parallel random numbers: as easy as 1, 2, 3" (SC'11): a 4x32-bit counter
   and a 2x32-bit key, ten rounds of two 32x32->64 multiplies with the
   constants 0xD2511F53 / 0xCD9E8D57 and a Weyl key schedule 0x9E3779B9 /
   0xBB67AE85.  This file is the oracle's own copy; the product has an
   independent one, and the tests check both against the published
   known-answer vectors.

   Draw contract (the oracle and the GPU path must agree on it):
     key      = { (uint32) seed, stream_base | stream }
     stream   0 = rejection sweeps, 1 = KMC events, 2 = replica exchange,
              3 = initial spins; stream_base = 0 for a single lattice and
              (r+1) << 8 for replica r of an ensemble
     replica exchange round k, group g, slot pair j:
       counter = { k, g, j, 0 }, word 0
     rejection sweep, site s = id-1 (0-based), sweep n, pass p within sweep:
       potts, potts/neighonly, potts/neigh: counter = { s>>1 (low 32), s>>33,
       n, p }, draw d of site s uses word 2*(s&1)+d  (two sites share one
       Philox block; d is 0 or 1)
       ising: counter = { s>>2 (low 32), s>>34, n, p }, site s takes the one
       word x = word s&3 (four sites share one block); draw 0 is
       u0 = (2*(x>>31) + 1) / 4 and draw 1 is u1 = ((x & 0x7FFFFFFF) + 1) 2^-31
     KMC event k of chain c:  counter = { c, k low, k high, 0 }; word 0 is
       the tree pick, word 1 the clock, word 2 the event choice
     initial spin of site s: counter = { s>>1, s>>33, 0, 0 }, word 2*(s&1)
   A draw x becomes the RandomPark::uniform() value u = (x+1) * 2^-32,
   which is exact in double and lies in (0,1].
*/
#ifndef SPK_PHILOX_ORACLE_H
#define SPK_PHILOX_ORACLE_H

#include <stdint.h>

#define SPKO_STREAM_SWEEP 0u
#define SPKO_STREAM_KMC 1u
#define SPKO_STREAM_EXCHANGE 2u
#define SPKO_STREAM_INIT 3u

static inline void spko_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                                      uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

/* the two draws of site s in sweep n, pass p (apps other than ising) */
static inline void spko_site_draws(uint32_t seed, uint32_t stream_base, uint64_t s, uint32_t sweep,
                                   uint32_t pass, uint32_t *x0, uint32_t *x1) {
  uint32_t ctr[4] = {(uint32_t)(s >> 1), (uint32_t)(s >> 33), sweep, pass};
  uint32_t key[2] = {seed, stream_base | SPKO_STREAM_SWEEP};
  uint32_t w[4];
  spko_philox4x32_10(ctr, key, w);
  int h = (int)(s & 1) * 2;
  *x0 = w[h];
  *x1 = w[h + 1];
}

/* the one word of ising site s in sweep n, pass p */
static inline uint32_t spko_ising_word(uint32_t seed, uint32_t stream_base, uint64_t s, uint32_t sweep,
                                       uint32_t pass) {
  uint32_t ctr[4] = {(uint32_t)(s >> 2), (uint32_t)(s >> 34), sweep, pass};
  uint32_t key[2] = {seed, stream_base | SPKO_STREAM_SWEEP};
  uint32_t w[4];
  spko_philox4x32_10(ctr, key, w);
  return w[s & 3];
}

/* the ising site's two uniforms from its word: the proposal from the top bit,
   the Boltzmann draw from the low 31 bits (both exact in double) */
static inline double spko_ising_u0(uint32_t x) { return (2.0 * (double)(x >> 31) + 1.0) * 0.25; }
static inline double spko_ising_u1(uint32_t x) {
  return ((double)(x & 0x7FFFFFFFu) + 1.0) * (1.0 / 2147483648.0);
}

static inline void spko_kmc_draws(uint32_t seed, uint32_t chain, uint64_t k, uint32_t w[4]) {
  uint32_t ctr[4] = {chain, (uint32_t)k, (uint32_t)(k >> 32), 0};
  uint32_t key[2] = {seed, SPKO_STREAM_KMC};
  spko_philox4x32_10(ctr, key, w);
}

/* initial spin of site s, uniform in lo..hi */
static inline int spko_init_spin(uint32_t seed, uint64_t s, int lo, int hi) {
  uint32_t ctr[4] = {(uint32_t)(s >> 1), (uint32_t)(s >> 33), 0, 0};
  uint32_t key[2] = {seed, SPKO_STREAM_INIT};
  uint32_t w[4];
  spko_philox4x32_10(ctr, key, w);
  uint32_t x = w[(s & 1) * 2];
  uint64_t range = (uint64_t)(hi - lo + 1);
  return lo + (int)((range * (uint64_t)x) >> 32);
}

static inline double spko_u(uint32_t x) { return ((double)x + 1.0) * (1.0 / 4294967296.0); }

#endif
