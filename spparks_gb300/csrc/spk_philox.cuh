// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11) for host and device, and the draw contract that
// replaces RandomPark::uniform (src/random_park.cpp:79-86) on the GPU path.
//
// Draw contract
//   key      = { seed, stream }; stream 0 = rejection sweeps, 1 = KMC events,
//              2 = replica exchange, 3 = initial spins
//   sweep:   site s (= id-1), sweep n, pass p (0..nloop-1 within the sweep)
//            potts, potts/neighonly, potts/neigh: counter = { s>>1, s>>33,
//            n, p }; draw d of site s is word 2*(s&1)+d, so the two sites of
//            an x-pair share one block
//            ising: counter = { s>>2, s>>34, n, p }; site s takes the one
//            word x = word s&3, so four sites share one block.  Its proposal
//            is the top bit and its Boltzmann draw the low 31 bits:
//              draw 0 u0 = (2*(x>>31) + 1) / 4        (u0 < 0.5 <=> x < 2^31)
//              draw 1 u1 = ((x & 0x7FFFFFFF) + 1) * 2^-31
//            u1 has the 31-bit resolution of RandomPark's own values
//   KMC:     event k of chain c: counter = { c, k, k>>32, 0 }; word 0 picks
//            the tree leaf, word 1 is the clock, word 2 the event choice
//   init:    site s: counter = { s>>1, s>>33, 0, 0 }, word 2*(s&1)
//   A word x stands for the uniform u = (x+1) * 2^-32 in (0,1], exact in
//   double, so every test the reference makes on u is an integer test on x:
//     u < 0.5                 <=>  x < 2^31 - 1
//     (int)(Q*u)              ==   (Q*(x+1)) >> 32        (Q < 2^21)
//     u > exp(-dE/T) (reject) <=>  x >= floor(exp(-dE/T) * 2^32)
//   and for the Ising split, with y = x & 0x7FFFFFFF,
//     u1 > exp(-dE/T) (reject) <=> y >= floor(exp(-dE/T) * 2^31)
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define SPK_HD __host__ __device__ __forceinline__
#else
#define SPK_HD inline
#endif

namespace spk {

constexpr uint32_t kPhiloxM0 = 0xD2511F53u;
constexpr uint32_t kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u;
constexpr uint32_t kPhiloxW1 = 0xBB67AE85u;

constexpr uint32_t kStreamSweep = 0;
constexpr uint32_t kStreamKmc = 1;
constexpr uint32_t kStreamExchange = 2;
constexpr uint32_t kStreamInit = 3;

struct U4 {
  uint32_t x, y, z, w;
};

// one 32x32->64 multiply (a single IMAD.WIDE.U32 on the device)
SPK_HD void mulhilo(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
  uint64_t p = (uint64_t)a * b;
  lo = (uint32_t)p;
  hi = (uint32_t)(p >> 32);
}

SPK_HD U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
  for (int r = 0; r < 10; r++) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo(kPhiloxM0, c.x, hi0, lo0);
    mulhilo(kPhiloxM1, c.z, hi1, lo1);
    U4 n;
    n.x = hi1 ^ c.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ c.w ^ k1;
    n.w = lo0;
    c = n;
    k0 += kPhiloxW0;
    k1 += kPhiloxW1;
  }
  return c;
}

// the ten round keys of a key, for callers that draw many blocks with one key
struct RoundKeys {
  uint32_t k0[10], k1[10];
};

SPK_HD RoundKeys round_keys(uint32_t k0, uint32_t k1) {
  RoundKeys r;
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
  for (int i = 0; i < 10; i++) {
    r.k0[i] = k0;
    r.k1[i] = k1;
    k0 += kPhiloxW0;
    k1 += kPhiloxW1;
  }
  return r;
}

SPK_HD U4 philox4x32_10_rk(U4 c, const RoundKeys &rk) {
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
  for (int r = 0; r < 10; r++) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo(kPhiloxM0, c.x, hi0, lo0);
    mulhilo(kPhiloxM1, c.z, hi1, lo1);
    U4 n;
    n.x = hi1 ^ c.y ^ rk.k0[r];
    n.y = lo1;
    n.z = hi0 ^ c.w ^ rk.k1[r];
    n.w = lo0;
    c = n;
  }
  return c;
}

constexpr uint32_t kIsingProposal1 = 0x80000000u;  // x below it proposes value 1
constexpr uint32_t kIsingAcceptMask = 0x7FFFFFFFu;  // the Boltzmann draw of x

// counter of the Philox block holding the word of Ising site s
SPK_HD U4 ising_counter(uint64_t s, uint32_t sweep, uint32_t pass) {
  return U4{(uint32_t)(s >> 2), (uint32_t)(s >> 34), sweep, pass};
}

// word k (0..3) of a block
SPK_HD uint32_t block_word(const U4 &w, int k) { return k == 0 ? w.x : (k == 1 ? w.y : (k == 2 ? w.z : w.w)); }

SPK_HD U4 kmc_block(uint32_t seed, uint32_t chain, uint64_t k) {
  U4 c{chain, (uint32_t)k, (uint32_t)(k >> 32), 0u};
  return philox4x32_10(c, seed, kStreamKmc);
}

SPK_HD int init_spin(uint32_t seed, uint64_t s, int lo, int hi) {
  U4 c{(uint32_t)(s >> 1), (uint32_t)(s >> 33), 0u, 0u};
  U4 w = philox4x32_10(c, seed, kStreamInit);
  uint32_t x = (s & 1) ? w.z : w.x;
  uint64_t range = (uint64_t)(hi - lo + 1);
  return lo + (int)((range * (uint64_t)x) >> 32);
}

// floor(n * u) for u = (x+1) 2^-32, n < 2^21 (RandomPark-style integer pick)
SPK_HD uint32_t scaled_pick(uint32_t n, uint32_t x) {
  return (uint32_t)(((uint64_t)n * ((uint64_t)x + 1u)) >> 32);
}

// u = (x+1) 2^-32 as a double (KMC tree pick and clock)
SPK_HD double word_to_uniform(uint32_t x) { return ((double)x + 1.0) * (1.0 / 4294967296.0); }

}  // namespace spk
