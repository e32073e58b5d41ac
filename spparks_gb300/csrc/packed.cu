// Bit-packed (multispin) Ising on sc/6n: 64 sites per uint64, bit b of word
// (w, y, z) holds site x = 64w + b as (value - 1).  Same per-site rule and
// Philox draws as the int8/int16/int32 path (AppIsing::site_event_rejection,
// src/app_ising.cpp:104-136; colours of Lattice::id2color SC_6N,
// src/lattice.cpp:256-260), so the lattices are bit-identical.
//
// Per sweep:
//   packed_draw_kernel   one thread per word computes the Philox blocks of
//                        its 64 sites (16 blocks, four sites each) once and
//                        stores three decision masks: the proposal (a site
//                        word x >= 2^31 proposes value 2) and the level of
//                        y = x & 0x7FFFFFFF among the thresholds of the
//                        three uphill moves dE = 2, 4, 6 (t2 >= t4 >= t6) as
//                        two bit planes: hi = [y < t4], lo = [y < t6] where
//                        hi is set and [y < t2] where it is not.  Then
//                        [y < t2] = hi | lo, [y < t4] = hi and
//                        [y < t6] = hi & lo.  A site takes two compares, one
//                        select and three predicated ORs.
//   packed_phase_kernel  per colour, one thread per word: the unlike count of
//                        every site against its six neighbours as a
//                        bit-sliced 3-bit sum of XOR masks; a site of the
//                        colour flips when its proposal differs from it and
//                        e0 >= 3 (dE <= 0) or the decision for
//                        dE = 6 - 2*e0 holds.  Words are updated in place:
//                        a colour's bits never neighbour each other, so
//                        concurrent readers only use bits that do not change.

#include <cuda_runtime.h>
#include <stdint.h>

#include "counters.cuh"
#include "site_update.cuh"
#include "spk_internal.h"

namespace spk {

// the three decision planes of nw words, one array each (coalesced loads)
struct PackedPlanes {
  uint64_t *prop, *hi, *lo;
};
__host__ __device__ inline PackedPlanes packed_planes(void *decisions, int64_t nw) {
  uint64_t *d = (uint64_t *)decisions;
  return PackedPlanes{d, d + nw, d + 2 * nw};
}

// c | BIT if x >= 2^31 (the site's word proposes value 2), as a compare and
// a predicated OR of an immediate
template <uint32_t BIT>
__device__ __forceinline__ uint32_t or_if_prop2(uint32_t c, uint32_t x) {
  asm("{\n\t.reg .pred q;\n\tsetp.ge.u32 q, %1, 0x80000000;\n\t@q or.b32 %0, %0, %2;\n\t}"
      : "+r"(c)
      : "r"(x), "n"(BIT));
  return c;
}

// c | BIT if x < t
template <uint32_t BIT>
__device__ __forceinline__ uint32_t or_if_below(uint32_t c, uint32_t x, uint32_t t) {
  asm("{\n\t.reg .pred q;\n\tsetp.lt.u32 q, %1, %2;\n\t@q or.b32 %0, %0, %3;\n\t}"
      : "+r"(c)
      : "r"(x), "r"(t), "n"(BIT));
  return c;
}

// the three decision planes of a word, as 32-bit halves (index 0: bits 0-31)
struct PackedHalves {
  uint32_t prop[2], hi[2], lo[2];
};

// the decision bits BIT of one site with Philox word x
template <uint32_t BIT, int H>
__device__ __forceinline__ void packed_site(PackedHalves &h, uint32_t x, uint32_t t2, uint32_t t4, uint32_t t6) {
  h.prop[H] = or_if_prop2<BIT>(h.prop[H], x);
  const uint32_t y = x & kIsingAcceptMask;
  const bool below4 = y < t4;
  if (below4) h.hi[H] |= BIT;
  h.lo[H] = or_if_below<BIT>(h.lo[H], y, below4 ? t6 : t2);
}

// block M (sites 4M .. 4M+3 of the word) and the blocks after it; the block
// index is a template argument so that every mask bit is an immediate
template <int M>
__device__ __forceinline__ void packed_blocks(U4 ctr, const RoundKeys &rk, uint32_t t2, uint32_t t4, uint32_t t6,
                                              PackedHalves &h) {
  if constexpr (M < 16) {
    const U4 q = philox4x32_10_rk(U4{ctr.x + (uint32_t)M, ctr.y, ctr.z, ctr.w}, rk);
    constexpr int H = M >> 3;
    constexpr uint32_t B = 1u << (4 * (M & 7));
    packed_site<B, H>(h, q.x, t2, t4, t6);
    packed_site<(B << 1), H>(h, q.y, t2, t4, t6);
    packed_site<(B << 2), H>(h, q.z, t2, t4, t6);
    packed_site<(B << 3), H>(h, q.w, t2, t4, t6);
    packed_blocks<M + 1>(ctr, rk, t2, t4, t6, h);
  }
}

// Every threshold is at most 2^31, so the tests are 32-bit compares.  The
// word's first site s0 is a multiple of 64, so the block counters
// (s0 >> 2) + M never carry.
__global__ void __launch_bounds__(256, 4) packed_draw_kernel(const PackedArgs a) {
  const int64_t nw = a.nwords;
  const int64_t words_per_row = a.nx >> 6;
  const RoundKeys rk = round_keys(a.seed, kStreamSweep);
  const uint32_t t2 = (uint32_t)a.thr2, t4 = (uint32_t)a.thr4, t6 = (uint32_t)a.thr6;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nw; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = t / words_per_row;
    const int64_t s0 = row * a.nx + ((t - row * words_per_row) << 6);  // site of bit 0
    PackedHalves h = {};
    packed_blocks<0>(ising_counter((uint64_t)s0, a.sweep, 0u), rk, t2, t4, t6, h);
    const PackedPlanes D = packed_planes(a.decisions, nw);
    D.prop[t] = (uint64_t)h.prop[1] << 32 | h.prop[0];
    D.hi[t] = (uint64_t)h.hi[1] << 32 | h.hi[0];
    D.lo[t] = (uint64_t)h.lo[1] << 32 | h.lo[0];
  }
}

__global__ void packed_phase_kernel(const PackedArgs a, int color) {
  uint64_t *W = (uint64_t *)a.words;
  int64_t words_per_row = a.nx >> 6;
  int64_t nw = a.nwords;
  const PackedPlanes D = packed_planes(a.decisions, nw);
  unsigned long long flips = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nw; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t row = t / words_per_row;
    int w = (int)(t - row * words_per_row);
    int y = (int)(row % a.ny);
    int z = (int)(row / a.ny);
    // colour of bit b: (x + y + z) even -> colour 1; x parity = bit parity
    uint64_t cmask = (((color - 1 + y + z) & 1) == 0) ? 0x5555555555555555ull : 0xAAAAAAAAAAAAAAAAull;
    uint64_t s = W[t];
    int wm = w == 0 ? (int)words_per_row - 1 : w - 1;
    int wp = w == (int)words_per_row - 1 ? 0 : w + 1;
    uint64_t xm = (s << 1) | (W[row * words_per_row + wm] >> 63);
    uint64_t xp = (s >> 1) | (W[row * words_per_row + wp] << 63);
    int ym = y == 0 ? a.ny - 1 : y - 1, yp = y == a.ny - 1 ? 0 : y + 1;
    int zm = z == 0 ? a.nz - 1 : z - 1, zp = z == a.nz - 1 ? 0 : z + 1;
    uint64_t nym = W[((int64_t)z * a.ny + ym) * words_per_row + w];
    uint64_t nyp = W[((int64_t)z * a.ny + yp) * words_per_row + w];
    uint64_t nzm = W[((int64_t)zm * a.ny + y) * words_per_row + w];
    uint64_t nzp = W[((int64_t)zp * a.ny + y) * words_per_row + w];
    // bit-sliced count of unlike neighbours: e0 = b2 b1 b0 (0..6)
    uint64_t d[6] = {s ^ xm, s ^ nym, s ^ nyp, s ^ nzm, s ^ nzp, s ^ xp};
    uint64_t b0 = 0, b1 = 0, b2 = 0;
#pragma unroll
    for (int j = 0; j < 6; j++) {
      uint64_t c0 = b0 & d[j];
      b0 ^= d[j];
      uint64_t c1 = b1 & c0;
      b1 ^= c0;
      b2 |= c1;
    }
    const uint64_t hi = D.hi[t], lo = D.lo[t];
    uint64_t ge3 = b2 | (b1 & b0);                 // e0 >= 3: downhill or level
    uint64_t e2 = ~b2 & b1 & ~b0;                  // dE = 2: y < t2
    uint64_t e1 = ~b2 & ~b1 & b0;                  // dE = 4: y < t4
    uint64_t e0z = ~b2 & ~b1 & ~b0;                // dE = 6: y < t6
    uint64_t accept = ge3 | (e2 & (hi | lo)) | (e1 & hi) | (e0z & hi & lo);
    uint64_t flip = (D.prop[t] ^ s) & cmask & accept;
    if (flip) W[t] = s ^ flip;
    flips += __popcll(flip);
  }
  block_count_add(a.naccept, flips);
}

// int32 site values (1 or 2) -> bits; sets *bad on any other value
__global__ void packed_pack_kernel(const int32_t *src, uint64_t *dst, int64_t nwords, int *bad) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nwords; t += (int64_t)gridDim.x * blockDim.x) {
    uint64_t v = 0;
    const int32_t *p = src + (t << 6);
    for (int b = 0; b < 64; b++) {
      int s = p[b];
      if (s < 1 || s > 2) *bad = 1;
      v |= (uint64_t)(s == 2) << b;
    }
    dst[t] = v;
  }
}

__global__ void packed_unpack_kernel(const uint64_t *src, int32_t *dst, int64_t nwords) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nwords; t += (int64_t)gridDim.x * blockDim.x) {
    uint64_t v = src[t];
    int32_t *p = dst + (t << 6);
    for (int b = 0; b < 64; b++) p[b] = 1 + (int)((v >> b) & 1);
  }
}

// total energy: sum over sites of unlike neighbours = 2 * unlike bonds
__global__ void packed_energy_kernel(const uint64_t *W, int nx, int ny, int nz, int64_t nwords,
                                     unsigned long long *out) {
  int64_t words_per_row = nx >> 6;
  unsigned long long e = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nwords; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t row = t / words_per_row;
    int w = (int)(t - row * words_per_row);
    int y = (int)(row % ny), z = (int)(row / ny);
    uint64_t s = W[t];
    int wp = w == (int)words_per_row - 1 ? 0 : w + 1;
    uint64_t xp = (s >> 1) | (W[row * words_per_row + wp] << 63);
    int yp = y == ny - 1 ? 0 : y + 1, zp = z == nz - 1 ? 0 : z + 1;
    uint64_t nyp = W[((int64_t)z * ny + yp) * words_per_row + w];
    uint64_t nzp = W[((int64_t)zp * ny + y) * words_per_row + w];
    e += 2ull * (__popcll(s ^ xp) + __popcll(s ^ nyp) + __popcll(s ^ nzp));
  }
  for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xFFFFFFFFu, e, o);
  if ((threadIdx.x & 31) == 0 && e) atomicAdd(out, e);
}

static unsigned grid_for(int64_t n, int sms, int per_sm = 8) {
  int64_t b = (n + 255) / 256;
  int64_t cap = (int64_t)sms * per_sm;
  return (unsigned)(b < cap ? (b > 0 ? b : 1) : cap);
}

cudaError_t launch_packed_sweep(const PackedArgs &a, cudaStream_t s, int num_sms) {
  packed_draw_kernel<<<grid_for(a.nwords, num_sms), 256, 0, s>>>(a);
  packed_phase_kernel<<<grid_for(a.nwords, num_sms), 256, 0, s>>>(a, 1);
  packed_phase_kernel<<<grid_for(a.nwords, num_sms), 256, 0, s>>>(a, 2);
  return cudaGetLastError();
}

cudaError_t launch_packed_pack(const int32_t *src, uint64_t *dst, int64_t nwords, int *bad, cudaStream_t s, int num_sms) {
  packed_pack_kernel<<<grid_for(nwords, num_sms), 256, 0, s>>>(src, dst, nwords, bad);
  return cudaGetLastError();
}

cudaError_t launch_packed_unpack(const uint64_t *src, int32_t *dst, int64_t nwords, cudaStream_t s, int num_sms) {
  packed_unpack_kernel<<<grid_for(nwords, num_sms), 256, 0, s>>>(src, dst, nwords);
  return cudaGetLastError();
}

cudaError_t launch_packed_energy(const uint64_t *W, int nx, int ny, int nz, unsigned long long *out, cudaStream_t s,
                                 int num_sms) {
  int64_t nw = (int64_t)(nx >> 6) * ny * nz;
  packed_energy_kernel<<<grid_for(nw, num_sms), 256, 0, s>>>(W, nx, ny, nz, nw, out);
  return cudaGetLastError();
}

}  // namespace spk
