// One whole sq/4n colour sweep of a 32x32 tile, both colours in one pass.
//
// AppLattice::iterate_rejection with sweep color visits colour 1 then
// colour 2 (src/app_lattice.cpp:672-680).  A tile is staged into shared
// memory with a halo of two sites; the colour-1 sites of the tile and of the
// one-site ring around it are updated first (the ring redundantly: its
// owners compute the same values from the same counter-based draws), then
// the colour-2 sites of the tile, which now see every colour-1 neighbour in
// its post-phase state.  The tile is read from `src` and written to `dst`
// (double buffering), so tiles never observe each other's writes.
//
// The Philox block of a site is computed once per sweep and serves the
// colour-1 sites it holds in the first phase and the colour-2 sites in the
// second (an x-pair shares a block; for Ising, four sites do).  A tile has 64
// threads and each owns eight x-pairs: for Ising on int8 site values they are
// two 8-site row segments (two blocks each), updated as eight byte lanes of a
// 64-bit word (tile_segments_ising8); otherwise eight pairs of one column
// updated site by site (tile_pairs_sq4).  With 64 threads every
// thread also updates exactly one ring site, so the first phase is balanced.
#pragma once

#include <stdint.h>

#include "site_update.cuh"
#include "spk_philox.cuh"

namespace spk {

constexpr int kTile = 32;             // tile edge (sites)
constexpr int kHalo = 2;              // halo rows of one fused sq/4n sweep
constexpr int kTileThreads = 64;      // threads per tile
constexpr int kPairsPerThread = kTile * kTile / 2 / kTileThreads;  // 8
// the stage holds rows y0-2 .. y0+33 and columns x0-8 .. x0+39: eight halo
// columns instead of two so that staged rows are whole 8-byte chunks and
// every 8-site row segment of the tile starts on an 8-byte boundary
constexpr int kXOff = 8;
constexpr int kStageX = kTile + 2 * kXOff;  // 48
constexpr int kStageY = kTile + 2 * kHalo;  // 36
constexpr int kStageSites = kStageX * kStageY;
// colour-1 sites one step outside the tile that a colour-2 site of the tile
// neighbours: kTile/2 in each of rows -1 and 32 and columns -1 and 32 (the
// two colour-1 corners (-1,-1) and (32,32) touch the tile only diagonally)
constexpr int kRing = 4 * (kTile / 2);                            // 64 = two warps
static_assert(kRing == 64 && kRing <= kTileThreads, "ring sites must fit one per thread");
static_assert(kPairsPerThread * kTileThreads * 2 == kTile * kTile, "pairs must cover the tile");

struct TileJob {
  const void *src;
  void *dst;
  int L;              // sites per row
  int Ly;             // rows
  int x0, y0;         // tile origin
  int64_t base;       // added to the Philox site counter (0: counters are per lattice)
  uint32_t seed, key1, sweep;
  int nspins;
  int replica;        // ensemble: temperature index of the tile's replica
  const uint64_t *thr;  // thr[dE], dE = 0..4 (all 0 at zero temperature)
  uint64_t t2, t4;      // thr[2] and thr[4] in registers (warp_tile.cuh)
};

__device__ __forceinline__ int stage_at(int lx, int ly) { return (ly + kHalo) * kStageX + lx + kXOff; }

// update one site of the stage in place; returns 1 if its value changed
template <int APP, typename S>
__device__ __forceinline__ int site4(S *stage, int lx, int ly, uint32_t x0, uint32_t x1, int nspins,
                                     const uint64_t *thr) {
  // neighbour order of sq/4n: x-1, y-1, y+1, x+1 (src/create_sites.cpp:1313-1330)
  const int c = stage_at(lx, ly);
  int own = stage[c];
  int nb[4];
  nb[0] = stage[c - 1];
  nb[1] = stage[c - kStageX];
  nb[2] = stage[c + kStageX];
  nb[3] = stage[c + 1];
  int e0;
  int news = update_philox<4, APP>(own, nb, x0, x1, nspins, thr, &e0);
  if (news != own) {
    stage[c] = (S)news;
    return 1;
  }
  return 0;
}

// Issue the staging of a tile (tile + halo, periodic wrap) as 8-byte
// cp.async copies into `stage`; the caller commits, waits and synchronises
// before tile_sweep_sq4 reads it.  Chunks never straddle the wrap: x0 and L
// are multiples of 32 and a chunk holds at most 8 sites.
template <typename S>
__device__ __forceinline__ void tile_stage_async(const TileJob &j, S *stage) {
  constexpr int VEC = 8 / (int)sizeof(S);  // sites per 8-byte chunk
  constexpr int CPR = kStageX / VEC;       // chunks per staged row
  static_assert(kXOff % VEC == 0 && kStageX % VEC == 0, "staged rows are whole chunks");
  const S *src = (const S *)j.src;
  for (int k = threadIdx.x; k < kStageY * CPR; k += kTileThreads) {
    int ly = k / CPR, wc = k - ly * CPR;
    int gy = j.y0 + ly - kHalo, gx = j.x0 - kXOff + wc * VEC;
    gy = gy < 0 ? gy + j.Ly : (gy >= j.Ly ? gy - j.Ly : gy);
    gx = gx < 0 ? gx + j.L : (gx >= j.L ? gx - j.L : gx);
    const void *g = src + (int64_t)gy * j.L + gx;
    unsigned sa = (unsigned)__cvta_generic_to_shared(stage + ly * kStageX + wc * VEC);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(g) : "memory");
  }
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// ring: colour-1 sites one step outside the tile that a colour-2 site of the
// tile neighbours, one per thread tid < kRing (their owners compute the same
// values from the same draws)
template <int APP, typename S>
__device__ __forceinline__ void ring_site(const TileJob &j, S *stage, const RoundKeys &rk, int tid) {
  int q = tid & (kTile / 2 - 1);
  int rlx, rly;
  if (tid < kTile / 2) {               // row -1: lx odd in [1, 31]
    rly = -1;
    rlx = 2 * q + 1;
  } else if (tid < kTile) {            // row 32: lx even in [0, 30]
    rly = kTile;
    rlx = 2 * q;
  } else if (tid < 3 * kTile / 2) {    // column -1: ly odd
    rlx = -1;
    rly = 2 * q + 1;
  } else {                             // column 32: ly even
    rlx = kTile;
    rly = 2 * q;
  }
  int gy = j.y0 + rly, gx = j.x0 + rlx;
  gy = gy < 0 ? gy + j.Ly : (gy >= j.Ly ? gy - j.Ly : gy);
  gx = gx < 0 ? gx + j.L : (gx >= j.L ? gx - j.L : gx);
  int64_t s = j.base + (int64_t)gy * j.L + gx;
  U4 w = philox4x32_10_rk(sweep_counter<APP>((uint64_t)s, j.sweep, 0u), rk);
  uint32_t a0, a1;
  site_words<APP>(w, (uint64_t)s, a0, a1);
  site4<APP, S>(stage, rlx, rly, a0, a1, j.nspins, j.thr);
}

// Site-by-site form: thread tid owns the x-pairs p = tid + k*kTileThreads,
// row p/16, sites 2(p%16) and 2(p%16)+1.
template <int APP, typename S>
__device__ __forceinline__ int tile_pairs_sq4(const TileJob &j, S *stage) {
  S *dst = (S *)j.dst;
  const int tid = threadIdx.x;
  const RoundKeys rk = round_keys(j.seed, j.key1);
  int changed = 0;
  uint32_t keep0[kPairsPerThread], keep1[kPairsPerThread];
  // phase 1: colour-1 sites ((gx+gy) even <=> lx == ly mod 2), in place:
  // their neighbours are all colour 2
#pragma unroll
  for (int k = 0; k < kPairsPerThread; k++) {
    int p = tid + k * kTileThreads;
    int ly = p >> 4, m = p & 15;
    int64_t s = j.base + (int64_t)(j.y0 + ly) * j.L + j.x0 + 2 * m;  // even
    U4 w = philox4x32_10_rk(sweep_counter<APP>((uint64_t)s, j.sweep, 0u), rk);
    int h = ly & 1;  // which site of the pair is colour 1
    uint32_t a0, a1;
    site_words<APP>(w, (uint64_t)(s + h), a0, a1);
    site_words<APP>(w, (uint64_t)(s + 1 - h), keep0[k], keep1[k]);
    changed += site4<APP, S>(stage, 2 * m + h, ly, a0, a1, j.nspins, j.thr);
  }
  if (tid < kRing) ring_site<APP, S>(j, stage, rk, tid);
  __syncthreads();
  // phase 2: colour-2 sites, seeing every colour-1 neighbour updated; each
  // thread then writes its own x-pairs (both values are final) to dst, so no
  // barrier is needed before the next tile (it stages into another buffer)
#pragma unroll
  for (int k = 0; k < kPairsPerThread; k++) {
    int p = tid + k * kTileThreads;
    int ly = p >> 4, m = p & 15;
    int h = ly & 1;  // the pair's colour-1 site
    changed += site4<APP, S>(stage, 2 * m + 1 - h, ly, keep0[k], keep1[k], j.nspins, j.thr);
    S v0 = stage[stage_at(2 * m, ly)], v1 = stage[stage_at(2 * m + 1, ly)];
    S *out = dst + (int64_t)(j.y0 + ly) * j.L + j.x0 + 2 * m;
    if (sizeof(S) == 1) {
      *(uint16_t *)out = (uint16_t)((uint8_t)v0 | ((uint16_t)(uint8_t)v1 << 8));
    } else if (sizeof(S) == 2) {
      *(uint32_t *)out = (uint32_t)(uint16_t)v0 | ((uint32_t)(uint16_t)v1 << 16);
    } else {
      *(uint64_t *)out = (uint64_t)(uint32_t)v0 | ((uint64_t)(uint32_t)v1 << 32);
    }
  }
  return changed;
}

// ---- Ising on int8 site values, eight byte lanes per 64-bit word ----------
//
// A lane holds a site value, 1 or 2; its bit 0 (1 for value 1, 0 for value
// 2) tells the two states apart, so the number of unlike neighbours e0 is the
// sum of four XORs of bit 0, at most 4 per lane (no carry between lanes).
// AppIsing::site_event_rejection (src/app_ising.cpp:104-136) then reads:
// the site's word x proposes value 1 iff x < 2^31; a proposal equal to the
// current value changes nothing; otherwise e1 = 4 - e0, the flip is taken iff
// e1 <= e0 (e0 >= 2) or y < thr[e1-e0] (y = x & 0x7FFFFFFF, thr <= 2^31)
// with e1-e0 = 2 (e0 = 1) or 4 (e0 = 0).  Each site's word is folded into a
// lane code
//   lvl + 4*p,  lvl = [y < thr[4]] + [y < thr[2]],  p = [x < 2^31]
// (thr[4] <= thr[2], so lvl >= 2 - e0 <=> the Boltzmann test passes for that
// e0), and the flip condition becomes e0 + lvl >= 2 and p != bit 0, both
// evaluated for all lanes at once.  At zero temperature thr[] is all zero,
// so lvl = 0 and only e0 >= 2 flips.
constexpr uint64_t kLaneBit = 0x0101010101010101ull;
constexpr uint64_t kEvenLanes = 0x0001000100010001ull;  // bit 0 of lanes 0, 2, 4, 6
constexpr uint64_t kOddLanes = 0x0100010001000100ull;   // bit 0 of lanes 1, 3, 5, 7
constexpr int kSegPerThread = kTile * kTile / 8 / kTileThreads;  // 8-site segments
static_assert(kSegPerThread * 4 == kPairsPerThread, "a segment holds two Philox blocks of four sites");
static_assert(kSegPerThread * 8 * kTileThreads == kTile * kTile, "segments must cover the tile");

// lane code of one site from its word x (thresholds at most 2^31, so the
// tests are 32-bit compares)
__device__ __forceinline__ uint32_t ising_lane_code(uint32_t x, uint32_t t2, uint32_t t4) {
  const uint32_t y = x & kIsingAcceptMask;
  return (uint32_t)(y < t4) + (uint32_t)(y < t2) + (x < kIsingProposal1 ? 4u : 0u);
}

// unlike-neighbour counts of the eight lanes of the segment at stage index c
// (8-byte aligned); v receives the segment itself
__device__ __forceinline__ uint64_t seg_unlike(const int8_t *stage, int c, uint64_t &v) {
  v = *(const uint64_t *)(stage + c);
  const uint64_t up = *(const uint64_t *)(stage + c - kStageX);
  const uint64_t dn = *(const uint64_t *)(stage + c + kStageX);
  const uint64_t lb = (uint8_t)stage[c - 1], rb = (uint8_t)stage[c + 8];
  const uint64_t b = v & kLaneBit;
  const uint64_t l = ((v << 8) | lb) & kLaneBit;          // lane i: site x-1
  const uint64_t r = ((v >> 8) | (rb << 56)) & kLaneBit;  // lane i: site x+1
  return (b ^ l) + (b ^ (up & kLaneBit)) + (b ^ (dn & kLaneBit)) + (b ^ r);
}

// lanes (bit 0) of `cmask` that flip, given unlike counts e, segment v, codes lv
__device__ __forceinline__ uint64_t seg_flips(uint64_t e, uint64_t v, uint64_t lv, uint64_t cmask) {
  const uint64_t acc = (((e + (lv & 0x0303030303030303ull)) + 0x7E7E7E7E7E7E7E7Eull) >> 7) & kLaneBit;
  const uint64_t p = (lv >> 2) & kLaneBit;
  return (p ^ v) & acc & cmask;
}

template <typename S>
__device__ __forceinline__ int tile_segments_ising8(const TileJob &j, S *stage_s) {
  static_assert(sizeof(S) == 1, "byte lanes");
  int8_t *stage = (int8_t *)stage_s;
  int8_t *dst = (int8_t *)j.dst;
  const int tid = threadIdx.x;
  const RoundKeys rk = round_keys(j.seed, j.key1);
  const uint32_t t2 = (uint32_t)j.thr[2], t4 = (uint32_t)j.thr[4];  // at most 2^31
  int changed = 0;
  uint64_t lv[kSegPerThread];
  // draws: the two Philox blocks of each segment, four sites each
#pragma unroll
  for (int k = 0; k < kSegPerThread; k++) {
    const int g = tid + k * kTileThreads;
    const int ly = g >> 2, x0 = (g & 3) * 8;
    const int64_t s = j.base + (int64_t)(j.y0 + ly) * j.L + j.x0 + x0;  // a multiple of 8
    uint64_t code = 0;
#pragma unroll
    for (int i = 0; i < 2; i++) {
      U4 w = philox4x32_10_rk(ising_counter((uint64_t)s + 4 * i, j.sweep, 0u), rk);
      uint32_t c4 = ising_lane_code(w.x, t2, t4) | (ising_lane_code(w.y, t2, t4) << 8) |
                    (ising_lane_code(w.z, t2, t4) << 16) | (ising_lane_code(w.w, t2, t4) << 24);
      code |= (uint64_t)c4 << (32 * i);
    }
    lv[k] = code;
  }
  // phase 1: colour-1 lanes (lane parity == row parity), in place
#pragma unroll
  for (int k = 0; k < kSegPerThread; k++) {
    const int g = tid + k * kTileThreads;
    const int ly = g >> 2, x0 = (g & 3) * 8;
    const int c = stage_at(x0, ly);
    uint64_t v;
    const uint64_t e = seg_unlike(stage, c, v);
    const uint64_t f = seg_flips(e, v, lv[k], (ly & 1) ? kOddLanes : kEvenLanes);
    if (f) {
      *(uint64_t *)(stage + c) = v ^ (f | (f << 1));  // 1 <-> 2
      changed += __popcll(f);
    }
  }
  if (tid < kRing) ring_site<SPKGPU_ISING, S>(j, stage_s, rk, tid);
  __syncthreads();
  // phase 2: colour-2 lanes, seeing every colour-1 neighbour updated; the
  // segment is then final and goes straight to dst
#pragma unroll
  for (int k = 0; k < kSegPerThread; k++) {
    const int g = tid + k * kTileThreads;
    const int ly = g >> 2, x0 = (g & 3) * 8;
    const int c = stage_at(x0, ly);
    uint64_t v;
    const uint64_t e = seg_unlike(stage, c, v);
    const uint64_t f = seg_flips(e, v, lv[k], (ly & 1) ? kEvenLanes : kOddLanes);
    changed += __popcll(f);
    *(uint64_t *)(dst + (int64_t)(j.y0 + ly) * j.L + j.x0 + x0) = v ^ (f | (f << 1));
  }
  return changed;
}

// One fused sweep of a staged tile (tile_stage_async, committed, waited for
// and followed by __syncthreads).  The stage buffer of this tile must not be
// the one the next tile is being staged into, and a thread may return while
// others still read this tile's stage: callers synchronise before reusing it.
// Returns the number of site values changed inside the tile.
template <int APP, typename S>
__device__ __forceinline__ int tile_sweep_sq4(const TileJob &j, S *stage) {
  if constexpr (APP == SPKGPU_ISING && sizeof(S) == 1)
    return tile_segments_ising8<S>(j, stage);
  else
    return tile_pairs_sq4<APP, S>(j, stage);
}

}  // namespace spk
