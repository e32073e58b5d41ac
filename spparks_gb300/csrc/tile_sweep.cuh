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
// Each thread owns four x-pairs of the tile; the Philox block of a pair is
// computed once per sweep and serves the colour-1 site of the pair in the
// first phase and the colour-2 site in the second.
#pragma once

#include <stdint.h>

#include "site_update.cuh"
#include "spk_philox.cuh"

namespace spk {

constexpr int kTile = 32;             // tile edge (sites)
constexpr int kHalo = 2;              // halo rows of one fused sq/4n sweep
constexpr int kTileThreads = 128;     // threads per tile
constexpr int kPairsPerThread = kTile * kTile / 2 / kTileThreads;  // 4
// the stage holds rows y0-2 .. y0+33 and columns x0-4 .. x0+35: four halo
// columns instead of two so that every staged row is whole 32-bit words
constexpr int kXOff = 4;
constexpr int kStageX = kTile + 2 * kXOff;  // 40
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
  int zero_t;
  const uint64_t *thr;  // thr[dE], dE = 0..4
};

__device__ __forceinline__ int stage_at(int lx, int ly) { return (ly + kHalo) * kStageX + lx + kXOff; }

// update one site of the stage in place; returns 1 if its value changed
template <int APP, typename S>
__device__ __forceinline__ int site4(S *stage, int lx, int ly, uint32_t x0, uint32_t x1, int nspins,
                                     const uint64_t *thr, int zero_t) {
  // neighbour order of sq/4n: x-1, y-1, y+1, x+1 (src/create_sites.cpp:1313-1330)
  const int c = stage_at(lx, ly);
  int own = stage[c];
  int nb[4];
  nb[0] = stage[c - 1];
  nb[1] = stage[c - kStageX];
  nb[2] = stage[c + kStageX];
  nb[3] = stage[c + 1];
  int e0;
  int news = update_philox<4, APP>(own, nb, x0, x1, nspins, thr, zero_t, &e0);
  if (news != own) {
    stage[c] = (S)news;
    return 1;
  }
  return 0;
}

// Issue the staging of a tile (tile + halo, periodic wrap) as 4-byte
// cp.async copies into `stage`; the caller commits, waits and synchronises
// before tile_sweep_sq4 reads it.  Word columns never straddle the wrap: x0
// and L are multiples of 32.
template <typename S>
__device__ __forceinline__ void tile_stage_async(const TileJob &j, S *stage) {
  constexpr int VEC = 4 / (int)sizeof(S);  // sites per 32-bit word
  constexpr int WPR = kStageX / VEC;       // words per staged row
  const S *src = (const S *)j.src;
  for (int k = threadIdx.x; k < kStageY * WPR; k += kTileThreads) {
    int ly = k / WPR, wc = k - ly * WPR;
    int gy = j.y0 + ly - kHalo, gx = j.x0 - kXOff + wc * VEC;
    gy = gy < 0 ? gy + j.Ly : (gy >= j.Ly ? gy - j.Ly : gy);
    gx = gx < 0 ? gx + j.L : (gx >= j.L ? gx - j.L : gx);
    const void *g = src + (int64_t)gy * j.L + gx;
    unsigned sa = (unsigned)__cvta_generic_to_shared(stage + ly * kStageX + wc * VEC);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(g) : "memory");
  }
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// One fused sweep of a staged tile (tile_stage_async, committed, waited for
// and followed by __syncthreads).  The stage buffer of this tile must not be
// the one the next tile is being staged into.  Returns the number of site
// values changed inside the tile.
template <int APP, typename S>
__device__ __forceinline__ int tile_sweep_sq4(const TileJob &j, S *stage) {
  constexpr int VEC = 4 / (int)sizeof(S);  // sites per 32-bit word
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
    U4 w = philox4x32_10_rk(U4{(uint32_t)(s >> 1), (uint32_t)(s >> 33), j.sweep, 0u}, rk);
    int h = ly & 1;  // which site of the pair is colour 1
    uint32_t a0 = h ? w.z : w.x, a1 = h ? w.w : w.y;
    keep0[k] = h ? w.x : w.z;
    keep1[k] = h ? w.y : w.w;
    changed += site4<APP, S>(stage, 2 * m + h, ly, a0, a1, j.nspins, j.thr, j.zero_t);
  }
  // ring: colour-1 sites one step outside the tile (their owners compute the
  // same values from the same draws)
  if (tid < kRing) {
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
    U4 w = philox4x32_10_rk(U4{(uint32_t)(s >> 1), (uint32_t)(s >> 33), j.sweep, 0u}, rk);
    uint32_t a0 = (s & 1) ? w.z : w.x, a1 = (s & 1) ? w.w : w.y;
    site4<APP, S>(stage, rlx, rly, a0, a1, j.nspins, j.thr, j.zero_t);
  }
  __syncthreads();
  // phase 2: colour-2 sites, in place, seeing every colour-1 neighbour updated
#pragma unroll
  for (int k = 0; k < kPairsPerThread; k++) {
    int p = tid + k * kTileThreads;
    int ly = p >> 4, m = p & 15;
    changed += site4<APP, S>(stage, 2 * m + 1 - (ly & 1), ly, keep0[k], keep1[k], j.nspins, j.thr, j.zero_t);
  }
  __syncthreads();
  // write the tile interior as 32-bit words
  constexpr int WROW = kTile / VEC;
  for (int k = tid; k < kTile * WROW; k += kTileThreads) {
    int ly = k / WROW, wc = k - ly * WROW;
    uint32_t v = *(const uint32_t *)(stage + stage_at(wc * VEC, ly));
    *(uint32_t *)(dst + (int64_t)(j.y0 + ly) * j.L + j.x0 + wc * VEC) = v;
  }
  return changed;
}

}  // namespace spk
