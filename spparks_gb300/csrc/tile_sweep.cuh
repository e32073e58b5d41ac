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
constexpr int kHalo = 2;              // halo width of one fused sq/4n sweep
constexpr int kTileThreads = 128;     // threads per tile
constexpr int kPairsPerThread = kTile * kTile / 2 / kTileThreads;  // 4
constexpr int kStage = kTile + 2 * kHalo;                         // 36
// colour-1 sites one step outside the tile: rows -1 and 32 hold kTile/2+1
// each, columns -1 and 32 (rows 0..31) kTile/2 each
constexpr int kRing = 2 * (kTile / 2 + 1) + 2 * (kTile / 2);      // 66
static_assert(kRing == 66 && kRing <= kTileThreads, "ring sites must fit one per thread");
static_assert(kPairsPerThread * kTileThreads * 2 == kTile * kTile, "pairs must cover the tile");

struct TileJob {
  const void *src;
  void *dst;
  int L;              // replica edge: sites per row and rows (square)
  int Ly;             // rows
  int x0, y0;         // tile origin
  int64_t base;       // added to the Philox site counter (0: counters are per lattice)
  uint32_t seed, key1, sweep;
  int nspins;
  int zero_t;
  const uint64_t *thr;  // thr[dE], dE = 0..4
};

template <int APP, typename S>
__device__ __forceinline__ int site4(const S *stage, int lx, int ly, uint32_t x0, uint32_t x1, int nspins,
                                     const uint64_t *thr, int zero_t, S *out) {
  // neighbour order of sq/4n: x-1, y-1, y+1, x+1 (src/create_sites.cpp:1313-1330)
  int own = stage[(ly + kHalo) * kStage + lx + kHalo];
  int nb[4];
  nb[0] = stage[(ly + kHalo) * kStage + lx + kHalo - 1];
  nb[1] = stage[(ly + kHalo - 1) * kStage + lx + kHalo];
  nb[2] = stage[(ly + kHalo + 1) * kStage + lx + kHalo];
  nb[3] = stage[(ly + kHalo) * kStage + lx + kHalo + 1];
  int e0;
  int news = update_philox<4, APP>(own, nb, x0, x1, nspins, thr, zero_t, &e0);
  *out = (S)news;
  return news != own;
}

// returns the number of site values changed inside the tile
template <int APP, typename S>
__device__ int tile_sweep_sq4(const TileJob &j, S *stage) {
  const S *src = (const S *)j.src;
  S *dst = (S *)j.dst;
  const int tid = threadIdx.x;
  // stage tile + halo with periodic wrap
  for (int k = tid; k < kStage * kStage; k += kTileThreads) {
    int ly = k / kStage, lx = k - ly * kStage;
    int gy = j.y0 + ly - kHalo, gx = j.x0 + lx - kHalo;
    gy = gy < 0 ? gy + j.Ly : (gy >= j.Ly ? gy - j.Ly : gy);
    gx = gx < 0 ? gx + j.L : (gx >= j.L ? gx - j.L : gx);
    stage[k] = src[(int64_t)gy * j.L + gx];
  }
  __syncthreads();

  int changed = 0;
  uint32_t keep0[kPairsPerThread], keep1[kPairsPerThread];
  S newA[kPairsPerThread];
  // phase 1: colour-1 sites ((gx+gy) even <=> lx == ly mod 2) of my pairs
#pragma unroll
  for (int k = 0; k < kPairsPerThread; k++) {
    int p = tid + k * kTileThreads;
    int ly = p >> 4, m = p & 15;
    int64_t s = j.base + (int64_t)(j.y0 + ly) * j.L + j.x0 + 2 * m;  // even
    U4 w = philox4x32_10(U4{(uint32_t)(s >> 1), (uint32_t)(s >> 33), j.sweep, 0u}, j.seed, j.key1);
    int h = ly & 1;  // which site of the pair is colour 1
    uint32_t a0 = h ? w.z : w.x, a1 = h ? w.w : w.y;
    keep0[k] = h ? w.x : w.z;
    keep1[k] = h ? w.y : w.w;
    changed += site4<APP, S>(stage, 2 * m + h, ly, a0, a1, j.nspins, j.thr, j.zero_t, &newA[k]);
  }
  // ring: colour-1 sites one step outside the tile
  S ringv = 0;
  int rlx = 0, rly = 0;
  bool ring = tid < kRing;
  if (ring) {
    if (tid < kTile / 2 + 1) {           // row -1: lx odd in [-1, 31]
      rly = -1;
      rlx = 2 * tid - 1;
    } else if (tid < kTile + 2) {        // row 32: lx even in [0, 32]
      rly = kTile;
      rlx = 2 * (tid - (kTile / 2 + 1));
    } else if (tid < kTile + 2 + kTile / 2) {  // column -1: ly odd
      rlx = -1;
      rly = 2 * (tid - (kTile + 2)) + 1;
    } else {                             // column 32: ly even
      rlx = kTile;
      rly = 2 * (tid - (kTile + 2 + kTile / 2));
    }
    int gy = j.y0 + rly, gx = j.x0 + rlx;
    gy = gy < 0 ? gy + j.Ly : (gy >= j.Ly ? gy - j.Ly : gy);
    gx = gx < 0 ? gx + j.L : (gx >= j.L ? gx - j.L : gx);
    int64_t s = j.base + (int64_t)gy * j.L + gx;
    U4 w = philox4x32_10(U4{(uint32_t)(s >> 1), (uint32_t)(s >> 33), j.sweep, 0u}, j.seed, j.key1);
    uint32_t a0 = (s & 1) ? w.z : w.x, a1 = (s & 1) ? w.w : w.y;
    site4<APP, S>(stage, rlx, rly, a0, a1, j.nspins, j.thr, j.zero_t, &ringv);
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kPairsPerThread; k++) {
    int p = tid + k * kTileThreads;
    int ly = p >> 4, m = p & 15;
    stage[(ly + kHalo) * kStage + 2 * m + (ly & 1) + kHalo] = newA[k];
  }
  if (ring) stage[(rly + kHalo) * kStage + rlx + kHalo] = ringv;
  __syncthreads();
  // phase 2: colour-2 sites, reading the post-phase-1 stage
  S newB[kPairsPerThread];
#pragma unroll
  for (int k = 0; k < kPairsPerThread; k++) {
    int p = tid + k * kTileThreads;
    int ly = p >> 4, m = p & 15;
    int h = 1 - (ly & 1);
    changed += site4<APP, S>(stage, 2 * m + h, ly, keep0[k], keep1[k], j.nspins, j.thr, j.zero_t, &newB[k]);
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kPairsPerThread; k++) {
    int p = tid + k * kTileThreads;
    int ly = p >> 4, m = p & 15;
    stage[(ly + kHalo) * kStage + 2 * m + 1 - (ly & 1) + kHalo] = newB[k];
  }
  __syncthreads();
  // write the tile interior
  for (int k = tid; k < kTile * kTile; k += kTileThreads) {
    int ly = k >> 5, lx = k & 31;
    dst[(int64_t)(j.y0 + ly) * j.L + j.x0 + lx] = stage[(ly + kHalo) * kStage + lx + kHalo];
  }
  __syncthreads();
  return changed;
}

}  // namespace spk
