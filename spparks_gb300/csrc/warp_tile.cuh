// One whole sq/4n colour sweep of a 32x32 tile of Ising sites stored as int8,
// swept by ONE warp (AppIsing::site_event_rejection, src/app_ising.cpp:104-136,
// under AppLattice::iterate_rejection with sweep color,
// src/app_lattice.cpp:672-680: colour 1, then colour 2).
//
// Same schedule and draws as tile_sweep.cuh (stage with a two-row halo,
// colour-1 sites of the tile and of its one-site ring first, then the
// colour-2 sites), with three differences that cut the work per site:
//   * one warp owns the tile, so the two phases are separated by __syncwarp,
//     and a CTA of two warps sweeps two tiles of one lattice (one Philox key);
//   * the Philox blocks and lane codes are computed while the tile's staging
//     copies are in flight (they do not depend on site values);
//   * the stage holds 16 halo columns on each side so that every row is four
//     16-byte cp.async chunks.
//
// Lane arithmetic.  Each 32-bit word holds four sites (byte lanes), values 1
// or 2.  For a lane with value v and neighbour values summing to S (4..8):
//   unlike neighbours e = S - 4 (v = 1) or 8 - S (v = 2) = (S ^ X) - 3v - 1,
//   with X = 15 where v = 2 and 0 where v = 1 (15 - S = S ^ 15 for S <= 15).
// The Philox word x of a site (four sites per block) is folded into one code
// byte
//   0x9D + lvl - 0x40 p,  lvl = [y < thr[4]] + [y < thr[2]],  p = [x < 2^31],
//   y = x & 0x7FFFFFFF (the Boltzmann draw; every threshold is at most 2^31,
//   so the compares are 32-bit and a threshold of 2^31 passes every y),
// so that s = (S ^ X) + code - 3v = e + lvl + 0x1E + 0x40 (2 - p) per lane:
// bits 0-5 stay below 0x25, bit 5 is set iff e + lvl >= 2 (the flip, or a
// proposal equal to the current value, is accepted: e >= 2 means dE <= 0;
// e = 1 needs y < thr[2]; e = 0 needs y < thr[4], and thr[4] <= thr[2]),
// and bits 6-7 hold the proposed value 2 - p.  The new lane value is the
// proposal where bit 5 is set, else v.  No step carries or borrows across
// lanes.  At zero temperature thr[] is all zero, so lvl = 0 and only e >= 2
// is accepted.
//
// A colour phase takes the four sites of the phase's colour out of each
// 8-site segment (every other byte: the colours alternate along x) into one
// word with __byte_perm, so the lane rule runs once per four sites of the
// phase, and puts the new values back in x order.
//
// Site values must be 1 or 2 (uploads check the range).  The Philox site
// counter of a tile is its lattice index (TileJob::base is not used): with
// x0 and L multiples of 32, every 8-site segment starts at a multiple of 8
// and takes two whole blocks.
#pragma once

#include <stdint.h>

#include "spk_philox.cuh"
#include "tile_sweep.cuh"

namespace spk {

constexpr int kWXOff = 16;                          // halo columns on each side
constexpr int kWStageX = kTile + 2 * kWXOff;        // 64 bytes per staged row
constexpr int kWStageBytes = kWStageX * kStageY;    // 2304
constexpr int kWChunks = kStageY * kWStageX / 16;   // 144 chunks of 16 bytes
constexpr int kWSegPerLane = kTile * kTile / 8 / 32;  // 4 segments of 8 sites
static_assert(kWSegPerLane * 8 * 32 == kTile * kTile, "segments must cover the tile");
static_assert(kRing == 2 * 32, "two ring sites per lane");

__device__ __forceinline__ int wstage_at(int lx, int ly) { return (ly + kHalo) * kWStageX + lx + kWXOff; }

// Issue the staging of the tile (rows y0-2 .. y0+33, columns x0-16 .. x0+47,
// periodic wrap) as 16-byte cp.async copies; the caller commits, waits and
// synchronises the warp.  src and L must keep every chunk 16-byte aligned.
__device__ __forceinline__ void warp_stage_async(const TileJob &j, int8_t *stage, int lane) {
  // lane: chunk column lane & 3, rows (lane >> 2) + 8m; one chunk at a time
  // (a rolled loop keeps a single address live)
  int gx = j.x0 - kWXOff + 16 * (lane & 3);
  gx = gx < 0 ? gx + j.L : (gx >= j.L ? gx - j.L : gx);
  const int8_t *src = (const int8_t *)j.src + gx;
  unsigned sa = (unsigned)__cvta_generic_to_shared(stage + (lane >> 2) * kWStageX + 16 * (lane & 3));
#pragma unroll 1
  for (int ly = lane >> 2; ly < kStageY; ly += 8, sa += 8 * kWStageX) {
    int gy = j.y0 + ly - kHalo;
    gy = gy < 0 ? gy + j.Ly : (gy >= j.Ly ? gy - j.Ly : gy);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src + (int64_t)gy * j.L) : "memory");
  }
}

// c + INC if x < t (unsigned), as a compare and a predicated add of an
// immediate (a constant in a register would stay live across the draws)
template <uint32_t INC>
__device__ __forceinline__ uint32_t add_if_below(uint32_t c, uint32_t x, uint32_t t) {
  asm("{\n\t.reg .pred q;\n\tsetp.lt.u32 q, %1, %2;\n\t@q add.u32 %0, %0, %3;\n\t}"
      : "+r"(c)
      : "r"(x), "r"(t), "n"(INC));
  return c;
}

// adds the code of a site with Philox word x to the byte at bit SH of c,
// which starts at 0x9D; t2 and t4 are thr[2] and thr[4] (at most 2^31)
template <int SH>
__device__ __forceinline__ uint32_t add_lane_code(uint32_t c, uint32_t x, uint32_t t2, uint32_t t4) {
  asm("{\n\t.reg .pred q;\n\tsetp.lt.u32 q, %1, 0x80000000;\n\t@q add.u32 %0, %0, %2;\n\t}"
      : "+r"(c)
      : "r"(x), "n"(0u - (0x40u << SH)));
  const uint32_t y = x & kIsingAcceptMask;
  c = add_if_below<1u << SH>(c, y, t4);
  return add_if_below<1u << SH>(c, y, t2);
}

// ring site k (0..63) of the tile, as in ring_site: rows -1 and 32, then
// columns -1 and 32, sixteen colour-1 sites each
__device__ __forceinline__ void warp_ring_pos(int k, int &rlx, int &rly) {
  const int q = k & (kTile / 2 - 1);
  if (k < kTile / 2) {
    rly = -1;
    rlx = 2 * q + 1;
  } else if (k < kTile) {
    rly = kTile;
    rlx = 2 * q;
  } else if (k < 3 * kTile / 2) {
    rlx = -1;
    rly = 2 * q + 1;
  } else {
    rlx = kTile;
    rly = 2 * q;
  }
}

// __byte_perm selectors taking the sites of x parity 0 (x0, x0+2, x0+4, x0+6)
// or parity 1 out of a segment held as (sites x0..x0+3, sites x0+4..x0+7)
constexpr uint32_t kSelEven = 0x6420u, kSelOdd = 0x7531u;

// selector of the x parity of the colour-1 sites of this lane's rows (all its
// rows have the parity of row lane>>2)
__device__ __forceinline__ uint32_t colour1_selector(int lane) { return kSelEven + 0x1111u * ((lane >> 2) & 1); }

// the codes of a lane's sites: segment m (row (lane>>2) + 8m, columns
// 8(lane&3) .. +7) as its four colour-1 sites in code[2m] and its four
// colour-2 sites in code[2m+1], in x order; the lane's ring sites k = lane
// and lane+32 in the low bytes of ring[]
struct WarpDraws {
  uint32_t code[2 * kWSegPerLane];
  uint32_t ring[2];
};

// the draws of segments M0 .. M1-1 and, if RING, of the ring sites
template <int M0, int M1, bool RING>
__device__ __forceinline__ void warp_draws(const TileJob &j, int lane, WarpDraws &d) {
  const RoundKeys rk = round_keys(j.seed, j.key1);
  const uint32_t t2 = (uint32_t)j.t2, t4 = (uint32_t)j.t4;  // at most 2^31
  // the ring first: its codes then stay live in two registers only
#pragma unroll
  for (int r = 0; r < (RING ? 2 : 0); r++) {
    int rlx, rly;
    warp_ring_pos(lane + 32 * r, rlx, rly);
    int gy = j.y0 + rly, gx = j.x0 + rlx;
    gy = gy < 0 ? gy + j.Ly : (gy >= j.Ly ? gy - j.Ly : gy);
    gx = gx < 0 ? gx + j.L : (gx >= j.L ? gx - j.L : gx);
    const int64_t s = (int64_t)gy * j.L + gx;
    const U4 w = philox4x32_10_rk(ising_counter((uint64_t)s, j.sweep, 0u), rk);
    d.ring[r] = add_lane_code<0>(0x9Du, block_word(w, (int)(s & 3)), t2, t4);
  }
  const uint32_t sel1 = colour1_selector(lane);
#pragma unroll
  for (int m = M0; m < M1; m++) {
    const int ly = (lane >> 2) + 8 * m;
    const int64_t s = (int64_t)(j.y0 + ly) * j.L + j.x0 + 8 * (lane & 3);  // a multiple of 8
    uint32_t cw[2];  // codes of sites x0..x0+3 and x0+4..x0+7
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const U4 w = philox4x32_10_rk(ising_counter((uint64_t)s + 4 * h, j.sweep, 0u), rk);
      uint32_t c = add_lane_code<0>(0x9D9D9D9Du, w.x, t2, t4);
      c = add_lane_code<8>(c, w.y, t2, t4);
      c = add_lane_code<16>(c, w.z, t2, t4);
      cw[h] = add_lane_code<24>(c, w.w, t2, t4);
    }
    d.code[2 * m] = __byte_perm(cw[0], cw[1], sel1);
    d.code[2 * m + 1] = __byte_perm(cw[0], cw[1], sel1 ^ 0x1111u);
  }
}

// new values of four lanes v, all of the phase's colour, with neighbour
// values summing to `sum` per lane and codes `code`
__device__ __forceinline__ uint32_t warp_lanes(uint32_t v, uint32_t sum, uint32_t code) {
  const uint32_t x = v * 15u - 0x0F0F0F0Fu;
  const uint32_t s = (sum ^ x) + (code - 3u * v);
  const uint32_t am = (s & 0x20202020u) * 6u;  // bits 6-7 of the accepted lanes
  return ((s & am) | ((v << 6) & ~am)) >> 6;
}

// __byte_perm selectors and offsets of one colour phase for a lane whose
// active sites (the phase's colour) have x parity P
struct PhaseSel {
  uint32_t act, other;  // the active / other x parity of a segment
  uint32_t side;        // the active sites' neighbours across the segment edge
  int side_off;         // stage offset of the word holding that edge site
  uint32_t lo, hi;      // interleave (new active, other) back into x order
};

__device__ __forceinline__ PhaseSel phase_sel(uint32_t act) {
  const bool odd = act == kSelOdd;
  PhaseSel p;
  p.act = act;
  p.other = act ^ 0x1111u;
  // parity 0: left neighbours [x0-1, x0+1, x0+3, x0+5] from the word ending
  // at x0-1 and the odd sites; parity 1: right neighbours [x0+2 .. x0+8]
  p.side = odd ? 0x4321u : 0x2107u;
  p.side_off = odd ? 8 : -4;
  p.lo = odd ? 0x1504u : 0x5140u;
  p.hi = odd ? 0x3726u : 0x7362u;
  return p;
}

// one colour phase of a segment at stage index c: the four active sites are
// gathered into one word (their left and right neighbours are the other
// four sites and one edge site, their up and down neighbours the same x
// parity of the rows above and below), updated, and put back in x order;
// *diff gets the changed lanes (3 in each changed byte)
__device__ __forceinline__ uint2 warp_segment(const int8_t *stage, int c, uint32_t code, const PhaseSel &p,
                                              uint32_t *diff) {
  const uint2 v = *(const uint2 *)(stage + c);
  const uint2 up = *(const uint2 *)(stage + c - kWStageX);
  const uint2 dn = *(const uint2 *)(stage + c + kWStageX);
  const uint32_t edge = *(const uint32_t *)(stage + c + p.side_off);
  const uint32_t a = __byte_perm(v.x, v.y, p.act), b = __byte_perm(v.x, v.y, p.other);
  const uint32_t sum = b + __byte_perm(b, edge, p.side) + __byte_perm(up.x, up.y, p.act) +
                       __byte_perm(dn.x, dn.y, p.act);
  const uint32_t an = warp_lanes(a, sum, code);
  *diff = a ^ an;
  return make_uint2(__byte_perm(an, b, p.lo), __byte_perm(an, b, p.hi));
}

// bit 7 of each byte lane set where the lane of d is non-zero
__device__ __forceinline__ uint32_t bytes_nonzero(uint32_t d) {
  return (((d & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | d) & 0x80808080u;
}

// Unlike bonds counted by this tile after both phases, from the stage holding
// the tile's final values and its final colour-1 ring: every bond inside the
// tile (right and down neighbour of each site), and every bond across the
// tile's edge whose colour-2 end is in the tile (the other end is a ring
// site).  Each bond across two tiles has exactly one colour-2 end, so the
// tiles of a lattice count each unlike bond once.  This lane's share.
__device__ __forceinline__ unsigned int warp_tile_bonds(const int8_t *stage, int lane) {
  const int x0 = 8 * (lane & 3);
  const bool odd_rows = (lane >> 2) & 1;  // the parity of every row of this lane
  unsigned int b = 0;
#pragma unroll
  for (int m = 0; m < kWSegPerLane; m++) {
    const int ly = (lane >> 2) + 8 * m;
    const int c = wstage_at(x0, ly);
    const uint2 v = *(const uint2 *)(stage + c);
    const uint32_t rw = *(const uint32_t *)(stage + c + 8);
    const uint32_t h_lo = bytes_nonzero(v.x ^ __funnelshift_r(v.x, v.y, 8));
    uint32_t h_hi = bytes_nonzero(v.y ^ __funnelshift_r(v.y, rw, 8));
    // column 31 meets column 32 outside the tile: counted where (31, y) is colour 2, y even
    if (x0 == kTile - 8 && odd_rows) h_hi &= 0x00808080u;
    const uint2 dn = *(const uint2 *)(stage + c + kWStageX);
    uint32_t d_lo = bytes_nonzero(v.x ^ dn.x), d_hi = bytes_nonzero(v.y ^ dn.y);
    // row 31 meets row 32 outside the tile: counted where (x, 31) is colour 2, x even
    if (ly == kTile - 1) {
      d_lo &= 0x00800080u;
      d_hi &= 0x00800080u;
    }
    b += __popc(h_lo) + __popc(h_hi) + __popc(d_lo) + __popc(d_hi);
    if (ly == 0) {  // row 0 meets row -1: counted where (x, 0) is colour 2, x odd
      const uint2 up = *(const uint2 *)(stage + c - kWStageX);
      b += __popc(bytes_nonzero(v.x ^ up.x) & 0x80008000u) + __popc(bytes_nonzero(v.y ^ up.y) & 0x80008000u);
    }
    if (x0 == 0 && odd_rows) {  // column 0 meets column -1: counted where (0, y) is colour 2, y odd
      const uint32_t lw = *(const uint32_t *)(stage + c - 4);
      b += ((v.x ^ (lw >> 24)) & 0xFFu) != 0;
    }
  }
  return b;
}

// Both colour phases of the staged tile (warp_stage_async, waited for and
// followed by __syncwarp); the tile's final values go to j.dst.  Returns the
// number of this lane's sites that changed; with BONDS, also this lane's
// share of the unlike bonds after the sweep in *bonds (warp_tile_bonds).
template <bool BONDS>
__device__ __forceinline__ unsigned int warp_phases(const TileJob &j, int8_t *stage, int lane, const WarpDraws &d,
                                                    unsigned int *bonds) {
  int8_t *dst = (int8_t *)j.dst;
  const int x0 = 8 * (lane & 3);
  // colour-1 sites have the x parity of the row; rows of a lane share a parity
  const PhaseSel p1 = phase_sel(colour1_selector(lane));
  uint32_t cnt = 0;  // 3 per changed site, per byte lane
#pragma unroll
  for (int m = 0; m < kWSegPerLane; m++) {
    const int c = wstage_at(x0, (lane >> 2) + 8 * m);
    uint32_t diff;
    const uint2 n = warp_segment(stage, c, d.code[2 * m], p1, &diff);
    cnt += diff;
    // only colour-1 sites change; readers of this word in this phase use only
    // its colour-2 sites, which are written back unchanged
    *(uint2 *)(stage + c) = n;
  }
#pragma unroll
  for (int r = 0; r < 2; r++) {
    int rlx, rly;
    warp_ring_pos(lane + 32 * r, rlx, rly);
    const int c = wstage_at(rlx, rly);
    const uint32_t own = (uint8_t)stage[c];
    const uint32_t sum =
        (uint32_t)(uint8_t)stage[c - 1] + (uint8_t)stage[c + 1] + (uint8_t)stage[c - kWStageX] +
        (uint8_t)stage[c + kWStageX];
    const uint32_t s = (sum ^ (own * 15u - 15u)) + (d.ring[r] - 3u * own);
    if ((s & 0x20u) && (s >> 6) != own) stage[c] = (int8_t)(s >> 6);
  }
  __syncwarp();
  const PhaseSel p2 = phase_sel(p1.other);
#pragma unroll
  for (int m = 0; m < kWSegPerLane; m++) {
    const int ly = (lane >> 2) + 8 * m;
    const int c = wstage_at(x0, ly);
    uint32_t diff;
    const uint2 n = warp_segment(stage, c, d.code[2 * m + 1], p2, &diff);
    cnt += diff;
    *(uint2 *)(dst + (int64_t)(j.y0 + ly) * j.L + j.x0 + x0) = n;
    // the colour-2 lanes are final; readers of this word in this phase use
    // only its colour-1 lanes, which do not change
    if (BONDS) *(uint2 *)(stage + c) = n;
  }
  if (BONDS) {
    __syncwarp();
    *bonds = warp_tile_bonds(stage, lane);
  }
  return ((cnt * 0x01010101u) >> 24) / 3u;
}

// stage, draws, then both phases of one tile; j.t2 and j.t4 are the
// thresholds thr[2] and thr[4] (thr[2] >= thr[4]); returns this lane's changes
// AFTER_GRID: the kernel was launched as a programmatic dependent of the
// previous sweep, whose output this tile reads: the ring's and half the
// segments' draws (which read no site) run first, then griddepcontrol.wait
// holds the warp until that grid has completed and its writes are visible,
// then the tile is staged while the other half of the draws runs.
template <bool AFTER_GRID, bool BONDS = false>
__device__ __forceinline__ unsigned int warp_tile_ising8(const TileJob &j, int8_t *stage, int lane,
                                                         unsigned int *bonds = nullptr) {
  WarpDraws d;
  if (AFTER_GRID) {
    warp_draws<0, kWSegPerLane / 2, true>(j, lane, d);
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    warp_stage_async(j, stage, lane);
    cp_async_commit();
    warp_draws<kWSegPerLane / 2, kWSegPerLane, false>(j, lane, d);
  } else {
    warp_stage_async(j, stage, lane);
    cp_async_commit();
    warp_draws<0, kWSegPerLane, true>(j, lane, d);
  }
  cp_async_wait<0>();
  __syncwarp();
  return warp_phases<BONDS>(j, stage, lane, d, bonds);
}

}  // namespace spk
