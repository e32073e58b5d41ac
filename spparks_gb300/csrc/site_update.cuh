// Per-site rejection update shared by every sweep kernel: the device form of
//   AppIsing::site_event_rejection          src/app_ising.cpp:104-136
//   AppPotts::site_event_rejection          src/app_potts.cpp:112-146
//   AppPottsNeighOnly::site_event_rejection src/app_potts_neighonly.cpp:71-117
//   AppPottsNeigh::site_event_rejection     src/app_potts_neigh.cpp:71-116
// with site_energy (src/app_ising.cpp:88-95) as a count of unlike neighbours.
// Neighbour values arrive in the reference's neighbour order
// (CreateSites::offsets_2d/3d, src/create_sites.cpp:1303-1371), which fixes
// the first-appearance order of the distinct-value list.
#pragma once

#include <stdint.h>

#include "../../include/spkgpu.h"
#include "spk_philox.cuh"

namespace spk {

// neighbour offsets of a lattice style in reference order: dx outer, then dy,
// then dz, each -1..1, keeping |d|=1 (4n/6n) or 0<|d|<=sqrt(dim) (8n/26n)
template <int LAT>
struct Stencil {
  static constexpr bool k3d = (LAT == SPKGPU_SC_6N || LAT == SPKGPU_SC_26N);
  static constexpr int NN = (LAT == SPKGPU_SQ_4N) ? 4 : (LAT == SPKGPU_SQ_8N) ? 8 : (LAT == SPKGPU_SC_6N) ? 6 : 26;
  static constexpr int NCOLOR = (LAT == SPKGPU_SQ_8N) ? 4 : (LAT == SPKGPU_SC_26N) ? 8 : 2;
  // offset j as (dx,dy,dz)
  __host__ __device__ static constexpr void offset(int j, int &dx, int &dy, int &dz) {
    int n = 0;
    dx = dy = dz = 0;
    for (int a = -1; a <= 1; a++)
      for (int b = -1; b <= 1; b++)
        for (int c = (k3d ? -1 : 0); c <= (k3d ? 1 : 0); c++) {
          int r2 = a * a + b * b + c * c;
          bool keep = (LAT == SPKGPU_SQ_4N || LAT == SPKGPU_SC_6N) ? (r2 == 1) : (r2 >= 1);
          if (!keep) continue;
          if (n == j) {
            dx = a;
            dy = b;
            dz = c;
          }
          n++;
        }
  }
  // Lattice::id2color (src/lattice.cpp:234-283), 1-based
  __host__ __device__ static int color(int x, int y, int z) {
    if (LAT == SPKGPU_SQ_4N) return ((x + y) & 1) + 1;
    if (LAT == SPKGPU_SQ_8N) return 2 * (y & 1) + (x & 1) + 1;
    if (LAT == SPKGPU_SC_6N) return ((x + y + z) & 1) + 1;
    return 4 * (z & 1) + 2 * (y & 1) + (x & 1) + 1;
  }
};

// linear index of the periodic neighbour (x+dx, y+dy, z+dz) (site index =
// id-1 = x + nx*(y + ny*z), src/create_sites.cpp:506-655)
template <int LAT>
__device__ __forceinline__ int64_t wrap_index(int x, int y, int z, int dx, int dy, int dz, int nx, int ny,
                                              int nz) {
  int xn = x + dx, yn = y + dy, zn = z + dz;
  xn = xn < 0 ? xn + nx : (xn >= nx ? xn - nx : xn);
  yn = yn < 0 ? yn + ny : (yn >= ny ? yn - ny : yn);
  if (Stencil<LAT>::k3d) zn = zn < 0 ? zn + nz : (zn >= nz ? zn - nz : zn);
  else zn = 0;
  return (int64_t)xn + (int64_t)nx * ((int64_t)yn + (int64_t)ny * zn);
}

// bit j set <=> neighbour j holds a value that differs from `own` and from
// every earlier neighbour: the reference's unique[] list in order
template <int NN>
__device__ __forceinline__ uint32_t first_appearance(int own, const int (&nb)[NN]) {
  uint32_t first = 0;
#pragma unroll
  for (int j = 0; j < NN; j++) {
    bool f = nb[j] != own;
#pragma unroll
    for (int k = 0; k < j; k++) f = f && (nb[k] != nb[j]);
    first |= (f ? 1u : 0u) << j;
  }
  return first;
}

template <int NN>
__device__ __forceinline__ int pick_value(const int (&nb)[NN], int j) {
  int v = nb[0];
#pragma unroll
  for (int k = 1; k < NN; k++)
    if (k == j) v = nb[k];
  return v;
}

template <int NN>
__device__ __forceinline__ int count_unlike(int v, const int (&nb)[NN]) {
  int e = 0;
#pragma unroll
  for (int j = 0; j < NN; j++) e += (nb[j] != v);
  return e;
}

// Philox counter of the block holding site s's draws, and the draws x0
// (proposal) and x1 (Boltzmann test) of site s from that block: ising takes
// one word per site (x1 = its low 31 bits), the other apps two words of the
// x-pair's block.  Two sites s, s+1 with s even share one block in both.
template <int APP>
SPK_HD U4 sweep_counter(uint64_t s, uint32_t sweep, uint32_t pass) {
  return APP == SPKGPU_ISING ? ising_counter(s, sweep, pass)
                             : U4{(uint32_t)(s >> 1), (uint32_t)(s >> 33), sweep, pass};
}

template <int APP>
SPK_HD void site_words(const U4 &w, uint64_t s, uint32_t &x0, uint32_t &x1) {
  if (APP == SPKGPU_ISING) {
    x0 = block_word(w, (int)(s & 3));
    x1 = x0 & kIsingAcceptMask;
  } else {
    x0 = (s & 1) ? w.z : w.x;
    x1 = (s & 1) ? w.w : w.y;
  }
}

// Philox form: x0 = draw 0 (proposal), x1 = draw 1 (Boltzmann test).
// thr[dE] in shared or register memory.  At zero temperature every thr[dE]
// is 0, so "x1 < thr" rejects every uphill move, which is the reference's
// temperature == 0 branch; no separate flag is tested.  Returns the new
// site value.
template <int NN, int APP>
__device__ __forceinline__ int update_philox(int own, const int (&nb)[NN], uint32_t x0, uint32_t x1,
                                             int nspins, const uint64_t *thr, int *e0_out) {
  int e0 = count_unlike<NN>(own, nb);
  *e0_out = e0;
  int news;
  if (APP == SPKGPU_ISING) {
    news = (x0 < kIsingProposal1) ? 1 : 2;
  } else if (APP == SPKGPU_POTTS) {
    uint32_t r = scaled_pick((uint32_t)nspins, x0);
    if (r > (uint32_t)(nspins - 1)) r = nspins - 1;
    news = (int)r + 1;
  } else {
    uint32_t first = first_appearance<NN>(own, nb);
    int nevent = __popc(first);
    uint32_t iran;
    if (APP == SPKGPU_POTTS_NEIGHONLY) {
      if (nevent == 0) return own;
      iran = scaled_pick((uint32_t)nevent, x0);
      if (iran > (uint32_t)(nevent - 1)) iran = nevent - 1;
    } else {
      iran = scaled_pick((uint32_t)NN, x0);
      if ((int)iran >= nevent) return own;
    }
    int j = __fns(first, 0, (int)iran + 1);
    news = pick_value<NN>(nb, j);
  }
  if (news == own) return own;
  // two-state Ising: every neighbour equals either own or news
  int e1 = (APP == SPKGPU_ISING) ? NN - e0 : count_unlike<NN>(news, nb);
  if (e1 <= e0) return news;
  return ((uint64_t)x1 < thr[e1 - e0]) ? news : own;
}

// Park-Miller step of RandomPark::uniform (src/random_park.cpp:79-86)
__device__ __forceinline__ double park_uniform(int &seed) {
  int k = seed / 127773;
  seed = 16807 * (seed - k * 127773) - 2836 * k;
  if (seed < 0) seed += 2147483647;
  return (1.0 / 2147483647) * seed;
}

// strict form: draws come from the site's own Park-Miller state, in the
// reference's order and number (no draw when the move cannot happen)
template <int NN, int APP>
__device__ __forceinline__ int update_strict(int own, const int (&nb)[NN], int &pm, int nspins,
                                             const double *pexp, int zero_t, int *e0_out) {
  int e0 = count_unlike<NN>(own, nb);
  *e0_out = e0;
  int news;
  if (APP == SPKGPU_ISING) {
    news = (park_uniform(pm) < 0.5) ? 1 : 2;
  } else if (APP == SPKGPU_POTTS) {
    int iran = (int)(nspins * park_uniform(pm)) + 1;
    if (iran > nspins) iran = nspins;
    news = iran;
  } else {
    uint32_t first = first_appearance<NN>(own, nb);
    int nevent = __popc(first);
    int iran;
    if (APP == SPKGPU_POTTS_NEIGHONLY) {
      if (nevent == 0) return own;
      iran = (int)(nevent * park_uniform(pm));
      if (iran >= nevent) iran = nevent - 1;
    } else {
      iran = (int)(NN * park_uniform(pm));
      if (iran >= nevent) return own;
    }
    int j = __fns(first, 0, iran + 1);
    news = pick_value<NN>(nb, j);
  }
  int e1 = count_unlike<NN>(news, nb);
  if (e1 <= e0) return news;
  if (zero_t) return own;
  if (park_uniform(pm) > pexp[e1 - e0]) return own;
  return news;
}

}  // namespace spk
