// Batched ensemble: hundreds of independent sq/4n lattices of uneven size and
// temperature swept by one persistent cooperative kernel per step, with
// parallel-tempering replica exchange on the device, replayed from a
// captured CUDA graph.
//
// Each sweep every CTA takes 32x32 tiles of all replicas round-robin and runs
// tile_sweep_sq4 (both colours of the sweep, double-buffered); a bounded grid
// barrier separates sweeps.  Every exchange_every sweeps the kernel counts the
// unlike bonds of each replica, then one thread walks the exchange pairs:
// replicas of equal L form a group whose temperature slots are sorted
// ascending; round k tries slot pairs (j, j+1) with j = k mod 2 and accepts
// with probability min(1, exp((1/T_j - 1/T_j+1) (H_j - H_j+1))), H = bonds.
// An accepted exchange swaps the two replicas' temperatures.
//
// The reference has no ensemble (one AppLattice per process); per replica
// the update rule is exactly that of `sweep color` on sq/4n.

#include <cuda/atomic>
#include <cuda_runtime.h>
#include <stdio.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "counters.cuh"
#include "spk_internal.h"
#include "tile_sweep.cuh"
#include "warp_tile.cuh"

namespace spk {

// device control block of an ensemble
struct EnsCtl {
  unsigned int bar_count;
  unsigned int bar_gen;
  int err;
  int parity;                   // buffer holding the current state
  uint32_t sweep;               // next sweep index
  uint32_t xround;              // next exchange round
  unsigned long long naccept;
  unsigned long long xtries;
  unsigned long long xaccepts;
};

struct EnsArgs {
  void *buf0, *buf1;
  const int32_t *L;
  const int64_t *base;
  const int32_t *tile_start;    // nrep+1 prefix of tiles per replica
  const int32_t *tile_rep;      // replica of each tile (launch-per-sweep mode)
  const int2 *tile_pos;         // {replica, (y0/32) << 16 | x0/32} of each tile
  int nrep, ntiles;
  int32_t *tidx;                // replica -> temperature index
  const uint64_t *thr;          // [ntemp][5]
  const double *beta;           // [ntemp]
  const int32_t *group_start;   // ngroups+1 prefix of slots
  const int32_t *slot_t;        // temperature index of each slot (ascending T)
  const int32_t *slot_group;    // group of each slot
  int32_t *who;                 // replica in each slot
  unsigned long long *bonds;    // per replica, accumulated at an exchange
  long long *last_bonds;        // per replica, copy at the last exchange
  int ngroups;
  int nsweeps;
  int exchange_every;
  int nspins;
  uint32_t seed;
  EnsCtl *ctl;
  unsigned long long *nacc_slots;  // kCounterSlots change counters (launch-per-sweep mode)
  const int32_t *pair_rep;      // warp form: replica of each CTA's tile pair
  const int32_t *pair_tile;     // warp form: the pair's two tiles (-1: none)
  int npairs;
  long long spin_limit;         // grid barrier: waits before giving up
  int skip_block;               // grid barrier: this CTA never arrives (error-path test), -1 none
};

constexpr long long kBarrierSpinLimit = 1LL << 25;  // ~seconds with nanosleep: then give up

// grid-wide barrier for a cooperative launch, bounded: a block that waits
// too long sets ctl->err and stops waiting; callers then leave the kernel.
// Arrival is a release RMW and the wait an acquire load at device scope, so
// the writes of every block before the barrier (spins, temperatures) are
// visible to every block after it.
// A CTA whose index is `skip` (the error-path test; -1 in every normal run)
// neither arrives nor waits: the others give up after `limit` waits.
__device__ bool grid_barrier(EnsCtl *ctl, long long limit, int skip) {
  if ((int)blockIdx.x == skip) return false;
  __syncthreads();
  if (threadIdx.x == 0) {
    cuda::atomic_ref<unsigned int, cuda::thread_scope_device> gen(ctl->bar_gen);
    cuda::atomic_ref<unsigned int, cuda::thread_scope_device> count(ctl->bar_count);
    cuda::atomic_ref<int, cuda::thread_scope_device> err(ctl->err);
    unsigned int my = gen.load(cuda::memory_order_acquire);
    unsigned int arrived = count.fetch_add(1u, cuda::memory_order_acq_rel);
    if (arrived == gridDim.x - 1) {
      count.store(0u, cuda::memory_order_relaxed);
      gen.fetch_add(1u, cuda::memory_order_acq_rel);
    } else {
      long long it = 0;
      while (gen.load(cuda::memory_order_acquire) == my) {
        if (++it > limit || err.load(cuda::memory_order_relaxed)) {
          err.store(1, cuda::memory_order_relaxed);
          break;
        }
        __nanosleep(64);
      }
    }
  }
  __syncthreads();
  return *(volatile int *)&ctl->err == 0;
}

__device__ __forceinline__ int replica_of_tile(const int32_t *tile_start, int nrep, int t) {
  int lo = 0, hi = nrep;  // largest r with tile_start[r] <= t
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (tile_start[mid] <= t) lo = mid;
    else hi = mid;
  }
  return lo;
}

// adds the unlike bonds (right and down neighbour of each site) of tile t of
// replica r in `curbuf` to a.bonds[r]; every thread of the block calls it.
// int8 sites, eight per 64-bit word: a byte lane is "unlike" where the XOR
// with the neighbour word is non-zero.
__device__ __forceinline__ uint64_t lanes_nonzero(uint64_t d) {
  return ((d & 0x7F7F7F7F7F7F7F7Full) + 0x7F7F7F7F7F7F7F7Full | d) & 0x8080808080808080ull;
}

template <typename S>
__device__ void tile_bonds(const EnsArgs &a, int t, int r, const S *curbuf) {
  static_assert(sizeof(S) == 1, "ensemble sites are int8");
  const int L = a.L[r];
  const int tpr = L / kTile;
  const int lt = t - a.tile_start[r];
  const int x0 = (lt % tpr) * kTile, y0 = (lt / tpr) * kTile;
  const uint8_t *rep = (const uint8_t *)curbuf + a.base[r];
  unsigned int b = 0;
  // 128 segments of 8 sites per tile
  for (int g = threadIdx.x; g < kTile * kTile / 8; g += kTileThreads) {
    const int y = y0 + (g >> 2), x = x0 + (g & 3) * 8;
    const int xr = x + 8 == L ? 0 : x + 8;
    const int yd = y + 1 == L ? 0 : y + 1;
    const uint64_t v = *(const uint64_t *)(rep + (int64_t)y * L + x);
    const uint64_t dn = *(const uint64_t *)(rep + (int64_t)yd * L + x);
    const uint64_t rb = rep[(int64_t)y * L + xr];
    const uint64_t right = (v >> 8) | (rb << 56);
    b += __popcll(lanes_nonzero(v ^ right)) + __popcll(lanes_nonzero(v ^ dn));
  }
  unsigned int w = __reduce_add_sync(0xFFFFFFFFu, b);
  if ((threadIdx.x & 31) == 0 && w) atomicAdd(&a.bonds[r], (unsigned long long)w);
}

// exchange round `xround` over all groups, by every thread of one block,
// once the bonds of every replica are complete: in a round the slot pairs
// (j, j+1), j - group start = xround mod 2, are disjoint, so each thread
// takes pairs on its own.  Swaps the temperatures of accepted pairs, keeps
// the bonds as last_bonds and clears them.
__device__ void exchange_round(const EnsArgs &a, uint32_t xround) {
  __shared__ unsigned int cnt[2];
  if (threadIdx.x == 0) cnt[0] = cnt[1] = 0;
  __syncthreads();
  unsigned int tries = 0, acc = 0;
  const int n = a.nrep;
  for (int jj = threadIdx.x; jj < n; jj += blockDim.x) {
    const int g = a.slot_group[jj];
    const int lo = a.group_start[g], hi = a.group_start[g + 1];
    if (((jj - lo) & 1) != (int)(xround & 1u) || jj + 1 >= hi) continue;
    int ra = a.who[jj], rb = a.who[jj + 1];
    int ta = a.slot_t[jj], tb = a.slot_t[jj + 1];
    double delta = (a.beta[ta] - a.beta[tb]) * ((double)a.bonds[ra] - (double)a.bonds[rb]);
    U4 w = philox4x32_10(U4{xround, (uint32_t)g, (uint32_t)(jj - lo), 0u}, a.seed, kStreamExchange);
    bool accept = delta >= 0.0;
    if (!accept) {
      double p = exp(delta) * 4294967296.0;
      accept = (double)w.x < floor(p);
    }
    tries++;
    if (accept) {
      a.who[jj] = rb;
      a.who[jj + 1] = ra;
      a.tidx[ra] = tb;
      a.tidx[rb] = ta;
      acc++;
    }
  }
  if (tries) atomicAdd(&cnt[0], tries);
  if (acc) atomicAdd(&cnt[1], acc);
  __syncthreads();  // every pair read its bonds before they are cleared
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    a.last_bonds[r] = (long long)a.bonds[r];
    a.bonds[r] = 0;
  }
  if (threadIdx.x == 0) {
    a.ctl->xtries += cnt[0];
    a.ctl->xaccepts += cnt[1];
  }
  __threadfence();
  __syncthreads();
}

// walks the tiles of a contiguous range, keeping the current replica's
// parameters in registers; replica = temperature index of the tile's replica
// (the thresholds are indexed by temperature)
struct ReplicaCursor {
  int r = 0, tend = 0, L = 0, tpr = 1, tbeg = 0, tidx = 0;
  int64_t base = 0;
  __device__ void load(const EnsArgs &a, int rr) {
    r = rr;
    tbeg = a.tile_start[r];
    tend = a.tile_start[r + 1];
    L = a.L[r];
    tpr = L / kTile;
    base = a.base[r];
    tidx = a.tidx[r];
  }
  __device__ void seek(const EnsArgs &a, int t) { load(a, replica_of_tile(a.tile_start, a.nrep, t)); }
  template <typename S>
  __device__ void job(const EnsArgs &a, int t, const void *src, void *dst, uint32_t sweep, TileJob *j) {
    while (t >= tend) load(a, r + 1);
    int lt = t - tbeg;
    j->src = (const S *)src + base;
    j->dst = (S *)dst + base;
    j->L = L;
    j->Ly = L;
    j->x0 = (lt % tpr) * kTile;
    j->y0 = (lt / tpr) * kTile;
    j->base = 0;  // replicas differ by Philox stream word; site counter is local
    j->seed = a.seed;
    j->key1 = ((uint32_t)(r + 1) << 8) | kStreamSweep;
    j->sweep = sweep;
    j->nspins = a.nspins;
    j->replica = tidx;
    j->thr = nullptr;
  }
};

// 16 CTAs of 64 threads per SM (64 registers) for the byte-lane Ising tile;
// the site-by-site Potts tile keeps more draws live and gets 12 (80)
template <int APP, typename S>
__global__ void __launch_bounds__(kTileThreads, APP == SPKGPU_ISING ? 16 : 12) ensemble_kernel(EnsArgs a) {
  __shared__ __align__(16) S stage[3][kStageSites];
  __shared__ uint64_t thr[3][5];
  __shared__ unsigned long long red[kTileThreads / 32];
  EnsCtl *ctl = a.ctl;
  int parity = *(volatile int *)&ctl->parity;
  uint32_t sweep0 = *(volatile uint32_t *)&ctl->sweep;
  uint32_t xround = *(volatile uint32_t *)&ctl->xround;
  unsigned long long my_changed = 0;
  bool ok = true;
  for (int s = 0; s < a.nsweeps && ok; s++) {
    const void *src = parity ? a.buf1 : a.buf0;
    void *dst = parity ? a.buf0 : a.buf1;
    // each CTA sweeps a contiguous range of tiles (all tiles cost the same),
    // so consecutive tiles almost always share a replica and its parameters
    // are looked up only when the replica changes.  Software pipeline: tile
    // t+1 is staged (cp.async) into the next of three buffers while tile t is
    // swept; by the time a buffer is staged again every thread has passed the
    // barriers of the tile in between, so no thread still reads it.
    const int t0 = (int)(((int64_t)a.ntiles * blockIdx.x) / gridDim.x);
    const int t1 = (int)(((int64_t)a.ntiles * (blockIdx.x + 1)) / gridDim.x);
    const uint32_t sweep = sweep0 + (uint32_t)s;
    ReplicaCursor rc;
    if (t0 < t1) {
      rc.seek(a, t0);
      TileJob first;
      rc.job<S>(a, t0, src, dst, sweep, &first);
      tile_stage_async<S>(first, stage[0]);
    }
    cp_async_commit();
    int sb = 0;
    for (int t = t0; t < t1; t++) {
      const int sn = sb == 2 ? 0 : sb + 1;
      // the job of tile t is rebuilt from the cursor (which the staging of t
      // left at t's replica) rather than carried over, so only one job is
      // live while the tile is swept
      TileJob cur;
      rc.job<S>(a, t, src, dst, sweep, &cur);
      if (threadIdx.x < 5) thr[sb][threadIdx.x] = a.thr[(int64_t)cur.replica * 5 + threadIdx.x];
      if (t + 1 < t1) {
        TileJob nxt;
        rc.job<S>(a, t + 1, src, dst, sweep, &nxt);
        tile_stage_async<S>(nxt, stage[sn]);
      }
      cp_async_commit();
      cp_async_wait<1>();
      __syncthreads();
      cur.thr = thr[sb];
      my_changed += (unsigned long long)tile_sweep_sq4<APP, S>(cur, stage[sb]);
      sb = sn;
    }
    cp_async_wait<0>();
    parity ^= 1;
    ok = grid_barrier(ctl, a.spin_limit, a.skip_block);
    if (!ok) break;
    uint32_t done = sweep0 + (uint32_t)s + 1;
    if (a.exchange_every > 0 && done % (uint32_t)a.exchange_every == 0) {
      // unlike bonds of each replica (right and down neighbour of each site)
      const S *curbuf = (const S *)(parity ? a.buf1 : a.buf0);
      for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x)
        tile_bonds<S>(a, t, replica_of_tile(a.tile_start, a.nrep, t), curbuf);
      ok = grid_barrier(ctl, a.spin_limit, a.skip_block);
      if (!ok) break;
      if (blockIdx.x == 0) exchange_round(a, xround);
      xround++;
      ok = grid_barrier(ctl, a.spin_limit, a.skip_block);
    }
  }
  unsigned long long w = my_changed;
  for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xFFFFFFFFu, w, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = w;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long tot = 0;
    for (int k = 0; k < kTileThreads / 32; k++) tot += red[k];
    if (tot) atomicAdd(&ctl->naccept, tot);
  }
  ok = grid_barrier(ctl, a.spin_limit, a.skip_block) && ok;
  if (blockIdx.x == 0 && threadIdx.x == 0 && ok) {
    ctl->parity = parity;
    ctl->sweep = sweep0 + (uint32_t)a.nsweeps;
    ctl->xround = xround;
  }
}

// ---- launch-per-sweep mode ------------------------------------------------
// (the byte-lane Ising tile fits 32 registers: 32 CTAs of 64 threads per SM;
// the site-by-site Potts tile gets 80)
// The same sweep as one launch per sweep: one CTA per tile of every replica
// (tile -> replica from a table), sweep index ctl->sweep + k and source
// buffer ctl->parity ^ (k & 1), so that a captured graph of k = 0..m-1 can be
// replayed; ensemble_advance_kernel then moves ctl on by m sweeps.  Bonds and
// the exchange round run as their own launches between the last sweep of a
// period and the advance.
// the job of tile t in sweep k of the launch-per-sweep form
template <typename S>
__device__ __forceinline__ void sweep_job(const EnsArgs &a, int t, int parity, uint32_t sweep, TileJob &j) {
  const int2 tp = a.tile_pos[t];
  const int r = tp.x;
  const int L = a.L[r];
  const int64_t base = a.base[r];
  j.src = (const S *)(parity ? a.buf1 : a.buf0) + base;
  j.dst = (S *)(parity ? a.buf0 : a.buf1) + base;
  j.L = L;
  j.Ly = L;
  j.x0 = (tp.y & 0xFFFF) * kTile;
  j.y0 = (tp.y >> 16) * kTile;
  j.base = 0;  // replicas differ by Philox stream word; site counter is local
  j.seed = a.seed;
  j.key1 = ((uint32_t)(r + 1) << 8) | kStreamSweep;
  j.sweep = sweep;
  j.nspins = a.nspins;
  j.replica = a.tidx[r];
}

// TPC consecutive tiles per CTA: tile t+1 is staged (cp.async) into the
// next of three buffers while tile t is swept; a buffer is staged again
// only after every thread has passed the barrier of the tile in between.
// Change counts go from each warp to a spread counter slot (no block barrier).
template <int APP, typename S, int TPC>
__global__ void __launch_bounds__(kTileThreads, APP == SPKGPU_ISING ? 32 : 12) ensemble_sweep_kernel(EnsArgs a,
                                                                                                     int k) {
  constexpr int NB = TPC > 1 ? 3 : 1;
  __shared__ __align__(16) S stage[NB][kStageSites];
  __shared__ uint64_t thr[NB][5];
  const int parity = *(volatile int *)&a.ctl->parity ^ (k & 1);
  const uint32_t sweep = *(volatile uint32_t *)&a.ctl->sweep + (uint32_t)k;
  unsigned int changed = 0;
  if constexpr (TPC == 1) {
    TileJob j;
    sweep_job<S>(a, blockIdx.x, parity, sweep, j);
    if (threadIdx.x < 5) thr[0][threadIdx.x] = a.thr[(int64_t)j.replica * 5 + threadIdx.x];
    tile_stage_async<S>(j, stage[0]);
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    j.thr = thr[0];
    changed = (unsigned int)tile_sweep_sq4<APP, S>(j, stage[0]);
  } else {
    const int t0 = blockIdx.x * TPC;
    const int t1 = min(t0 + TPC, a.ntiles);
    {
      TileJob j;
      sweep_job<S>(a, t0, parity, sweep, j);
      if (threadIdx.x < 5) thr[0][threadIdx.x] = a.thr[(int64_t)j.replica * 5 + threadIdx.x];
      tile_stage_async<S>(j, stage[0]);
      cp_async_commit();
    }
    int b = 0;
    for (int t = t0; t < t1; t++) {
      const int bn = (b + 1 == NB) ? 0 : b + 1;
      if (t + 1 < t1) {
        TileJob nj;
        sweep_job<S>(a, t + 1, parity, sweep, nj);
        if (threadIdx.x < 5) thr[bn][threadIdx.x] = a.thr[(int64_t)nj.replica * 5 + threadIdx.x];
        tile_stage_async<S>(nj, stage[bn]);
      }
      cp_async_commit();
      cp_async_wait<1>();
      __syncthreads();
      // the job is rebuilt from the tables rather than carried across tiles
      TileJob j;
      sweep_job<S>(a, t, parity, sweep, j);
      j.thr = thr[b];
      changed += (unsigned int)tile_sweep_sq4<APP, S>(j, stage[b]);
      b = bn;
    }
  }
  cp_async_wait<0>();
  const unsigned int w = __reduce_add_sync(0xFFFFFFFFu, changed);
  if ((threadIdx.x & 31) == 0 && w)
    atomicAdd(&a.nacc_slots[(blockIdx.x * (kTileThreads / 32) + (threadIdx.x >> 5)) & (kCounterSlots - 1)],
              (unsigned long long)w);
}

// Ising, warp form: CTA b sweeps the tiles pair_tile[2b] and pair_tile[2b+1]
// of replica pair_rep[b], one per warp (warp_tile.cuh); no block barrier.
// Every launch lets the next sweep launch early (griddepcontrol); a sweep
// launched as a programmatic dependent (AFTER_GRID: sweeps 2.. of a group,
// which follow a sweep kernel, never the exchange) computes its draws while
// the previous sweep finishes: the temperature index, thresholds and ctl it
// reads before the wait are written only by the exchange launch.  BONDS (the
// last sweep before an exchange round): the tiles also add the replica's
// unlike bonds after the sweep to a.bonds (warp_tile_bonds), in place of
// ensemble_bonds_kernel.
// this warp's tile of pair pb (none if the pair has one tile)
template <bool AFTER_GRID, bool BONDS>
__device__ __forceinline__ unsigned int warp_pair_tile(const EnsArgs &a, int pb, int warp, int lane, int parity,
                                                       uint32_t sweep, int8_t *stage) {
  const int t = a.pair_tile[2 * pb + warp];
  if (t < 0) return 0;
  const int r = a.pair_rep[pb];
  const int L = a.L[r];
  const int64_t base = a.base[r];
  const int pos = a.tile_pos[t].y;
  TileJob j;
  j.src = (const int8_t *)(parity ? a.buf1 : a.buf0) + base;
  j.dst = (int8_t *)(parity ? a.buf0 : a.buf1) + base;
  j.L = L;
  j.Ly = L;
  j.x0 = (pos & 0xFFFF) * kTile;
  j.y0 = (pos >> 16) * kTile;
  j.base = 0;
  j.seed = a.seed;
  j.key1 = ((uint32_t)(r + 1) << 8) | kStreamSweep;
  j.sweep = sweep;
  j.nspins = a.nspins;
  j.replica = a.tidx[r];
  j.thr = a.thr + (int64_t)j.replica * 5;
  j.t2 = j.thr[2];
  j.t4 = j.thr[4];
  unsigned int bonds = 0;
  const unsigned int changed = warp_tile_ising8<AFTER_GRID, BONDS>(j, stage, lane, &bonds);
  if (BONDS) {
    const unsigned int b = __reduce_add_sync(0xFFFFFFFFu, bonds);
    if (lane == 0 && b) atomicAdd(&a.bonds[r], (unsigned long long)b);
  }
  return changed;
}

template <bool AFTER_GRID, bool BONDS>
__global__ void __launch_bounds__(64, 20) ensemble_warp_kernel(EnsArgs a, int k) {
  __shared__ __align__(16) int8_t stage[2][kWStageBytes];
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = a.pair_tile[2 * blockIdx.x + warp];
  if (t < 0) return;
  const int r = a.pair_rep[blockIdx.x];
  const int parity = *(volatile int *)&a.ctl->parity ^ (k & 1);
  const int L = a.L[r];
  const int64_t base = a.base[r];
  const int pos = a.tile_pos[t].y;
  TileJob j;
  j.src = (const int8_t *)(parity ? a.buf1 : a.buf0) + base;
  j.dst = (int8_t *)(parity ? a.buf0 : a.buf1) + base;
  j.L = L;
  j.Ly = L;
  j.x0 = (pos & 0xFFFF) * kTile;
  j.y0 = (pos >> 16) * kTile;
  j.base = 0;
  j.seed = a.seed;
  j.key1 = ((uint32_t)(r + 1) << 8) | kStreamSweep;
  j.sweep = *(volatile uint32_t *)&a.ctl->sweep + (uint32_t)k;
  j.nspins = a.nspins;
  j.replica = a.tidx[r];
  j.thr = a.thr + (int64_t)j.replica * 5;
  j.t2 = j.thr[2];
  j.t4 = j.thr[4];
  unsigned int bonds = 0;
  const unsigned int w =
      __reduce_add_sync(0xFFFFFFFFu, warp_tile_ising8<AFTER_GRID, BONDS>(j, stage[warp], lane, &bonds));
  if (lane == 0 && w)
    atomicAdd(&a.nacc_slots[(2 * blockIdx.x + warp) & (kCounterSlots - 1)], (unsigned long long)w);
  if (BONDS) {
    const unsigned int b = __reduce_add_sync(0xFFFFFFFFu, bonds);
    if (lane == 0 && b) atomicAdd(&a.bonds[r], (unsigned long long)b);
  }
}

// warps2 / warps4: CTA b sweeps pairs b*TPW .. b*TPW+TPW-1, each warp its
// tile of each pair in turn; only the first tile waits for the previous
// grid, and the warp's lanes finish reading the stage before the next tile
// is staged.  Warps that run several tiles drift apart in phase, so the
// ALU-heavy colour phases of some overlap the multiply-heavy draws of others.
template <bool AFTER_GRID, bool BONDS, int TPW>
__global__ void __launch_bounds__(64, 16) ensemble_warp_multi_kernel(EnsArgs a, int k) {
  __shared__ __align__(16) int8_t stage[2][kWStageBytes];
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int parity = *(volatile int *)&a.ctl->parity ^ (k & 1);
  const uint32_t sweep = *(volatile uint32_t *)&a.ctl->sweep + (uint32_t)k;
  const int pb0 = blockIdx.x * TPW;
  unsigned int changed = warp_pair_tile<AFTER_GRID, BONDS>(a, pb0, warp, lane, parity, sweep, stage[warp]);
#pragma unroll 1
  for (int q = 1; q < TPW; q++) {
    if (pb0 + q >= a.npairs) break;
    __syncwarp();
    changed += warp_pair_tile<false, BONDS>(a, pb0 + q, warp, lane, parity, sweep, stage[warp]);
  }
  const unsigned int w = __reduce_add_sync(0xFFFFFFFFu, changed);
  if (lane == 0 && w)
    atomicAdd(&a.nacc_slots[(2 * blockIdx.x + warp) & (kCounterSlots - 1)], (unsigned long long)w);
}

// unlike bonds (right and down neighbour of each site) of every replica in
// the buffer the sweep k-1 wrote: one warp per 32x32 tile, lane = tile row,
// read as two 16-byte loads; the row below comes from the next lane, the last
// lane loads row 32 itself.  Eight int8 sites per 64-bit word, as in
// tile_bonds.
constexpr int kBondWarps = 8;

__global__ void __launch_bounds__(32 * kBondWarps) ensemble_bonds_kernel(EnsArgs a, int k) {
  const int t = blockIdx.x * kBondWarps + (threadIdx.x >> 5);
  if (t >= a.ntiles) return;
  const int lane = threadIdx.x & 31;
  const int parity = *(volatile int *)&a.ctl->parity ^ (k & 1);
  const int2 tp = a.tile_pos[t];
  const int r = tp.x;
  const int L = a.L[r];
  const int x0 = (tp.y & 0xFFFF) * kTile, y0 = (tp.y >> 16) * kTile;
  const uint8_t *rep = (const uint8_t *)(parity ? a.buf1 : a.buf0) + a.base[r];
  const int y = y0 + lane;
  const int xr = x0 + kTile == L ? 0 : x0 + kTile;
  const uint4 *row = (const uint4 *)(rep + (int64_t)y * L + x0);
  const uint4 p = row[0], q = row[1];
  uint64_t w[4] = {(uint64_t)p.y << 32 | p.x, (uint64_t)p.w << 32 | p.z, (uint64_t)q.y << 32 | q.x,
                   (uint64_t)q.w << 32 | q.z};
  uint64_t dn[4];
#pragma unroll
  for (int i = 0; i < 4; i++) dn[i] = __shfl_down_sync(0xFFFFFFFFu, w[i], 1);
  if (lane == 31) {
    const int yd = y0 + kTile == L ? 0 : y0 + kTile;
    const uint4 *below = (const uint4 *)(rep + (int64_t)yd * L + x0);
    const uint4 bp = below[0], bq = below[1];
    dn[0] = (uint64_t)bp.y << 32 | bp.x;
    dn[1] = (uint64_t)bp.w << 32 | bp.z;
    dn[2] = (uint64_t)bq.y << 32 | bq.x;
    dn[3] = (uint64_t)bq.w << 32 | bq.z;
  }
  const uint64_t rb = rep[(int64_t)y * L + xr];
  unsigned int b = 0;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const uint64_t right = (w[i] >> 8) | ((i < 3 ? w[i + 1] : rb) << 56);
    b += __popcll(lanes_nonzero(w[i] ^ right)) + __popcll(lanes_nonzero(w[i] ^ dn[i]));
  }
  const unsigned int s = __reduce_add_sync(0xFFFFFFFFu, b);
  if (lane == 0 && s) atomicAdd(&a.bonds[r], (unsigned long long)s);
}

// one block: the exchange round (if `exchange`), then ctl moves on by m sweeps
__global__ void __launch_bounds__(256) ensemble_advance_kernel(EnsArgs a, int m, int exchange) {
  EnsCtl *ctl = a.ctl;
  if (exchange) exchange_round(a, *(volatile uint32_t *)&ctl->xround);
  if (threadIdx.x == 0) {
    if (exchange) ctl->xround += 1;
    ctl->sweep += (uint32_t)m;
    ctl->parity ^= (m & 1);
    __threadfence();
  }
}

template <int APP, typename S>
static void *ensemble_fn() {
  return (void *)ensemble_kernel<APP, S>;
}

}  // namespace spk

using namespace spk;

struct spkgpu_ensemble {
  spkgpu_ensemble_desc d;
  std::vector<int32_t> L;
  std::vector<double> T0;
  std::vector<int64_t> base;
  int64_t nsites = 0;
  int ntiles = 0;
  int spin_bytes = 1;
  int num_sms = 1;
  int grid = 1;
  int chunk = 10;
  void *kfn = nullptr;
  void *buf[2] = {nullptr, nullptr};
  int2 *d_tile_pos = nullptr;
  int32_t *d_L = nullptr, *d_tile_start = nullptr, *d_tile_rep = nullptr, *d_tidx = nullptr,
          *d_group_start = nullptr, *d_slot_t = nullptr, *d_slot_group = nullptr, *d_who = nullptr;
  unsigned long long *d_nacc_slots = nullptr;
  int mode = SPKGPU_ENSEMBLE_PERSISTENT;
  float tune_ms[SPKGPU_ENSEMBLE_NMODES] = {-1.0f, -1.0f, -1.0f, -1.0f, -1.0f};  // the autotuner's step times per mode
  int32_t *d_pair_rep = nullptr, *d_pair_tile = nullptr;
  int npairs = 0;
  // pipelined host I/O (spkgpu_ensemble_run_io): two int32 device staging
  // buffers of the input and two of the output (call k uses pair k % 2), one
  // copy stream per direction, events between
  int32_t *io_in32[2] = {nullptr, nullptr}, *io_out32[2] = {nullptr, nullptr};
  cudaStream_t io_in = nullptr, io_out = nullptr;
  cudaEvent_t ev_in_ready[2] = {}, ev_in_free[2] = {}, ev_snap_ready[2] = {}, ev_snap_free[2] = {};
  int io_calls = 0;
  bool io_pending = false;  // run_io calls since the last synchronize (bad-value flag armed)
  int64_t enq = 0;  // sweeps enqueued so far (the host's copy of ctl->sweep)
  std::vector<int32_t> slot_init;  // replica in each exchange slot at creation
  int64_t *d_base = nullptr;
  uint64_t *d_thr = nullptr;
  double *d_beta = nullptr;
  unsigned long long *d_bonds = nullptr;
  long long *d_last_bonds = nullptr;
  EnsCtl *d_ctl = nullptr;
  int32_t *d_stage = nullptr;
  int *d_bad = nullptr;
  int ngroups = 0;
  int parity = 0;
  int64_t nsweeps_done = 0;
  int64_t launches = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t kev0 = nullptr, kev1 = nullptr;  // around the sweep kernels of the captured step
  bool kev_in_graph = false;
  bool replayed = false;  // a graph replay has been enqueued since the capture
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  EnsArgs args;
  std::string err;
};

static int ens_fail(spkgpu_ensemble *e, int code, const std::string &m) {
  if (e) e->err = m;
  return code;
}

static int ens_cuda(spkgpu_ensemble *e, cudaError_t c, const char *what) {
  return ens_fail(e, SPKGPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(c));
}

#define ENS_CUDA(e, call)                                   \
  do {                                                      \
    cudaError_t c__ = (call);                               \
    if (c__ != cudaSuccess) return ens_cuda(e, c__, #call); \
  } while (0)

static cudaError_t ens_launch(spkgpu_ensemble *e, int nsweeps) {
  EnsArgs a = e->args;
  a.nsweeps = nsweeps;
  void *params[] = {&a};
  return cudaLaunchCooperativeKernel(e->kfn, dim3(e->grid), dim3(kTileThreads), params, 0, e->stream);
}

// the warp forms: one, two or four tiles per warp and launch
static bool is_warp_mode(int mode) {
  return mode == SPKGPU_ENSEMBLE_WARPS || mode == SPKGPU_ENSEMBLE_WARPS2 || mode == SPKGPU_ENSEMBLE_WARPS4;
}

// the warp form with TPW tile pairs per CTA; after_grid: launched as a
// programmatic dependent of the previous sweep
template <bool AG, bool BONDS, int TPW>
static constexpr auto warp_kernel() {
  if constexpr (TPW == 1) return ensemble_warp_kernel<AG, BONDS>;
  else return ensemble_warp_multi_kernel<AG, BONDS, TPW>;
}

template <int TPW>
static void launch_warp_t(bool after_grid, bool bonds, unsigned g, const EnsArgs &a, int k, cudaStream_t st) {
  if (!after_grid) {
    if (bonds) warp_kernel<false, true, TPW>()<<<g, 64, 0, st>>>(a, k);
    else warp_kernel<false, false, TPW>()<<<g, 64, 0, st>>>(a, k);
    return;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(g);
  cfg.blockDim = dim3(64);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (bonds) cudaLaunchKernelEx(&cfg, warp_kernel<true, true, TPW>(), a, k);
  else cudaLaunchKernelEx(&cfg, warp_kernel<true, false, TPW>(), a, k);
}

static void launch_warp_sweep(int tpw, bool after_grid, bool bonds, unsigned g, const EnsArgs &a, int k,
                              cudaStream_t st) {
  if (tpw == 4) launch_warp_t<4>(after_grid, bonds, g, a, k, st);
  else if (tpw == 2) launch_warp_t<2>(after_grid, bonds, g, a, k, st);
  else launch_warp_t<1>(after_grid, bonds, g, a, k, st);
}

// one sweep launch of the per-sweep forms (1, 2 or 4 tiles per CTA)
// (warp form: `bonds` = the last sweep before an exchange round counts the
// replicas' unlike bonds itself)
static void launch_sweep(const spkgpu_ensemble *e, const EnsArgs &a, int k, cudaStream_t st, bool bonds) {
  if (is_warp_mode(e->mode)) {
    const int tpw = e->mode == SPKGPU_ENSEMBLE_WARPS4 ? 4 : (e->mode == SPKGPU_ENSEMBLE_WARPS2 ? 2 : 1);
    const unsigned g = (unsigned)((a.npairs + tpw - 1) / tpw);
    launch_warp_sweep(tpw, k > 0, bonds, g, a, k, st);
    return;
  }
  const int tpc = e->mode == SPKGPU_ENSEMBLE_LAUNCHES4 ? 4 : (e->mode == SPKGPU_ENSEMBLE_LAUNCHES2 ? 2 : 1);
  const unsigned grid = (unsigned)((e->ntiles + tpc - 1) / tpc);
  if (e->d.app == SPKGPU_ISING) {
    if (tpc == 4) ensemble_sweep_kernel<SPKGPU_ISING, int8_t, 4><<<grid, kTileThreads, 0, st>>>(a, k);
    else if (tpc == 2) ensemble_sweep_kernel<SPKGPU_ISING, int8_t, 2><<<grid, kTileThreads, 0, st>>>(a, k);
    else ensemble_sweep_kernel<SPKGPU_ISING, int8_t, 1><<<grid, kTileThreads, 0, st>>>(a, k);
  } else {
    if (tpc == 4) ensemble_sweep_kernel<SPKGPU_POTTS, int8_t, 4><<<grid, kTileThreads, 0, st>>>(a, k);
    else if (tpc == 2) ensemble_sweep_kernel<SPKGPU_POTTS, int8_t, 2><<<grid, kTileThreads, 0, st>>>(a, k);
    else ensemble_sweep_kernel<SPKGPU_POTTS, int8_t, 1><<<grid, kTileThreads, 0, st>>>(a, k);
  }
}

// launch-per-sweep mode: m sweeps, the bonds and exchange round if `exchange`,
// then the advance of ctl; returns the number of kernels through *nk
static cudaError_t ens_launch_group(spkgpu_ensemble *e, int m, bool exchange, int64_t *nk) {
  const EnsArgs &a = e->args;
  const unsigned nt = (unsigned)e->ntiles;
  // the warp form counts the bonds in the last sweep of the group
  const bool sweep_bonds = exchange && is_warp_mode(e->mode);
  for (int k = 0; k < m; k++) launch_sweep(e, a, k, e->stream, sweep_bonds && k == m - 1);
  if (exchange && !sweep_bonds)
    ensemble_bonds_kernel<<<(nt + kBondWarps - 1) / kBondWarps, 32 * kBondWarps, 0, e->stream>>>(a, m);
  ensemble_advance_kernel<<<1, 256, 0, e->stream>>>(a, m, exchange ? 1 : 0);
  *nk += m + (exchange && !sweep_bonds ? 1 : 0) + 1;
  return cudaGetLastError();
}

// kernels one step (chunk sweeps) launches in the current mode
static int64_t ens_step_kernels(const spkgpu_ensemble *e) {
  if (e->mode == SPKGPU_ENSEMBLE_PERSISTENT) return 1;
  const bool exchange = e->d.exchange_every > 0;
  return e->chunk + (exchange && !is_warp_mode(e->mode) ? 1 : 0) + 1;
}

// captures one step (chunk sweeps, ending on an exchange point when
// exchanges are on) in the current mode as e->gexec; leaves e->gexec null if
// capture is unavailable (steps are then launched directly)
static void ens_capture(spkgpu_ensemble *e) {
  if (e->gexec) cudaGraphExecDestroy(e->gexec);
  if (e->graph) cudaGraphDestroy(e->graph);
  e->gexec = nullptr;
  e->graph = nullptr;
  cudaStream_t cap = e->stream;
  if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  // external event nodes around the sweep kernels time them in every replay
  bool kev = cudaEventRecordWithFlags(e->kev0, cap, cudaEventRecordExternal) == cudaSuccess;
  cudaError_t le;
  if (e->mode == SPKGPU_ENSEMBLE_PERSISTENT) {
    le = ens_launch(e, e->chunk);
    kev = kev && cudaEventRecordWithFlags(e->kev1, cap, cudaEventRecordExternal) == cudaSuccess;
  } else {
    const EnsArgs &a = e->args;
    const unsigned nt = (unsigned)e->ntiles;
    const bool exchange = e->d.exchange_every > 0;
    const bool sweep_bonds = exchange && is_warp_mode(e->mode);
    for (int k = 0; k < e->chunk; k++) launch_sweep(e, a, k, cap, sweep_bonds && k == e->chunk - 1);
    kev = kev && cudaEventRecordWithFlags(e->kev1, cap, cudaEventRecordExternal) == cudaSuccess;
    if (exchange && !sweep_bonds)
      ensemble_bonds_kernel<<<(nt + kBondWarps - 1) / kBondWarps, 32 * kBondWarps, 0, cap>>>(a, e->chunk);
    ensemble_advance_kernel<<<1, 256, 0, cap>>>(a, e->chunk, exchange ? 1 : 0);
    le = cudaGetLastError();
  }
  cudaGraph_t g = nullptr;
  cudaError_t ce = cudaStreamEndCapture(cap, &g);
  if (le == cudaSuccess && ce == cudaSuccess && g && cudaGraphInstantiate(&e->gexec, g, 0) == cudaSuccess) {
    e->graph = g;
    e->kev_in_graph = kev;
  } else {
    if (g) cudaGraphDestroy(g);
    e->gexec = nullptr;
    e->kev_in_graph = false;
    cudaGetLastError();
  }
  e->replayed = false;
}

// the mutable device state of a fresh ensemble: zero buffers and counters,
// every replica at its own temperature
static cudaError_t ens_reset(spkgpu_ensemble *e) {
  const int n = e->d.nreplica;
  std::vector<int32_t> ident(n);
  std::iota(ident.begin(), ident.end(), 0);
  std::vector<int32_t> who(n);
  for (int k = 0; k < n; k++) who[k] = e->slot_init[k];
  size_t sb = (size_t)e->spin_bytes;
  cudaMemset(e->buf[0], 0, e->nsites * sb);
  cudaMemset(e->buf[1], 0, e->nsites * sb);
  cudaMemset(e->d_bonds, 0, n * 8);
  cudaMemset(e->d_last_bonds, 0, n * 8);
  cudaMemset(e->d_ctl, 0, sizeof(EnsCtl));
  cudaMemset(e->d_nacc_slots, 0, kCounterSlots * sizeof(unsigned long long));
  cudaMemcpy(e->d_tidx, ident.data(), n * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(e->d_who, who.data(), n * 4, cudaMemcpyHostToDevice);
  e->parity = 0;
  e->enq = 0;
  return cudaDeviceSynchronize();
}

// Autotuner: times one captured step of each mode on this replica set
// (after a warm-up step, sites all 1) and keeps the faster; the choice is
// cached per (device, app, replicas, tiles, exchange period) for the process.
// SPKGPU_ENSEMBLE_MODE=persistent|launches|launches2|launches4|warps|warps2|warps4
// forces a mode (the warp forms only for Ising).
static const char *const kModeNames[SPKGPU_ENSEMBLE_NMODES] = {"persistent", "launches", "launches2", "launches4",
                                                                "warps", "warps2", "warps4"};

// the warp form sweeps Ising sites only
static bool ens_mode_ok(const spkgpu_ensemble *e, int mode) {
  return !is_warp_mode(mode) || e->d.app == SPKGPU_ISING;
}

static int ens_pick_mode(spkgpu_ensemble *e, float *ms_out) {
  for (int m = 0; m < SPKGPU_ENSEMBLE_NMODES; m++) ms_out[m] = -1.0f;
  if (const char *env = getenv("SPKGPU_ENSEMBLE_MODE")) {
    for (int m = 0; m < SPKGPU_ENSEMBLE_NMODES; m++)
      if (!strcmp(env, kModeNames[m]) && ens_mode_ok(e, m)) return m;
  }
  static std::mutex mu;
  static std::map<std::vector<int64_t>, int> cache;
  std::vector<int64_t> key{e->d.device, e->d.app, e->d.nreplica, e->ntiles, e->d.exchange_every};
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  int best = SPKGPU_ENSEMBLE_PERSISTENT;
  float best_ms = -1.0f;
  for (int mode = 0; mode < SPKGPU_ENSEMBLE_NMODES; mode++) {
    if (!ens_mode_ok(e, mode)) continue;
    e->mode = mode;
    ens_capture(e);
    if (!e->gexec) continue;
    cudaMemset(e->buf[0], 1, e->nsites * (size_t)e->spin_bytes);
    float ms = 0.0f;
    bool ok = cudaGraphLaunch(e->gexec, e->stream) == cudaSuccess &&
              cudaEventRecord(e->ev0, e->stream) == cudaSuccess &&
              cudaGraphLaunch(e->gexec, e->stream) == cudaSuccess &&
              cudaEventRecord(e->ev1, e->stream) == cudaSuccess && cudaEventSynchronize(e->ev1) == cudaSuccess &&
              cudaEventElapsedTime(&ms, e->ev0, e->ev1) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      continue;
    }
    ms_out[mode] = ms;
    if (best_ms < 0.0f || ms < best_ms) {
      best_ms = ms;
      best = mode;
    }
  }
  std::lock_guard<std::mutex> lock(mu);
  cache[key] = best;
  return best;
}

extern "C" {

const char *spkgpu_ensemble_last_error(const spkgpu_ensemble *e) { return e ? e->err.c_str() : "null handle"; }

int spkgpu_ensemble_destroy(spkgpu_ensemble *e) {
  if (!e) return SPKGPU_ERR_ARG;
  if (e->stream) cudaStreamSynchronize(e->stream);
  if (e->io_in) cudaStreamSynchronize(e->io_in);
  if (e->io_out) cudaStreamSynchronize(e->io_out);
  if (e->gexec) cudaGraphExecDestroy(e->gexec);
  if (e->graph) cudaGraphDestroy(e->graph);
  cudaFree(e->buf[0]);
  cudaFree(e->buf[1]);
  cudaFree(e->d_L);
  cudaFree(e->d_tile_start);
  cudaFree(e->d_tile_rep);
  cudaFree(e->d_tile_pos);
  cudaFree(e->d_pair_rep);
  cudaFree(e->d_pair_tile);
  cudaFree(e->d_nacc_slots);
  cudaFree(e->d_tidx);
  cudaFree(e->d_group_start);
  cudaFree(e->d_slot_t);
  cudaFree(e->d_slot_group);
  cudaFree(e->d_who);
  cudaFree(e->d_base);
  cudaFree(e->d_thr);
  cudaFree(e->d_beta);
  cudaFree(e->d_bonds);
  cudaFree(e->d_last_bonds);
  cudaFree(e->d_ctl);
  cudaFree(e->d_stage);
  cudaFree(e->d_bad);
  if (e->ev0) cudaEventDestroy(e->ev0);
  if (e->ev1) cudaEventDestroy(e->ev1);
  if (e->kev0) cudaEventDestroy(e->kev0);
  if (e->kev1) cudaEventDestroy(e->kev1);
  for (int b = 0; b < 2; b++) {
    cudaFree(e->io_in32[b]);
    cudaFree(e->io_out32[b]);
    for (cudaEvent_t ev : {e->ev_in_ready[b], e->ev_in_free[b], e->ev_snap_ready[b], e->ev_snap_free[b]})
      if (ev) cudaEventDestroy(ev);
  }
  if (e->io_in) cudaStreamDestroy(e->io_in);
  if (e->io_out) cudaStreamDestroy(e->io_out);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
  return SPKGPU_OK;
}

int spkgpu_ensemble_create(const spkgpu_ensemble_desc *desc, spkgpu_ensemble **out) {
  if (!desc || !out || !desc->L || !desc->temperature) return SPKGPU_ERR_ARG;
  *out = nullptr;
  const spkgpu_ensemble_desc &d = *desc;
  if (d.nreplica <= 0 || d.nreplica > (1 << 20)) return SPKGPU_ERR_ARG;
  if (d.app != SPKGPU_ISING && d.app != SPKGPU_POTTS) return SPKGPU_ERR_ARG;
  if (d.app == SPKGPU_ISING && d.nspins != 2) return SPKGPU_ERR_ARG;
  if (d.nspins < 1 || d.nspins > 127) return SPKGPU_ERR_ARG;
  if (d.exchange_every < 0) return SPKGPU_ERR_ARG;
  for (int r = 0; r < d.nreplica; r++) {
    if (d.L[r] < kTile || d.L[r] % kTile || d.L[r] > (1 << 16)) return SPKGPU_ERR_ARG;
    if (!(d.temperature[r] > 0.0) || isinf(d.temperature[r])) return SPKGPU_ERR_ARG;
  }
  spkgpu_ensemble *e = new (std::nothrow) spkgpu_ensemble();
  if (!e) return SPKGPU_ERR_NOMEM;
  e->d = d;
  e->L.assign(d.L, d.L + d.nreplica);
  e->T0.assign(d.temperature, d.temperature + d.nreplica);
  e->d.L = nullptr;
  e->d.temperature = nullptr;
  auto fail = [&](int c) {
    spkgpu_ensemble_destroy(e);
    return c;
  };
  if (cudaSetDevice(d.device) != cudaSuccess) return fail(SPKGPU_ERR_CUDA);
  cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, d.device);
  int n = d.nreplica;
  std::vector<int32_t> tile_start(n + 1, 0);
  e->base.resize(n);
  int64_t off = 0;
  for (int r = 0; r < n; r++) {
    e->base[r] = off;
    off += (int64_t)e->L[r] * e->L[r];
    tile_start[r + 1] = tile_start[r] + (e->L[r] / kTile) * (e->L[r] / kTile);
  }
  e->nsites = off;
  e->ntiles = tile_start[n];
  std::vector<int32_t> tile_rep(e->ntiles);
  std::vector<int2> tile_pos(e->ntiles);
  for (int r = 0; r < n; r++) {
    const int tpr = e->L[r] / kTile;
    for (int t = tile_start[r]; t < tile_start[r + 1]; t++) {
      const int lt = t - tile_start[r];
      tile_rep[t] = r;
      tile_pos[t] = make_int2(r, ((lt / tpr) << 16) | (lt % tpr));
    }
  }
  // warp form: consecutive tiles of a replica in pairs (an odd last tile alone)
  std::vector<int32_t> pair_rep, pair_tile;
  for (int r = 0; r < n; r++)
    for (int t = tile_start[r]; t < tile_start[r + 1]; t += 2) {
      pair_rep.push_back(r);
      pair_tile.push_back(t);
      pair_tile.push_back(t + 1 < tile_start[r + 1] ? t + 1 : -1);
    }
  e->npairs = (int)pair_rep.size();
  // temperatures: index t = the replica that started with it
  std::vector<uint64_t> thr((size_t)n * 5);
  std::vector<double> beta(n);
  for (int t = 0; t < n; t++) {
    AcceptTable at;
    build_accept_table(e->T0[t], e->d.app, &at);
    for (int k = 0; k < 5; k++) thr[(size_t)t * 5 + k] = at.thr[k];
    beta[t] = 1.0 / e->T0[t];
  }
  // exchange groups: equal L, slots by ascending (T, replica)
  std::vector<int32_t> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    if (e->L[a] != e->L[b]) return e->L[a] < e->L[b];
    if (e->T0[a] != e->T0[b]) return e->T0[a] < e->T0[b];
    return a < b;
  });
  std::vector<int32_t> group_start{0}, slot_t(n), who(n), tidx(n);
  for (int k = 0; k < n; k++) {
    if (k > 0 && e->L[order[k]] != e->L[order[k - 1]]) group_start.push_back(k);
    slot_t[k] = order[k];
    who[k] = order[k];
  }
  group_start.push_back(n);
  e->ngroups = (int)group_start.size() - 1;
  e->slot_init = who;
  std::vector<int32_t> slot_group(n);
  for (int g = 0; g < e->ngroups; g++)
    for (int k = group_start[g]; k < group_start[g + 1]; k++) slot_group[k] = g;
  std::iota(tidx.begin(), tidx.end(), 0);

  if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(SPKGPU_ERR_CUDA);
  if (cudaEventCreate(&e->ev0) != cudaSuccess || cudaEventCreate(&e->ev1) != cudaSuccess ||
      cudaEventCreate(&e->kev0) != cudaSuccess || cudaEventCreate(&e->kev1) != cudaSuccess)
    return fail(SPKGPU_ERR_CUDA);
  auto dmalloc = [&](void **p, size_t bytes) { return cudaMalloc(p, bytes == 0 ? 16 : bytes) == cudaSuccess; };
  size_t sb = (size_t)e->spin_bytes;
  if (!dmalloc(&e->buf[0], e->nsites * sb) || !dmalloc(&e->buf[1], e->nsites * sb) ||
      !dmalloc((void **)&e->d_L, n * 4) || !dmalloc((void **)&e->d_tile_start, (n + 1) * 4) ||
      !dmalloc((void **)&e->d_tidx, n * 4) || !dmalloc((void **)&e->d_group_start, group_start.size() * 4) ||
      !dmalloc((void **)&e->d_slot_t, n * 4) || !dmalloc((void **)&e->d_who, n * 4) ||
      !dmalloc((void **)&e->d_base, n * 8) || !dmalloc((void **)&e->d_thr, thr.size() * 8) ||
      !dmalloc((void **)&e->d_beta, n * 8) || !dmalloc((void **)&e->d_bonds, n * 8) ||
      !dmalloc((void **)&e->d_last_bonds, n * 8) || !dmalloc((void **)&e->d_ctl, sizeof(EnsCtl)) ||
      !dmalloc((void **)&e->d_bad, sizeof(int)) || !dmalloc((void **)&e->d_tile_rep, (size_t)e->ntiles * 4) ||
      !dmalloc((void **)&e->d_nacc_slots, kCounterSlots * sizeof(unsigned long long)) ||
      !dmalloc((void **)&e->d_slot_group, n * 4) || !dmalloc((void **)&e->d_tile_pos, (size_t)e->ntiles * 8) ||
      !dmalloc((void **)&e->d_pair_rep, (size_t)e->npairs * 4) ||
      !dmalloc((void **)&e->d_pair_tile, (size_t)e->npairs * 8))
    return fail(SPKGPU_ERR_NOMEM);
  cudaMemcpy(e->d_pair_rep, pair_rep.data(), (size_t)e->npairs * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(e->d_pair_tile, pair_tile.data(), (size_t)e->npairs * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(e->d_tile_pos, tile_pos.data(), (size_t)e->ntiles * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(e->d_slot_group, slot_group.data(), n * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(e->d_tile_rep, tile_rep.data(), (size_t)e->ntiles * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(e->d_L, e->L.data(), n * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(e->d_tile_start, tile_start.data(), (n + 1) * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(e->d_tidx, tidx.data(), n * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(e->d_group_start, group_start.data(), group_start.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(e->d_slot_t, slot_t.data(), n * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(e->d_who, who.data(), n * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(e->d_base, e->base.data(), n * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(e->d_thr, thr.data(), thr.size() * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(e->d_beta, beta.data(), n * 8, cudaMemcpyHostToDevice);
  cudaMemset(e->d_bonds, 0, n * 8);
  cudaMemset(e->d_last_bonds, 0, n * 8);
  cudaMemset(e->d_ctl, 0, sizeof(EnsCtl));
  cudaMemset(e->buf[0], 0, e->nsites * sb);
  cudaMemset(e->buf[1], 0, e->nsites * sb);
  e->kfn = (d.app == SPKGPU_ISING) ? ensemble_fn<SPKGPU_ISING, int8_t>() : ensemble_fn<SPKGPU_POTTS, int8_t>();
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, e->kfn, kTileThreads, 0) != cudaSuccess || per_sm < 1)
    return fail(ens_cuda(e, cudaGetLastError(), "occupancy query"));
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, d.device);
  if (!coop) return fail(ens_fail(e, SPKGPU_ERR_UNSUPPORTED, "device lacks cooperative launch"));
  e->grid = std::min(e->ntiles, per_sm * e->num_sms);
  e->chunk = d.exchange_every > 0 ? d.exchange_every : 10;
  EnsArgs &a = e->args;
  a.buf0 = e->buf[0];
  a.buf1 = e->buf[1];
  a.L = e->d_L;
  a.base = e->d_base;
  a.tile_start = e->d_tile_start;
  a.tile_rep = e->d_tile_rep;
  a.tile_pos = e->d_tile_pos;
  a.nrep = n;
  a.ntiles = e->ntiles;
  a.tidx = e->d_tidx;
  a.thr = e->d_thr;
  a.beta = e->d_beta;
  a.group_start = e->d_group_start;
  a.slot_t = e->d_slot_t;
  a.slot_group = e->d_slot_group;
  a.who = e->d_who;
  a.bonds = e->d_bonds;
  a.last_bonds = e->d_last_bonds;
  a.ngroups = e->ngroups;
  a.nsweeps = 0;
  a.exchange_every = d.exchange_every;
  a.nspins = d.nspins;
  a.seed = d.seed;
  a.ctl = e->d_ctl;
  a.nacc_slots = e->d_nacc_slots;
  a.pair_rep = e->d_pair_rep;
  a.pair_tile = e->d_pair_tile;
  a.npairs = e->npairs;
  a.spin_limit = kBarrierSpinLimit;
  a.skip_block = -1;
  // error-path test of the persistent form: SPKGPU_ENSEMBLE_BARRIER_TEST=
  // "limit,cta" makes the grid barrier give up after `limit` waits and CTA
  // `cta` skip its arrival, so the bounded wait runs out without a hang
  if (const char *env = getenv("SPKGPU_ENSEMBLE_BARRIER_TEST")) {
    long long lim = 0;
    int cta = -1;
    if (sscanf(env, "%lld,%d", &lim, &cta) == 2 && lim > 0) {
      a.spin_limit = lim;
      a.skip_block = cta;
    }
  }
  if (cudaDeviceSynchronize() != cudaSuccess) return fail(SPKGPU_ERR_CUDA);
  // pick the faster execution form for this replica set, then start from a
  // clean state and capture one step of it as a graph
  e->mode = ens_pick_mode(e, e->tune_ms);
  if (ens_reset(e) != cudaSuccess) return fail(ens_cuda(e, cudaGetLastError(), "ensemble reset"));
  ens_capture(e);
  *out = e;
  return SPKGPU_OK;
}

int spkgpu_ensemble_upload(spkgpu_ensemble *e, const int32_t *spin, int64_t n) {
  if (!e || !spin) return SPKGPU_ERR_ARG;
  if (n != e->nsites) return ens_fail(e, SPKGPU_ERR_ARG, "site count mismatch");
  const int64_t chunk = (int64_t)1 << 24;
  ENS_CUDA(e, cudaMemsetAsync(e->d_bad, 0, sizeof(int), e->stream));
  // registered pinned host memory: the conversion kernel reads it directly
  const int32_t *mapped = (const int32_t *)mapped_host_ptr(spin);
  if (mapped) {
    ENS_CUDA(e, launch_convert_in(1, mapped, (int8_t *)e->buf[e->parity], n, e->d.nspins, e->d_bad, e->stream));
    e->launches++;
  } else if (!e->d_stage) {
    ENS_CUDA(e, cudaMalloc(&e->d_stage, (size_t)std::min(chunk, n) * 4));
  }
  for (int64_t off = 0; !mapped && off < n; off += chunk) {
    int64_t m = std::min(chunk, n - off);
    ENS_CUDA(e, cudaMemcpyAsync(e->d_stage, spin + off, (size_t)m * 4, cudaMemcpyHostToDevice, e->stream));
    ENS_CUDA(e, launch_convert_in(1, e->d_stage, (int8_t *)e->buf[e->parity] + off, m, e->d.nspins, e->d_bad,
                                  e->stream));
    e->launches++;
  }
  int bad = 0;
  ENS_CUDA(e, cudaMemcpyAsync(&bad, e->d_bad, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
  ENS_CUDA(e, cudaStreamSynchronize(e->stream));
  if (bad) return ens_fail(e, SPKGPU_ERR_INVALID_SPIN, "One or more sites have invalid values");
  return SPKGPU_OK;
}

int spkgpu_ensemble_download(spkgpu_ensemble *e, int32_t *spin, int64_t n) {
  if (!e || !spin) return SPKGPU_ERR_ARG;
  if (n != e->nsites) return ens_fail(e, SPKGPU_ERR_ARG, "site count mismatch");
  const int64_t chunk = (int64_t)1 << 24;
  // registered pinned host memory: the conversion kernel writes it directly
  int32_t *mapped = (int32_t *)mapped_host_ptr(spin);
  if (mapped) {
    ENS_CUDA(e, launch_convert_out(1, (const int8_t *)e->buf[e->parity], mapped, n, e->stream));
    e->launches++;
    ENS_CUDA(e, cudaStreamSynchronize(e->stream));
    return SPKGPU_OK;
  }
  if (!e->d_stage) ENS_CUDA(e, cudaMalloc(&e->d_stage, (size_t)std::min(chunk, n) * 4));
  for (int64_t off = 0; off < n; off += chunk) {
    int64_t m = std::min(chunk, n - off);
    ENS_CUDA(e, launch_convert_out(1, (const int8_t *)e->buf[e->parity] + off, e->d_stage, m, e->stream));
    e->launches++;
    ENS_CUDA(e, cudaMemcpyAsync(spin + off, e->d_stage, (size_t)m * 4, cudaMemcpyDeviceToHost, e->stream));
  }
  ENS_CUDA(e, cudaStreamSynchronize(e->stream));
  return SPKGPU_OK;
}

static int ens_enqueue(spkgpu_ensemble *e, int32_t nsweeps) {
  int32_t left = nsweeps;
  const int every = e->d.exchange_every;
  while (left > 0) {
    int32_t m;
    if (e->mode == SPKGPU_ENSEMBLE_PERSISTENT) {
      // the kernel places exchanges itself (after every sweep whose count is
      // a multiple of the period)
      m = std::min(left, e->chunk);
      if (e->gexec && m == e->chunk) {
        ENS_CUDA(e, cudaGraphLaunch(e->gexec, e->stream));
        e->replayed = true;
      } else {
        ENS_CUDA(e, ens_launch(e, m));
      }
      e->launches++;
    } else {
      // groups end at exchange points; a whole period from one is the graph
      const int32_t pos = every > 0 ? (int32_t)(e->enq % every) : 0;
      const int32_t room = every > 0 ? every - pos : e->chunk;
      m = std::min(left, room);
      if (e->gexec && pos == 0 && m == e->chunk) {
        ENS_CUDA(e, cudaGraphLaunch(e->gexec, e->stream));
        e->replayed = true;
        e->launches += ens_step_kernels(e);
      } else {
        const bool exchange = every > 0 && (e->enq + m) % every == 0;
        ENS_CUDA(e, ens_launch_group(e, m, exchange, &e->launches));
      }
    }
    left -= m;
    e->enq += m;
    e->parity ^= (m & 1);
  }
  e->nsweeps_done += nsweeps;
  return SPKGPU_OK;
}

int spkgpu_ensemble_run(spkgpu_ensemble *e, int32_t nsweeps) {
  if (!e || nsweeps < 0) return SPKGPU_ERR_ARG;
  return ens_enqueue(e, nsweeps);
}

int spkgpu_ensemble_timed_run(spkgpu_ensemble *e, int32_t nsweeps, float *ms) {
  if (!e || !ms || nsweeps < 0) return SPKGPU_ERR_ARG;
  ENS_CUDA(e, cudaEventRecord(e->ev0, e->stream));
  int rc = ens_enqueue(e, nsweeps);
  if (rc) return rc;
  ENS_CUDA(e, cudaEventRecord(e->ev1, e->stream));
  ENS_CUDA(e, cudaEventSynchronize(e->ev1));
  ENS_CUDA(e, cudaEventElapsedTime(ms, e->ev0, e->ev1));
  return SPKGPU_OK;
}

// Pipelined host I/O.  Call k uses staging pair b = k % 2, on three streams:
//   io_in:   (once call k-2 converted io_in32[b]) DMA of the input,
//            page-locked host int32 -> io_in32[b]
//   stream:  io_in32[b] -> current buffer (int8, checked), the sweeps, current
//            buffer -> io_out32[b] (once call k-2's output left io_out32[b])
//   io_out:  DMA of io_out32[b] -> page-locked host int32
// The copy engines move the next calls' inputs and the previous calls'
// outputs while the SMs sweep, back to back in each direction: the host link
// (about 210 GB/s one way, 170 GB/s each way with both directions busy on a
// GB300 host) is the bound of a step whose sweeps take less time than its
// copies.  Kernels that read or write host memory directly reach the same
// link rate but hold SMs for the whole transfer.
static int ens_io_setup(spkgpu_ensemble *e) {
  if (e->io_in) return SPKGPU_OK;
  const size_t bytes = (size_t)e->nsites * sizeof(int32_t);
  for (int b = 0; b < 2; b++)
    if (cudaMalloc((void **)&e->io_in32[b], bytes) != cudaSuccess ||
        cudaMalloc((void **)&e->io_out32[b], bytes) != cudaSuccess)
      return ens_fail(e, SPKGPU_ERR_NOMEM, "run_io staging buffers");
  for (int b = 0; b < 2; b++)
    for (cudaEvent_t *ev : {&e->ev_in_ready[b], &e->ev_in_free[b], &e->ev_snap_ready[b], &e->ev_snap_free[b]})
      ENS_CUDA(e, cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
  ENS_CUDA(e, cudaStreamCreateWithFlags(&e->io_in, cudaStreamNonBlocking));
  ENS_CUDA(e, cudaStreamCreateWithFlags(&e->io_out, cudaStreamNonBlocking));
  for (int b = 0; b < 2; b++) {
    ENS_CUDA(e, cudaEventRecord(e->ev_in_free[b], e->stream));
    ENS_CUDA(e, cudaEventRecord(e->ev_snap_free[b], e->stream));
  }
  return SPKGPU_OK;
}

int spkgpu_ensemble_run_io(spkgpu_ensemble *e, const int32_t *in, int32_t *out, int32_t nsweeps) {
  if (!e || !in || !out || nsweeps < 0) return SPKGPU_ERR_ARG;
  if (!mapped_host_ptr(in) || !mapped_host_ptr(out)) {  // pageable: the three steps in turn
    int rc = spkgpu_ensemble_upload(e, in, e->nsites);
    if (!rc) rc = ens_enqueue(e, nsweeps);
    if (!rc) rc = spkgpu_ensemble_download(e, out, e->nsites);
    return rc;
  }
  int rc = ens_io_setup(e);
  if (rc) return rc;
  const int64_t n = e->nsites;
  const size_t bytes = (size_t)n * sizeof(int32_t);
  const int b = e->io_calls & 1;
  if (!e->io_pending) {
    ENS_CUDA(e, cudaMemsetAsync(e->d_bad, 0, sizeof(int), e->stream));
    e->io_pending = true;
  }
  ENS_CUDA(e, cudaStreamWaitEvent(e->io_in, e->ev_in_free[b], 0));
  ENS_CUDA(e, cudaMemcpyAsync(e->io_in32[b], in, bytes, cudaMemcpyHostToDevice, e->io_in));
  ENS_CUDA(e, cudaEventRecord(e->ev_in_ready[b], e->io_in));
  ENS_CUDA(e, cudaStreamWaitEvent(e->stream, e->ev_in_ready[b], 0));
  ENS_CUDA(e, launch_convert_in(e->spin_bytes, e->io_in32[b], e->buf[e->parity], n, e->d.nspins, e->d_bad, e->stream));
  ENS_CUDA(e, cudaEventRecord(e->ev_in_free[b], e->stream));
  e->launches += 1;
  rc = ens_enqueue(e, nsweeps);
  if (rc) return rc;
  ENS_CUDA(e, cudaStreamWaitEvent(e->stream, e->ev_snap_free[b], 0));
  ENS_CUDA(e, launch_convert_out(e->spin_bytes, e->buf[e->parity], e->io_out32[b], n, e->stream));
  ENS_CUDA(e, cudaEventRecord(e->ev_snap_ready[b], e->stream));
  e->launches += 1;
  ENS_CUDA(e, cudaStreamWaitEvent(e->io_out, e->ev_snap_ready[b], 0));
  ENS_CUDA(e, cudaMemcpyAsync(out, e->io_out32[b], bytes, cudaMemcpyDeviceToHost, e->io_out));
  ENS_CUDA(e, cudaEventRecord(e->ev_snap_free[b], e->io_out));
  e->io_calls++;
  return SPKGPU_OK;
}

int spkgpu_ensemble_synchronize(spkgpu_ensemble *e) {
  if (!e) return SPKGPU_ERR_ARG;
  ENS_CUDA(e, cudaStreamSynchronize(e->stream));
  if (e->io_in) ENS_CUDA(e, cudaStreamSynchronize(e->io_in));
  if (e->io_out) ENS_CUDA(e, cudaStreamSynchronize(e->io_out));
  if (e->io_pending) {
    e->io_pending = false;
    int bad = 0;
    ENS_CUDA(e, cudaMemcpy(&bad, e->d_bad, sizeof(int), cudaMemcpyDeviceToHost));
    if (bad) return ens_fail(e, SPKGPU_ERR_INVALID_SPIN, "One or more sites of a run_io input have invalid values");
  }
  EnsCtl c;
  ENS_CUDA(e, cudaMemcpy(&c, e->d_ctl, sizeof(c), cudaMemcpyDeviceToHost));
  if (c.err) return ens_fail(e, SPKGPU_ERR_DEVICE, "grid barrier wait gave up");
  return SPKGPU_OK;
}

int spkgpu_ensemble_get_stats(spkgpu_ensemble *e, spkgpu_ensemble_stats *out) {
  if (!e || !out) return SPKGPU_ERR_ARG;
  int rc = spkgpu_ensemble_synchronize(e);
  if (rc) return rc;
  EnsCtl c;
  ENS_CUDA(e, cudaMemcpy(&c, e->d_ctl, sizeof(c), cudaMemcpyDeviceToHost));
  unsigned long long slots[kCounterSlots];
  ENS_CUDA(e, cudaMemcpy(slots, e->d_nacc_slots, sizeof(slots), cudaMemcpyDeviceToHost));
  unsigned long long nacc = c.naccept;
  for (int k = 0; k < kCounterSlots; k++) nacc += slots[k];
  out->naccept = (int64_t)nacc;
  out->nattempt = e->nsites * e->nsweeps_done;
  out->nsweeps = e->nsweeps_done;
  out->exchange_tries = (int64_t)c.xtries;
  out->exchange_accepts = (int64_t)c.xaccepts;
  return SPKGPU_OK;
}

int spkgpu_ensemble_temperatures(spkgpu_ensemble *e, double *temperature) {
  if (!e || !temperature) return SPKGPU_ERR_ARG;
  int rc = spkgpu_ensemble_synchronize(e);
  if (rc) return rc;
  std::vector<int32_t> tidx(e->d.nreplica);
  ENS_CUDA(e, cudaMemcpy(tidx.data(), e->d_tidx, tidx.size() * 4, cudaMemcpyDeviceToHost));
  for (int r = 0; r < e->d.nreplica; r++) temperature[r] = e->T0[tidx[r]];
  return SPKGPU_OK;
}

int spkgpu_ensemble_energies(spkgpu_ensemble *e, int64_t *bonds) {
  if (!e || !bonds) return SPKGPU_ERR_ARG;
  int rc = spkgpu_ensemble_synchronize(e);
  if (rc) return rc;
  ENS_CUDA(e, cudaMemcpy(bonds, e->d_last_bonds, (size_t)e->d.nreplica * 8, cudaMemcpyDeviceToHost));
  return SPKGPU_OK;
}

int spkgpu_ensemble_sweep_kernel_ms(spkgpu_ensemble *e, float *ms, int32_t *nlaunch) {
  if (!e || !ms || !nlaunch) return SPKGPU_ERR_ARG;
  if (!e->kev_in_graph || !e->replayed)
    return ens_fail(e, SPKGPU_ERR_UNSUPPORTED, "no replay of a captured step to time");
  ENS_CUDA(e, cudaEventSynchronize(e->kev1));
  ENS_CUDA(e, cudaEventElapsedTime(ms, e->kev0, e->kev1));
  *nlaunch = (e->mode == SPKGPU_ENSEMBLE_PERSISTENT) ? 1 : e->chunk;
  return SPKGPU_OK;
}

int spkgpu_ensemble_mode(const spkgpu_ensemble *e, int32_t *mode, float *tune_ms) {
  if (!e || !mode) return SPKGPU_ERR_ARG;
  *mode = e->mode;
  if (tune_ms)
    for (int m = 0; m < SPKGPU_ENSEMBLE_NMODES; m++) tune_ms[m] = e->tune_ms[m];
  return SPKGPU_OK;
}

int spkgpu_ensemble_launch_count(const spkgpu_ensemble *e, int64_t *count) {
  if (!e || !count) return SPKGPU_ERR_ARG;
  *count = e->launches;
  return SPKGPU_OK;
}

}  // extern "C"
