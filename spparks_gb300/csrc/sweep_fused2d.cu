// Fused sq/4n sweep of a single lattice: one launch per sweep, one CTA per
// 32x32 tile, both colours of the sweep in shared memory (tile_sweep.cuh),
// reading one buffer and writing the other.  Used by spkgpu_sweep for sq/4n
// lattices without sectors, mask or strict RNG whose extents are multiples of
// 32; every other configuration takes the generic phase kernel.  Ising on
// int8 buffers with 16-byte alignment takes the warp form (warp_tile.cuh):
// one tile per warp, two per CTA, same draws and results.

#include "counters.cuh"
#include "spk_internal.h"
#include "tile_sweep.cuh"
#include "warp_tile.cuh"

namespace spk {

template <int APP, typename S>
__global__ void __launch_bounds__(kTileThreads) fused2d_kernel(FusedArgs a) {
  __shared__ __align__(16) S stage[kStageSites];
  __shared__ uint64_t thr[5];
  if (threadIdx.x < 5) thr[threadIdx.x] = a.acc.thr[threadIdx.x];
  int tpr = a.nx / kTile;
  TileJob j;
  j.src = a.src;
  j.dst = a.dst;
  j.L = a.nx;
  j.Ly = a.ny;
  j.x0 = (blockIdx.x % tpr) * kTile;
  j.y0 = (blockIdx.x / tpr) * kTile;
  j.base = 0;
  j.seed = a.seed;
  j.key1 = kStreamSweep;
  j.sweep = a.sweep;
  j.nspins = a.nspins;
  j.replica = 0;
  j.thr = thr;
  tile_stage_async<S>(j, stage);
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  const unsigned int changed = (unsigned int)tile_sweep_sq4<APP, S>(j, stage);
  // each warp adds its count to a spread slot (no block barrier)
  const unsigned int w = __reduce_add_sync(0xFFFFFFFFu, changed);
  if ((threadIdx.x & 31) == 0 && w)
    atomicAdd(&a.naccept[(blockIdx.x * (kTileThreads / 32) + (threadIdx.x >> 5)) & (kCounterSlots - 1)],
              (unsigned long long)w);
}

__global__ void __launch_bounds__(64, 20) fused2d_warp_kernel(FusedArgs a) {
  __shared__ __align__(16) int8_t stage[2][kWStageBytes];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tpr = a.nx / kTile;
  const int t = 2 * blockIdx.x + warp;
  if (t >= tpr * (a.ny / kTile)) return;
  TileJob j;
  j.src = a.src;
  j.dst = a.dst;
  j.L = a.nx;
  j.Ly = a.ny;
  j.x0 = (t % tpr) * kTile;
  j.y0 = (t / tpr) * kTile;
  j.base = 0;
  j.seed = a.seed;
  j.key1 = kStreamSweep;
  j.sweep = a.sweep;
  j.nspins = a.nspins;
  j.replica = 0;
  j.thr = nullptr;
  j.t2 = a.acc.thr[2];
  j.t4 = a.acc.thr[4];
  const unsigned int w = __reduce_add_sync(0xFFFFFFFFu, warp_tile_ising8<false>(j, stage[warp], lane));
  if (lane == 0 && w) atomicAdd(&a.naccept[t & (kCounterSlots - 1)], (unsigned long long)w);
}

bool fused2d_supported(int lattice, int app, int spin_bytes, int nx, int ny) {
  (void)app;
  return lattice == SPKGPU_SQ_4N && nx % kTile == 0 && ny % kTile == 0 &&
         (spin_bytes == 1 || spin_bytes == 2 || spin_bytes == 4);
}

template <typename S>
static cudaError_t launch_fused_t(int app, const FusedArgs &a, cudaStream_t s) {
  unsigned tiles = (unsigned)((a.nx / kTile) * (a.ny / kTile));
  if constexpr (sizeof(S) == 1) {
    if (app == SPKGPU_ISING && ((uintptr_t)a.src | (uintptr_t)a.dst) % 16 == 0) {
      fused2d_warp_kernel<<<(tiles + 1) / 2, 64, 0, s>>>(a);
      return cudaGetLastError();
    }
  }
  switch (app) {
    case SPKGPU_ISING: fused2d_kernel<SPKGPU_ISING, S><<<tiles, kTileThreads, 0, s>>>(a); break;
    case SPKGPU_POTTS: fused2d_kernel<SPKGPU_POTTS, S><<<tiles, kTileThreads, 0, s>>>(a); break;
    case SPKGPU_POTTS_NEIGHONLY: fused2d_kernel<SPKGPU_POTTS_NEIGHONLY, S><<<tiles, kTileThreads, 0, s>>>(a); break;
    case SPKGPU_POTTS_NEIGH: fused2d_kernel<SPKGPU_POTTS_NEIGH, S><<<tiles, kTileThreads, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_fused2d(int lattice, int app, int spin_bytes, const FusedArgs &a, cudaStream_t s, int num_sms) {
  (void)num_sms;
  if (!fused2d_supported(lattice, app, spin_bytes, a.nx, a.ny)) return cudaErrorNotSupported;
  switch (spin_bytes) {
    case 1: return launch_fused_t<int8_t>(app, a, s);
    case 2: return launch_fused_t<int16_t>(app, a, s);
    case 4: return launch_fused_t<int32_t>(app, a, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace spk
