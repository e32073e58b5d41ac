// Colour sweeps of a small sq/4n lattice held in the shared memory of one
// thread-block cluster: all nsweeps sweeps of one spkgpu_sweep call in a
// single launch.
//
// AppLattice::iterate_rejection with sweep color (src/app_lattice.cpp:672-680)
// sweeps colour 1, then colour 2, each site through the app's
// site_event_rejection (src/app_ising.cpp:104-136, src/app_potts.cpp:112-146,
// src/app_potts_neighonly.cpp:71-117, src/app_potts_neigh.cpp:71-116).  For a
// lattice of a few ten thousand sites the tile kernels are bound by their
// launches (one per sweep, a handful of CTAs each).  Here a cluster of eight
// CTAs holds the lattice, one band of ny/8 rows per CTA, in shared memory for
// the whole call.  Per sweep each CTA computes the Philox blocks of its band
// (each block serves the sites of both colours it holds), updates its colour-1
// sites, waits at a cluster barrier, updates its colour-2 sites and waits
// again; the rows just above and below a band are read from the neighbouring
// CTAs' shared memory (distributed shared memory).  During a colour phase a
// site reads only sites of the other colour, which no CTA writes in that
// phase, and the barriers order the phases, so the result is the lattice of
// the per-colour sweep: same per-site rule (update_philox), draws and
// neighbour order as every other sweep kernel.

#include <cooperative_groups.h>

#include "counters.cuh"
#include "spk_internal.h"
#include "site_update.cuh"

namespace cg = cooperative_groups;

namespace spk {

struct ResidentArgs {
  void *spin;
  int nx, ny;
  uint32_t seed, sweep0;
  int nsweeps;
  int nspins;
  unsigned long long *naccept;
  AcceptTable acc;
};

constexpr int kResidentCtas = 8;         // portable cluster size
constexpr int kResidentThreads = 512;
constexpr size_t kResidentMaxBytes = 64 * 1024;  // per CTA

// shared memory of one CTA's band of an n-site lattice (blocks, then sites)
inline size_t resident_bytes(int app, int spin_bytes, int64_t n) {
  const int spb = app == SPKGPU_ISING ? 4 : 2;
  const int64_t band = n / kResidentCtas;
  return (size_t)(band / spb) * sizeof(U4) + (size_t)band * (size_t)spin_bytes;
}

bool resident_supported(int lattice, int app, int spin_bytes, int nx, int ny) {
  return fused2d_supported(lattice, app, spin_bytes, nx, ny) && ny % kResidentCtas == 0 &&
         resident_bytes(app, spin_bytes, (int64_t)nx * ny) <= kResidentMaxBytes;
}

template <typename S, int APP>
__global__ void __cluster_dims__(kResidentCtas, 1, 1) __launch_bounds__(kResidentThreads)
    resident_sq4_kernel(ResidentArgs a) {
  extern __shared__ __align__(16) unsigned char resident_smem[];
  constexpr int SPB = APP == SPKGPU_ISING ? 4 : 2;  // sites per Philox block
  __shared__ uint64_t thr[5];
  __shared__ unsigned int red[kResidentThreads / 32];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int nx = a.nx, ny = a.ny;
  const int R = ny / kResidentCtas;                 // rows of this band
  const int r0 = rank * R;
  const int nb_sites = R * nx;
  const int nblk = nb_sites / SPB;
  const int blk0 = r0 * nx / SPB;                   // first Philox block of the band
  U4 *words = (U4 *)resident_smem;
  S *lat = (S *)(words + nblk);
  // the neighbouring bands: last row of the band above, first row of the band below
  const S *up = cluster.map_shared_rank(lat, (unsigned)((rank + kResidentCtas - 1) % kResidentCtas)) + (R - 1) * nx;
  const S *dn = cluster.map_shared_rank(lat, (unsigned)((rank + 1) % kResidentCtas));
  S *g = (S *)a.spin + (int64_t)r0 * nx;
  const int tid = threadIdx.x;
  if (tid < 5) thr[tid] = a.acc.thr[tid];
  for (int i = tid; i < nb_sites; i += kResidentThreads) lat[i] = g[i];
  const RoundKeys rk = round_keys(a.seed, kStreamSweep);
  cluster.sync();
  unsigned int changed = 0;
  const int half = nx / 2;
  for (int s = 0; s < a.nsweeps; s++) {
    const uint32_t sweep = a.sweep0 + (uint32_t)s;
    // block b holds sites SPB*b .. SPB*b+SPB-1 (counter {b, 0, sweep, 0})
    for (int b = tid; b < nblk; b += kResidentThreads)
      words[b] = philox4x32_10_rk(U4{(uint32_t)(blk0 + b), 0u, sweep, 0u}, rk);
    __syncthreads();
    for (int c = 0; c < 2; c++) {  // colour c+1: (x + y) & 1 == c
      for (int k = tid; k < nb_sites / 2; k += kResidentThreads) {
        const int ly = k / half;
        const int y = r0 + ly;
        const int x = 2 * (k - ly * half) + ((y + c) & 1);
        const int i = ly * nx + x;
        const int xm = x == 0 ? nx - 1 : x - 1, xp = x == nx - 1 ? 0 : x + 1;
        const S vu = ly == 0 ? up[x] : lat[i - nx];
        const S vd = ly == R - 1 ? dn[x] : lat[i + nx];
        // sq/4n neighbour order: x-1, y-1, y+1, x+1 (src/create_sites.cpp:1313-1330)
        const int nb[4] = {(int)lat[ly * nx + xm], (int)vu, (int)vd, (int)lat[ly * nx + xp]};
        const int own = (int)lat[i];
        uint32_t x0, x1;
        site_words<APP>(words[i / SPB], (uint64_t)(r0 * nx + i), x0, x1);
        int e0;
        const int news = update_philox<4, APP>(own, nb, x0, x1, a.nspins, thr, &e0);
        if (news != own) {
          lat[i] = (S)news;
          changed++;
        }
      }
      cluster.sync();
    }
  }
  for (int i = tid; i < nb_sites; i += kResidentThreads) g[i] = lat[i];
  const unsigned int w = __reduce_add_sync(0xFFFFFFFFu, changed);
  if ((tid & 31) == 0) red[tid >> 5] = w;
  __syncthreads();
  if (tid == 0) {
    unsigned long long tot = 0;
    for (int k = 0; k < kResidentThreads / 32; k++) tot += red[k];
    if (tot) atomicAdd(&a.naccept[rank & (kCounterSlots - 1)], tot);
  }
}

template <typename S, int APP>
static cudaError_t launch_resident_t(const ResidentArgs &a, size_t smem, cudaStream_t s) {
  auto f = resident_sq4_kernel<S, APP>;
  cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kResidentMaxBytes);
  if (e != cudaSuccess) return e;
  f<<<kResidentCtas, kResidentThreads, smem, s>>>(a);
  return cudaGetLastError();
}

template <typename S>
static cudaError_t launch_resident_s(int app, const ResidentArgs &a, size_t smem, cudaStream_t s) {
  switch (app) {
    case SPKGPU_ISING: return launch_resident_t<S, SPKGPU_ISING>(a, smem, s);
    case SPKGPU_POTTS: return launch_resident_t<S, SPKGPU_POTTS>(a, smem, s);
    case SPKGPU_POTTS_NEIGHONLY: return launch_resident_t<S, SPKGPU_POTTS_NEIGHONLY>(a, smem, s);
    case SPKGPU_POTTS_NEIGH: return launch_resident_t<S, SPKGPU_POTTS_NEIGH>(a, smem, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_resident_sweeps(int app, int spin_bytes, void *spin, int nx, int ny, uint32_t seed,
                                   uint32_t sweep0, int nsweeps, int nspins, unsigned long long *naccept,
                                   const AcceptTable &acc, cudaStream_t s) {
  if (!resident_supported(SPKGPU_SQ_4N, app, spin_bytes, nx, ny)) return cudaErrorNotSupported;
  ResidentArgs a;
  a.spin = spin;
  a.nx = nx;
  a.ny = ny;
  a.seed = seed;
  a.sweep0 = sweep0;
  a.nsweeps = nsweeps;
  a.nspins = nspins;
  a.naccept = naccept;
  a.acc = acc;
  const size_t smem = resident_bytes(app, spin_bytes, (int64_t)nx * ny);
  switch (spin_bytes) {
    case 1: return launch_resident_s<int8_t>(app, a, smem, s);
    case 2: return launch_resident_s<int16_t>(app, a, smem, s);
    case 4: return launch_resident_s<int32_t>(app, a, smem, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace spk
