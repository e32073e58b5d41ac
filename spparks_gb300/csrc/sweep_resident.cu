// Colour sweeps of a small sq/4n lattice held in the shared memory of one
// thread-block cluster: all nsweeps sweeps of one spkgpu_sweep call in a
// single launch.
//
// AppLattice::iterate_rejection with sweep color (src/app_lattice.cpp:672-680)
// sweeps colour 1, then colour 2, each site through the app's
// site_event_rejection (src/app_ising.cpp:104-136, src/app_potts.cpp:112-146,
// src/app_potts_neighonly.cpp:71-117, src/app_potts_neigh.cpp:71-116).  For a
// lattice of a few ten thousand sites the tile kernels are bound by their
// launches (one per sweep, a handful of CTAs each).  Here a cluster of 16
// CTAs (8 where 16 cannot be scheduled or the rows do not divide) holds the
// lattice, one band of ny/CL rows per CTA, in shared memory for the whole
// call.  Each thread owns x-pairs (2m, 2m+1) of its band: one site of each
// colour, whose draws come from one Philox block (four Ising words or the
// pair's two Potts word pairs), which the thread computes itself, in
// registers, while it waits at the cluster barrier that ends the previous
// sweep.  Per sweep: colour-1 sites, cluster barrier, colour-2 sites, cluster
// barrier; the rows just above and below a band are read from the
// neighbouring CTAs' shared memory (distributed shared memory).  During a
// colour phase a site reads only sites of the other colour, which no CTA
// writes in that phase, and the barriers order the phases, so the result is
// the lattice of the per-colour sweep: same per-site rule (update_philox),
// draws and neighbour order as every other sweep kernel.

#include <cooperative_groups.h>

#include <algorithm>

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

constexpr int kResidentMaxThreads = 512;
constexpr int kResidentMaxPairs = 4;              // x-pairs per thread
constexpr size_t kResidentMaxBytes = 64 * 1024;   // sites per CTA band

// shared memory of one CTA's band (its sites) in a cluster of cl CTAs
inline size_t resident_bytes(int spin_bytes, int64_t n, int cl) { return (size_t)(n / cl) * (size_t)spin_bytes; }

inline bool resident_fits(int spin_bytes, int nx, int ny, int cl) {
  const int64_t pairs = (int64_t)nx * ny / cl / 2;
  return ny % cl == 0 && ny >= cl && resident_bytes(spin_bytes, (int64_t)nx * ny, cl) <= kResidentMaxBytes &&
         pairs <= (int64_t)kResidentMaxThreads * kResidentMaxPairs;
}

bool resident_supported(int lattice, int app, int spin_bytes, int nx, int ny) {
  return fused2d_supported(lattice, app, spin_bytes, nx, ny) && (resident_fits(spin_bytes, nx, ny, 16) ||
                                                                 resident_fits(spin_bytes, nx, ny, 8));
}

// CL CTAs per cluster, P x-pairs per thread
template <typename S, int APP, int CL, int P>
__global__ void __launch_bounds__(kResidentMaxThreads) resident_sq4_kernel(ResidentArgs a) {
  extern __shared__ __align__(16) unsigned char resident_smem[];
  __shared__ uint64_t thr[5];
  __shared__ unsigned int red[kResidentMaxThreads / 32];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int nx = a.nx, ny = a.ny;
  const int R = ny / CL;  // rows of this band
  const int r0 = rank * R;
  const int nb_sites = R * nx, npairs = nb_sites / 2, hx = nx / 2;
  S *lat = (S *)resident_smem;
  // the neighbouring bands: last row of the band above, first row of the band below
  const S *up = cluster.map_shared_rank(lat, (unsigned)((rank + CL - 1) % CL)) + (R - 1) * nx;
  const S *dn = cluster.map_shared_rank(lat, (unsigned)((rank + 1) % CL));
  S *g = (S *)a.spin + (int64_t)r0 * nx;
  const int tid = threadIdx.x;
  if (tid < 5) thr[tid] = a.acc.thr[tid];
  for (int i = tid; i < nb_sites; i += blockDim.x) lat[i] = g[i];
  const RoundKeys rk = round_keys(a.seed, kStreamSweep);
  // pair q of this thread: band row ly, sites 2m and 2m+1; its colour-c
  // site at band index si[q][c] with its four neighbours' addresses
  int si[P][2], sl[P][2], sr[P][2];
  const S *pu[P][2], *pd[P][2];
  int64_t s_even[P];  // lattice index of the pair's even site
#pragma unroll
  for (int q = 0; q < P; q++) {
    const int pr = tid + (int)blockDim.x * q;
    s_even[q] = 0;
    si[q][0] = si[q][1] = -1;
    if (pr < npairs) {
      const int ly = pr / hx, m = pr - ly * hx, y = r0 + ly;
      s_even[q] = (int64_t)y * nx + 2 * m;
#pragma unroll
      for (int c = 0; c < 2; c++) {
        const int x = 2 * m + ((y + c) & 1), i = ly * nx + x;  // colour c+1: (x + y) & 1 == c
        si[q][c] = i;
        sl[q][c] = ly * nx + (x == 0 ? nx - 1 : x - 1);
        sr[q][c] = ly * nx + (x == nx - 1 ? 0 : x + 1);
        pu[q][c] = ly == 0 ? up + x : lat + i - nx;
        pd[q][c] = ly == R - 1 ? dn + x : lat + i + nx;
      }
    }
  }
  U4 w[P];  // the pair's Philox block of the current sweep
  auto draw = [&](uint32_t sweep) {
#pragma unroll
    for (int q = 0; q < P; q++) w[q] = philox4x32_10_rk(sweep_counter<APP>((uint64_t)s_even[q], sweep, 0u), rk);
  };
  draw(a.sweep0);
  cluster.sync();
  unsigned int changed = 0;
  for (int s = 0; s < a.nsweeps; s++) {
#pragma unroll
    for (int c = 0; c < 2; c++) {
#pragma unroll
      for (int q = 0; q < P; q++) {
        const int i = si[q][c];
        if (i >= 0) {
          // sq/4n neighbour order: x-1, y-1, y+1, x+1 (src/create_sites.cpp:1313-1330)
          const int nb[4] = {(int)lat[sl[q][c]], (int)*pu[q][c], (int)*pd[q][c], (int)lat[sr[q][c]]};
          const int own = (int)lat[i];
          uint32_t x0, x1;
          site_words<APP>(w[q], (uint64_t)(s_even[q] + (i & 1)), x0, x1);
          int e0;
          const int news = update_philox<4, APP>(own, nb, x0, x1, a.nspins, thr, &e0);
          if (news != own) {
            lat[i] = (S)news;
            changed++;
          }
        }
      }
      if (c == 0) {
        cluster.sync();
      } else {
        // the next sweep's blocks are this thread's own: drawn between its
        // arrival and the wait
        asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
        if (s + 1 < a.nsweeps) draw(a.sweep0 + (uint32_t)(s + 1));
        asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
      }
    }
  }
  for (int i = tid; i < nb_sites; i += blockDim.x) g[i] = lat[i];
  const unsigned int wsum = __reduce_add_sync(0xFFFFFFFFu, changed);
  if ((tid & 31) == 0) red[tid >> 5] = wsum;
  __syncthreads();
  if (tid == 0) {
    unsigned long long tot = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) tot += red[k];
    if (tot) atomicAdd(&a.naccept[rank & (kCounterSlots - 1)], tot);
  }
}

template <typename S, int APP, int CL, int P>
static cudaError_t launch_resident_cp(const ResidentArgs &a, int threads, size_t smem, cudaStream_t s) {
  auto f = resident_sq4_kernel<S, APP, CL, P>;
  cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kResidentMaxBytes);
  if (e == cudaSuccess && CL > 8) e = cudaFuncSetAttribute(f, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CL);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, f, a);
}

template <typename S, int APP, int CL>
static cudaError_t launch_resident_c(const ResidentArgs &a, int spin_bytes, cudaStream_t s) {
  const int pairs = a.nx * a.ny / CL / 2;
  const int threads = std::min(kResidentMaxThreads, (pairs + 31) / 32 * 32);
  const int per = (pairs + threads - 1) / threads;
  const size_t smem = resident_bytes(spin_bytes, (int64_t)a.nx * a.ny, CL);
  if (per <= 1) return launch_resident_cp<S, APP, CL, 1>(a, threads, smem, s);
  if (per <= 2) return launch_resident_cp<S, APP, CL, 2>(a, threads, smem, s);
  return launch_resident_cp<S, APP, CL, 4>(a, threads, smem, s);
}

// 16 CTAs where the rows divide and such a cluster can be scheduled, else 8
template <typename S, int APP>
static cudaError_t launch_resident_t(const ResidentArgs &a, int spin_bytes, cudaStream_t s) {
  if (resident_fits(spin_bytes, a.nx, a.ny, 16)) {
    const cudaError_t e = launch_resident_c<S, APP, 16>(a, spin_bytes, s);
    if (e == cudaSuccess || !resident_fits(spin_bytes, a.nx, a.ny, 8)) return e;
    cudaGetLastError();  // not launched: fall back to the portable cluster
  }
  return launch_resident_c<S, APP, 8>(a, spin_bytes, s);
}

template <typename S>
static cudaError_t launch_resident_s(int app, const ResidentArgs &a, int spin_bytes, cudaStream_t s) {
  switch (app) {
    case SPKGPU_ISING: return launch_resident_t<S, SPKGPU_ISING>(a, spin_bytes, s);
    case SPKGPU_POTTS: return launch_resident_t<S, SPKGPU_POTTS>(a, spin_bytes, s);
    case SPKGPU_POTTS_NEIGHONLY: return launch_resident_t<S, SPKGPU_POTTS_NEIGHONLY>(a, spin_bytes, s);
    case SPKGPU_POTTS_NEIGH: return launch_resident_t<S, SPKGPU_POTTS_NEIGH>(a, spin_bytes, s);
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
  switch (spin_bytes) {
    case 1: return launch_resident_s<int8_t>(app, a, spin_bytes, s);
    case 2: return launch_resident_s<int16_t>(app, a, spin_bytes, s);
    case 4: return launch_resident_s<int32_t>(app, a, spin_bytes, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace spk
