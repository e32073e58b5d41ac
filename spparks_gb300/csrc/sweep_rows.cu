// Row-pair sweep for sq/8n and sc/26n (no sectors): one launch per pair of
// colours.  On these lattices colour = 4(z%2) + 2(y%2) + (x%2) + 1
// (Lattice::id2color, src/lattice.cpp:240-276), so colours 2k-1 and 2k are
// the even and odd x of the rows with one (y%2, z%2), and the only
// colour-(2k-1) neighbours of a colour-2k site are its two x-neighbours in
// the same row.  A CTA therefore sweeps whole x-rows: it stages the row and
// its 8 (3d) or 2 (2d) neighbouring rows in shared memory, updates the even
// sites, synchronises, then the odd sites - each thread owning one x-pair
// whose Philox block serves both of its sites (for ising the block holds the
// words of four sites; the pair's two are used).  Rows of other parities are
// not written during the launch, so the order equals the reference's colour
// order (src/app_lattice.cpp:672-680).
//
// The distinct-value list of potts/neighonly and potts/neigh
// (src/app_potts_neighonly.cpp:80-88) is built with a 128-bit seen-set in the
// thread's 16 bytes of shared memory when every value is below 128, else with
// the pairwise scan.

#include <cuda_runtime.h>
#include <stdint.h>

#include "counters.cuh"
#include "site_update.cuh"
#include "spk_internal.h"

namespace spk {

// the value of neighbour j of the site at column x of the centre row, read
// again from the staged rows (a runtime j: one shared-memory load instead of
// a select over every neighbour)
// (sq/8n and sc/26n: every offset in {-1,0,1}^d but 0, dx outer and dz
// inner, so offset j is cell m = j or j+1 of that cube)
template <typename S, int LAT>
__device__ __forceinline__ int staged_neighbor(const S *rows, int nx, int x, int j) {
  static_assert(LAT == SPKGPU_SQ_8N || LAT == SPKGPU_SC_26N, "row kernel lattices");
  constexpr int MID = Stencil<LAT>::k3d ? 13 : 4;
  const int m = j < MID ? j : j + 1;
  int dx, dy, dz;
  if (Stencil<LAT>::k3d) {
    dx = m / 9 - 1;
    dy = (m / 3) % 3 - 1;
    dz = m % 3 - 1;
  } else {
    dx = m / 3 - 1;
    dy = m % 3 - 1;
    dz = 0;
  }
  int xn = x + dx;
  xn = xn < 0 ? xn + nx : (xn >= nx ? xn - nx : xn);
  const int r = Stencil<LAT>::k3d ? (dz + 1) * 3 + (dy + 1) : dy + 1;
  return (int)rows[r * nx + xn];
}

// first-appearance mask of the distinct values != own among nb[] (values
// 1..127; first_appearance's result) from a 128-bit seen-set in this
// thread's four words of shared memory: a load, a test and a store per
// neighbour
template <int NN>
__device__ __forceinline__ uint32_t first_appearance_shared(int own, const int (&nb)[NN], uint32_t *seen) {
  *(uint4 *)seen = make_uint4(0u, 0u, 0u, 0u);
  seen[own >> 5] = 1u << (own & 31);
  uint32_t first = 0;
#pragma unroll
  for (int j = 0; j < NN; j++) {
    const int v = nb[j];
    const uint32_t b = 1u << (v & 31);
    const uint32_t cur = seen[v >> 5];
    first |= ((cur & b) ? 0u : 1u) << j;
    seen[v >> 5] = cur | b;
  }
  return first;
}

template <typename S, int LAT, int APP, bool SMALLQ>
__device__ __forceinline__ int update_rows(int own, const int (&nb)[Stencil<LAT>::NN], uint32_t x0, uint32_t x1,
                                           int nspins, const uint64_t *thr, const S *rows, int nx, int x,
                                           uint32_t *seen) {
  constexpr int NN = Stencil<LAT>::NN;
  if (APP == SPKGPU_ISING || APP == SPKGPU_POTTS) {
    int e0;
    return update_philox<NN, APP>(own, nb, x0, x1, nspins, thr, &e0);
  }
  int e0 = count_unlike<NN>(own, nb);
  // no unlike neighbour: no event and no draw (nevent == 0 below)
  if (e0 == 0) return own;
  uint32_t first = SMALLQ ? first_appearance_shared<NN>(own, nb, seen) : first_appearance<NN>(own, nb);
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
  int news = staged_neighbor<S, LAT>(rows, nx, x, __fns(first, 0, (int)iran + 1));
  int e1 = count_unlike<NN>(news, nb);
  if (e1 <= e0) return news;
  return ((uint64_t)x1 < thr[e1 - e0]) ? news : own;  // thr is all 0 at zero temperature
}

struct RowArgs {
  void *spin;
  int nx, ny, nz;
  int qy, qz;          // parity of the rows of this colour pair
  uint32_t seed, sweep;
  int nspins;
  unsigned long long *naccept;
  AcceptTable acc;
};

// rows staged: index (dz+1)*3 + (dy+1) for 3d, (dy+1) for 2d
template <typename S, int LAT, int APP, bool SMALLQ>
__global__ void __launch_bounds__(512) row_pair_kernel(RowArgs a) {
  constexpr int NN = Stencil<LAT>::NN;
  constexpr int NROWS = Stencil<LAT>::k3d ? 9 : 3;
  extern __shared__ __align__(16) unsigned char row_smem[];
  S *rows = (S *)row_smem;
  // 16 bytes of seen-set per thread after the rows (16-byte aligned)
  const size_t rows_bytes = ((size_t)NROWS * a.nx * sizeof(S) + 15) & ~(size_t)15;
  uint32_t *seen = (uint32_t *)(row_smem + rows_bytes) + 4 * threadIdx.x;
  __shared__ uint64_t thr[kMaxNeigh + 1];
  if (threadIdx.x <= kMaxNeigh) thr[threadIdx.x] = a.acc.thr[threadIdx.x];
  const int nx = a.nx;
  // this CTA's row
  int rows_y = (a.ny - a.qy + 1) / 2;
  int iy = blockIdx.x % rows_y, iz = blockIdx.x / rows_y;
  int y = 2 * iy + a.qy;
  int z = Stencil<LAT>::k3d ? 2 * iz + a.qz : 0;
  S *spin = (S *)a.spin;
  for (int r = 0; r < NROWS; r++) {
    int dy = Stencil<LAT>::k3d ? (r % 3) - 1 : r - 1;
    int dz = Stencil<LAT>::k3d ? (r / 3) - 1 : 0;
    int yy = y + dy, zz = z + dz;
    yy = yy < 0 ? yy + a.ny : (yy >= a.ny ? yy - a.ny : yy);
    if (Stencil<LAT>::k3d) zz = zz < 0 ? zz + a.nz : (zz >= a.nz ? zz - a.nz : zz);
    const S *src = spin + ((int64_t)zz * a.ny + yy) * nx;
    for (int x = threadIdx.x; x < nx; x += blockDim.x) rows[r * nx + x] = src[x];
  }
  __syncthreads();
  const int center = Stencil<LAT>::k3d ? 4 : 1;
  const int64_t rowbase = ((int64_t)z * a.ny + y) * nx;
  unsigned int changed = 0;
  const RoundKeys rk = round_keys(a.seed, kStreamSweep);
  // thread p owns the pair (2p, 2p+1); blockDim.x >= nx/2
  const int p = threadIdx.x;
  const bool active = 2 * p < nx;
  uint32_t keep0 = 0, keep1 = 0;
#pragma unroll
  for (int half = 0; half < 2; half++) {
    if (active) {
      int x = 2 * p + half;
      uint32_t x0, x1;
      if (half == 0) {
        int64_t s = rowbase + 2 * p;
        U4 w = philox4x32_10_rk(sweep_counter<APP>((uint64_t)s, a.sweep, 0u), rk);
        site_words<APP>(w, (uint64_t)s, x0, x1);
        site_words<APP>(w, (uint64_t)s + 1, keep0, keep1);
      } else {
        x0 = keep0;
        x1 = keep1;
      }
      int nb[NN];
#pragma unroll
      for (int j = 0; j < NN; j++) {
        int dx, dy, dz;
        Stencil<LAT>::offset(j, dx, dy, dz);
        int xn = x + dx;
        xn = xn < 0 ? xn + nx : (xn >= nx ? xn - nx : xn);
        int r = Stencil<LAT>::k3d ? (dz + 1) * 3 + (dy + 1) : dy + 1;
        nb[j] = rows[r * nx + xn];
      }
      int own = rows[center * nx + x];
      int news = update_rows<S, LAT, APP, SMALLQ>(own, nb, x0, x1, a.nspins, thr, rows, nx, x, seen);
      if (news != own) {
        rows[center * nx + x] = (S)news;
        spin[rowbase + x] = (S)news;
        changed++;
      }
    }
    __syncthreads();
  }
  block_count_add(a.naccept, changed);
}

bool rows_supported(int lattice, int spin_bytes, int nx, int nspins) {
  return (lattice == SPKGPU_SQ_8N || lattice == SPKGPU_SC_26N) && nx <= 1024 && nx % 2 == 0 &&
         (spin_bytes == 1 || spin_bytes == 2 || spin_bytes == 4) && nspins >= 1;
}

template <typename S, int LAT, int APP>
static cudaError_t launch_rows_app(const RowArgs &a, bool smallq, cudaStream_t st) {
  constexpr int NROWS = Stencil<LAT>::k3d ? 9 : 3;
  int rows_y = (a.ny - a.qy + 1) / 2;
  int rows_z = Stencil<LAT>::k3d ? (a.nz - a.qz + 1) / 2 : 1;
  unsigned grid = (unsigned)(rows_y * rows_z);
  int threads = ((a.nx / 2 + 31) / 32) * 32;  // one x-pair per thread
  size_t smem = (((size_t)NROWS * a.nx * sizeof(S) + 15) & ~(size_t)15) + (size_t)threads * 16;
  if (smallq) {
    auto f = row_pair_kernel<S, LAT, APP, true>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    f<<<grid, threads, smem, st>>>(a);
  } else {
    auto f = row_pair_kernel<S, LAT, APP, false>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    f<<<grid, threads, smem, st>>>(a);
  }
  return cudaGetLastError();
}

template <typename S, int LAT>
static cudaError_t launch_rows_lat(int app, const RowArgs &a, bool smallq, cudaStream_t st) {
  switch (app) {
    case SPKGPU_ISING: return launch_rows_app<S, LAT, SPKGPU_ISING>(a, smallq, st);
    case SPKGPU_POTTS: return launch_rows_app<S, LAT, SPKGPU_POTTS>(a, smallq, st);
    case SPKGPU_POTTS_NEIGHONLY: return launch_rows_app<S, LAT, SPKGPU_POTTS_NEIGHONLY>(a, smallq, st);
    case SPKGPU_POTTS_NEIGH: return launch_rows_app<S, LAT, SPKGPU_POTTS_NEIGH>(a, smallq, st);
  }
  return cudaErrorInvalidValue;
}

template <typename S>
static cudaError_t launch_rows_t(int lattice, int app, const RowArgs &a, bool smallq, cudaStream_t st) {
  if (lattice == SPKGPU_SQ_8N) return launch_rows_lat<S, SPKGPU_SQ_8N>(app, a, smallq, st);
  return launch_rows_lat<S, SPKGPU_SC_26N>(app, a, smallq, st);
}

// one sweep: colour pairs (1,2), (3,4)[, (5,6), (7,8)] in order
cudaError_t launch_rows_sweep(int lattice, int app, int spin_bytes, void *spin, int nx, int ny, int nz,
                              uint32_t seed, uint32_t sweep, int nspins, unsigned long long *naccept,
                              const AcceptTable &acc, cudaStream_t st, int *launches) {
  bool smallq = nspins <= 127;
  int npairs = lattice == SPKGPU_SC_26N ? 4 : 2;
  for (int cp = 0; cp < npairs; cp++) {
    RowArgs a;
    a.spin = spin;
    a.nx = nx;
    a.ny = ny;
    a.nz = nz;
    a.qy = cp & 1;
    a.qz = (cp >> 1) & 1;
    a.seed = seed;
    a.sweep = sweep;
    a.nspins = nspins;
    a.naccept = naccept;
    a.acc = acc;
    cudaError_t e;
    switch (spin_bytes) {
      case 1: e = launch_rows_t<int8_t>(lattice, app, a, smallq, st); break;
      case 2: e = launch_rows_t<int16_t>(lattice, app, a, smallq, st); break;
      case 4: e = launch_rows_t<int32_t>(lattice, app, a, smallq, st); break;
      default: return cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    (*launches)++;
  }
  return cudaSuccess;
}

}  // namespace spk
