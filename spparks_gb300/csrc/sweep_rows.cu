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
// Staged rows hold one periodic-image column on each side of the row (so no
// neighbour index wraps), with the row's first site 16-byte aligned: rows
// whose length in bytes is a multiple of 16 arrive by 16-byte cp.async.
//
// The distinct-value list of potts/neighonly and potts/neigh
// (src/app_potts_neighonly.cpp:80-88) is built, when every value is below
// 128, with a stamp table: one byte per (value, thread), set to the site's
// stamp for the site's own value and then for each neighbour in order; a
// neighbour whose entry did not hold the stamp yet is a first appearance.
// The unlike counts then compare the neighbour values packed four per word.
// Larger values take the pairwise scan and per-neighbour compares.

#include <cuda_runtime.h>
#include <stdint.h>

#include "counters.cuh"
#include "site_update.cuh"
#include "spk_internal.h"

namespace spk {

// elements before a staged row's first site (16 bytes: the image of site
// nx-1 sits just before it, the image of site 0 just after site nx-1)
template <typename S>
__host__ __device__ constexpr int row_lead() {
  return 16 / (int)sizeof(S);
}

// staged row r (0..NROWS-1) of neighbour j of the row kernels' stencils:
// (dz+1)*3 + (dy+1) in 3d, dy+1 in 2d
template <int LAT>
__device__ __forceinline__ void row_of_neighbor(int j, int &r, int &dx) {
  int dy, dz;
  Stencil<LAT>::offset(j, dx, dy, dz);
  r = Stencil<LAT>::k3d ? (dz + 1) * 3 + (dy + 1) : dy + 1;
}

// position of set bit n (0-based, in ascending order) of m; n < popc(m)
__device__ __forceinline__ int nth_set_bit(uint32_t m, int n) {
  int pos = 0;
  int c = __popc(m & 0xFFFFu);
  if (n >= c) {
    n -= c;
    m >>= 16;
    pos += 16;
  }
  c = __popc(m & 0xFFu);
  if (n >= c) {
    n -= c;
    m >>= 8;
    pos += 8;
  }
  c = __popc(m & 0xFu);
  if (n >= c) {
    n -= c;
    m >>= 4;
    pos += 4;
  }
  c = __popc(m & 0x3u);
  if (n >= c) {
    n -= c;
    m >>= 2;
    pos += 2;
  }
  if (n >= (int)(m & 1u)) pos += 1;
  return pos;
}

// neighbour values below 128 packed four per word (bytes, neighbour order);
// the unused lanes of the last word hold 0, which no site value equals
template <int NN>
struct PackedNb {
  static constexpr int NW = (NN + 3) / 4;
  uint32_t w[NW];
};

template <int NN>
__device__ __forceinline__ PackedNb<NN> pack_neighbors(const int (&nb)[NN]) {
  PackedNb<NN> p;
#pragma unroll
  for (int k = 0; k < PackedNb<NN>::NW; k++) {
    const int j = 4 * k;
    // byte 1 of a value below 128 is 0: selector 1 fills the empty lanes
    const uint32_t lo = __byte_perm((uint32_t)nb[j], j + 1 < NN ? (uint32_t)nb[j + 1] : 0u, 0x1140u);
    const uint32_t hi = j + 2 < NN ? __byte_perm((uint32_t)nb[j + 2], j + 3 < NN ? (uint32_t)nb[j + 3] : 0u, 0x1140u)
                                   : 0u;
    p.w[k] = __byte_perm(lo, hi, 0x5410u);
  }
  return p;
}

// neighbours whose value differs from v (1..127): per byte lane, (b ^ v) is
// below 128, so adding 0x7F sets bit 7 exactly where it is non-zero and never
// carries into the next lane
template <int NN>
__device__ __forceinline__ int unlike_packed(const PackedNb<NN> &p, int v) {
  const uint32_t vv = (uint32_t)v * 0x01010101u;
  uint32_t acc = 0;
#pragma unroll
  for (int k = 0; k < PackedNb<NN>::NW; k++) acc += (((p.w[k] ^ vv) + 0x7F7F7F7Fu) & 0x80808080u) >> 7;
  return (int)((acc * 0x01010101u) >> 24) - (4 * PackedNb<NN>::NW - NN);  // empty lanes differ from every v
}

// first_appearance's result from the stamp table: tab + v * row_bytes is
// this thread's byte for value v
template <int NN>
__device__ __forceinline__ uint32_t first_appearance_stamped(int own, const int (&nb)[NN], unsigned char *tab,
                                                             int row_bytes, unsigned char stamp) {
  tab[own * row_bytes] = stamp;
  uint32_t first = 0;
#pragma unroll
  for (int j = 0; j < NN; j++) {
    unsigned char *e = tab + nb[j] * row_bytes;
    if (*e != stamp) first |= 1u << j;
    *e = stamp;
  }
  return first;
}

// the site's new value (src/app_ising.cpp:104-136, src/app_potts.cpp:112-146,
// src/app_potts_neighonly.cpp:71-117); pick_offset[j] is the staged-row
// offset of neighbour j from the site's position in row 0
template <typename S, int LAT, int APP, bool SMALLQ>
__device__ __forceinline__ int update_rows(int own, const int (&nb)[Stencil<LAT>::NN], uint32_t x0, uint32_t x1,
                                           int nspins, const uint64_t *thr, const S *site0, const int *pick_offset,
                                           unsigned char *tab, int row_bytes, unsigned char stamp) {
  constexpr int NN = Stencil<LAT>::NN;
  if (APP == SPKGPU_ISING || APP == SPKGPU_POTTS) {
    int e0;
    return update_philox<NN, APP>(own, nb, x0, x1, nspins, thr, &e0);
  }
  PackedNb<NN> pk;
  if (SMALLQ) pk = pack_neighbors<NN>(nb);
  const int e0 = SMALLQ ? unlike_packed<NN>(pk, own) : count_unlike<NN>(own, nb);
  // no unlike neighbour: no event and no draw (nevent == 0 below)
  if (e0 == 0) return own;
  const uint32_t first =
      SMALLQ ? first_appearance_stamped<NN>(own, nb, tab, row_bytes, stamp) : first_appearance<NN>(own, nb);
  const int nevent = __popc(first);
  uint32_t iran;
  if (APP == SPKGPU_POTTS_NEIGHONLY) {
    if (nevent == 0) return own;
    iran = scaled_pick((uint32_t)nevent, x0);
    if (iran > (uint32_t)(nevent - 1)) iran = nevent - 1;
  } else {
    iran = scaled_pick((uint32_t)NN, x0);
    if ((int)iran >= nevent) return own;
  }
  const int news = (int)site0[pick_offset[nth_set_bit(first, (int)iran)]];
  const int e1 = SMALLQ ? unlike_packed<NN>(pk, news) : count_unlike<NN>(news, nb);
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

// the stamp table of the distinct-value list: apps that build one, values below 128
template <int APP, bool SMALLQ>
__host__ __device__ constexpr bool row_stamps() {
  return SMALLQ && (APP == SPKGPU_POTTS_NEIGHONLY || APP == SPKGPU_POTTS_NEIGH);
}

// staged row pitch in elements: the row rounded up to 16 bytes plus a lead
// on each side, so every staged row starts at a multiple of 16 bytes
template <typename S>
__host__ __device__ __forceinline__ int row_pitch(int nx) {
  constexpr int LEAD = row_lead<S>();
  return (nx + LEAD - 1) / LEAD * LEAD + 2 * LEAD;
}

// bytes per value row of the stamp table: one per thread, in groups of four
// warps
__host__ __device__ __forceinline__ int stamp_row_bytes(int threads) { return (threads + 127) / 128 * 128; }

// shared memory of row_pair_kernel: the staged rows, then the stamp table
// ((nspins + 1) value rows)
template <typename S, int LAT>
inline size_t row_pair_smem(int nx, int threads, int nspins, bool stamps) {
  constexpr int NROWS = Stencil<LAT>::k3d ? 9 : 3;
  const size_t rows = (size_t)NROWS * row_pitch<S>(nx) * sizeof(S);
  const size_t tab = stamps ? (size_t)(nspins + 1) * stamp_row_bytes(threads) : 0;
  return rows + tab;
}

template <typename S, int LAT, int APP, bool SMALLQ>
__global__ void __launch_bounds__(512) row_pair_kernel(RowArgs a) {
  constexpr int NN = Stencil<LAT>::NN;
  constexpr int NROWS = Stencil<LAT>::k3d ? 9 : 3;
  constexpr int LEAD = row_lead<S>();
  constexpr bool STAMPS = row_stamps<APP, SMALLQ>();
  extern __shared__ __align__(16) unsigned char row_smem[];
  const int nx = a.nx;
  const int pitch = row_pitch<S>(nx);
  S *rows = (S *)row_smem;
  const size_t rows_bytes = (size_t)NROWS * pitch * sizeof(S);  // a multiple of 16
  const int t = threadIdx.x;
  // stamp table: value row v holds one byte per thread; the 32 lanes of a
  // warp use 32 distinct words of a row (no bank conflicts), four warps
  // share those words
  const int row_bytes = stamp_row_bytes(blockDim.x);
  unsigned char *tab = row_smem + rows_bytes + (t >> 7) * 128 + (t & 31) * 4 + ((t >> 5) & 3);
  if (STAMPS) {
    uint4 *z = (uint4 *)(row_smem + rows_bytes);
    const int n16 = (a.nspins + 1) * row_bytes / 16;
    for (int k = t; k < n16; k += blockDim.x) z[k] = make_uint4(0u, 0u, 0u, 0u);
  }
  __shared__ uint64_t thr[kMaxNeigh + 1];
  __shared__ int pick_offset[NN];  // staged offset of neighbour j from the site's position in row 0
  if (t <= kMaxNeigh) thr[t] = a.acc.thr[t];
  if (t < NN) {
    int r, dx;
    row_of_neighbor<LAT>(t, r, dx);
    pick_offset[t] = r * pitch + dx;
  }
  // this CTA's row
  const int rows_y = (a.ny - a.qy + 1) / 2;
  const int iy = blockIdx.x % rows_y, iz = blockIdx.x / rows_y;
  const int y = 2 * iy + a.qy;
  const int z = Stencil<LAT>::k3d ? 2 * iz + a.qz : 0;
  S *spin = (S *)a.spin;
  // the lattice row of staged row r
  auto row_src = [&](int r) {
    const int dy = Stencil<LAT>::k3d ? (r % 3) - 1 : r - 1;
    const int dz = Stencil<LAT>::k3d ? (r / 3) - 1 : 0;
    int yy = y + dy, zz = z + dz;
    yy = yy < 0 ? yy + a.ny : (yy >= a.ny ? yy - a.ny : yy);
    if (Stencil<LAT>::k3d) zz = zz < 0 ? zz + a.nz : (zz >= a.nz ? zz - a.nz : zz);
    return (const S *)(spin + ((int64_t)zz * a.ny + yy) * nx);
  };
  if ((nx * (int)sizeof(S)) % 16 == 0 && ((uintptr_t)spin & 15) == 0) {
    // 16-byte copies (rows of the lattice start at multiples of 16 bytes)
    const int cpr = nx / LEAD;  // chunks per row
    for (int k = t; k < NROWS * cpr; k += blockDim.x) {
      const int r = k / cpr, c = k - r * cpr;
      const unsigned sa = (unsigned)__cvta_generic_to_shared(rows + r * pitch + LEAD + c * LEAD);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(row_src(r) + c * LEAD) : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  } else {
    for (int r = 0; r < NROWS; r++) {
      const S *src = row_src(r);
      for (int x = t; x < nx; x += blockDim.x) rows[r * pitch + LEAD + x] = src[x];
    }
  }
  __syncthreads();
  if (t < 2 * NROWS) {  // the periodic images beside each row
    S *row = rows + (t >> 1) * pitch + LEAD;
    if (t & 1) row[nx] = row[0];
    else row[-1] = row[nx - 1];
  }
  __syncthreads();
  const int64_t rowbase = ((int64_t)z * a.ny + y) * nx;
  unsigned int changed = 0;
  const RoundKeys rk = round_keys(a.seed, kStreamSweep);
  // thread p owns the pair (2p, 2p+1); blockDim.x >= nx/2
  const int p = t;
  const bool active = 2 * p < nx;
  uint32_t keep0 = 0, keep1 = 0;
  const int crow = (NROWS / 2) * pitch + LEAD;  // the centre row's first site
#pragma unroll
  for (int half = 0; half < 2; half++) {
    if (active) {
      const int x = 2 * p + half;
      uint32_t x0, x1;
      if (half == 0) {
        const int64_t s = rowbase + 2 * p;
        const U4 w = philox4x32_10_rk(sweep_counter<APP>((uint64_t)s, a.sweep, 0u), rk);
        site_words<APP>(w, (uint64_t)s, x0, x1);
        site_words<APP>(w, (uint64_t)s + 1, keep0, keep1);
      } else {
        x0 = keep0;
        x1 = keep1;
      }
      const S *site0 = rows + LEAD + x;  // the site's position in staged row 0
      int nb[NN];
#pragma unroll
      for (int j = 0; j < NN; j++) {
        int r, dx;
        row_of_neighbor<LAT>(j, r, dx);
        nb[j] = site0[r * pitch + dx];
      }
      const int own = rows[crow + x];
      const int news = update_rows<S, LAT, APP, SMALLQ>(own, nb, x0, x1, a.nspins, thr, site0, pick_offset, tab,
                                                        row_bytes, (unsigned char)(half + 1));
      if (news != own) {
        rows[crow + x] = (S)news;
        // the images of sites 0 and nx-1 beside the centre row
        if (x == 0) rows[crow + nx] = (S)news;
        if (x == nx - 1) rows[crow - 1] = (S)news;
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
  int rows_y = (a.ny - a.qy + 1) / 2;
  int rows_z = Stencil<LAT>::k3d ? (a.nz - a.qz + 1) / 2 : 1;
  unsigned grid = (unsigned)(rows_y * rows_z);
  int threads = ((a.nx / 2 + 31) / 32) * 32;  // one x-pair per thread
  const bool stamps = smallq && (APP == SPKGPU_POTTS_NEIGHONLY || APP == SPKGPU_POTTS_NEIGH);
  const size_t smem = row_pair_smem<S, LAT>(a.nx, threads, a.nspins, stamps);
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
