// Generic colour-phase sweep kernel: one launch updates every site of one
// colour inside one set (a sector of every processor sub-domain, or the whole
// lattice), the inner loop of AppLattice::iterate_rejection
// (src/app_lattice.cpp:672-690) with sweep_nomask_nostrict /
// sweep_mask_nostrict / sweep_nomask_strict / sweep_mask_strict
// (src/app_lattice.cpp:776-819).  Sites of one colour never neighbour each
// other (Lattice::ncolors, src/lattice.cpp:187-228), so all of them update
// in parallel with the same result as the reference's ascending loop.
//
// It covers every lattice, app, storage width, sector layout, processor grid,
// mask and RNG mode; the fused kernels in sweep_fused2d.cu take the common
// no-sector cases faster.

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "counters.cuh"
#include "site_update.cuh"
#include "spk_internal.h"

namespace spk {

template <typename S, int LAT, int APP>
__global__ void __launch_bounds__(256) phase_kernel(PhaseArgs a) {
  constexpr int NN = Stencil<LAT>::NN;
  __shared__ uint64_t thr[kMaxNeigh + 1];
  __shared__ double pexp[kMaxNeigh + 1];
  if (threadIdx.x <= kMaxNeigh) {
    thr[threadIdx.x] = a.acc.thr[threadIdx.x];
    pexp[threadIdx.x] = a.acc.pexp[threadIdx.x];
  }
  __syncthreads();
  S *spin = (S *)a.spin;
  int nxh = a.nxl[0] > a.nxl[1] ? a.nxl[0] : a.nxl[1];
  int64_t total = (int64_t)nxh * a.nyl * a.nzl;
  unsigned int changed_count = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    int ix = (int)(t % nxh);
    int64_t r = t / nxh;
    int iy = (int)(r % a.nyl);
    int iz = (int)(r / a.nyl);
    int y = a.yl[iy];
    int z = a.zl[iz];
    int q = a.xpar_fixed ? 0 : ((a.color - 1 + y + z) & 1);
    if (ix >= a.nxl[q]) continue;
    int x = a.xl[q][ix];
    int64_t i = (int64_t)x + (int64_t)a.nx * ((int64_t)y + (int64_t)a.ny * z);
    if (a.mask_on && a.mask[i]) continue;
    int own = (int)spin[i];
    int nb[NN];
#pragma unroll
    for (int j = 0; j < NN; j++) {
      int dx, dy, dz;
      Stencil<LAT>::offset(j, dx, dy, dz);
      nb[j] = (int)spin[wrap_index<LAT>(x, y, z, dx, dy, dz, a.nx, a.ny, a.nz)];
    }
    int news, e0;
    if (a.rng == SPKGPU_RNG_PHILOX) {
      U4 w = philox4x32_10(sweep_counter<APP>((uint64_t)i, a.sweep, a.pass), a.seed, kStreamSweep);
      uint32_t x0, x1;
      site_words<APP>(w, (uint64_t)i, x0, x1);
      news = update_philox<NN, APP>(own, nb, x0, x1, a.nspins, thr, &e0);
    } else {
      int pm = a.siteseeds[i];
      news = update_strict<NN, APP>(own, nb, pm, a.nspins, pexp, a.acc.zero_t, &e0);
      a.siteseeds[i] = pm;
    }
    if (news != own) {
      spin[i] = (S)news;
      changed_count++;
    }
    if (a.mask_on) {
      // AppIsing::site_event_rejection mask update (src/app_ising.cpp:131-135)
      if (2 * e0 < NN) a.mask[i] = 1;
      if (news != own) {
#pragma unroll
        for (int j = 0; j < NN; j++) {
          int dx, dy, dz;
          Stencil<LAT>::offset(j, dx, dy, dz);
          a.mask[wrap_index<LAT>(x, y, z, dx, dy, dz, a.nx, a.ny, a.nz)] = 0;
        }
      }
    }
  }
  block_count_add(a.naccept, changed_count);
}

template <typename S, int LAT>
static cudaError_t launch_phase_app(int app, const PhaseArgs &a, cudaStream_t s, int num_sms) {
  int nxh = a.nxl[0] > a.nxl[1] ? a.nxl[0] : a.nxl[1];
  int64_t total = (int64_t)nxh * a.nyl * a.nzl;
  if (total <= 0) return cudaSuccess;
  int64_t blocks = (total + 255) / 256;
  int64_t cap = (int64_t)num_sms * 8;
  if (blocks > cap) blocks = cap;
  dim3 grid((unsigned)blocks);
  switch (app) {
    case SPKGPU_ISING: phase_kernel<S, LAT, SPKGPU_ISING><<<grid, 256, 0, s>>>(a); break;
    case SPKGPU_POTTS: phase_kernel<S, LAT, SPKGPU_POTTS><<<grid, 256, 0, s>>>(a); break;
    case SPKGPU_POTTS_NEIGHONLY: phase_kernel<S, LAT, SPKGPU_POTTS_NEIGHONLY><<<grid, 256, 0, s>>>(a); break;
    case SPKGPU_POTTS_NEIGH: phase_kernel<S, LAT, SPKGPU_POTTS_NEIGH><<<grid, 256, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <typename S>
static cudaError_t launch_phase_lat(int lattice, int app, const PhaseArgs &a, cudaStream_t s, int num_sms) {
  switch (lattice) {
    case SPKGPU_SQ_4N: return launch_phase_app<S, SPKGPU_SQ_4N>(app, a, s, num_sms);
    case SPKGPU_SQ_8N: return launch_phase_app<S, SPKGPU_SQ_8N>(app, a, s, num_sms);
    case SPKGPU_SC_6N: return launch_phase_app<S, SPKGPU_SC_6N>(app, a, s, num_sms);
    case SPKGPU_SC_26N: return launch_phase_app<S, SPKGPU_SC_26N>(app, a, s, num_sms);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_phase(int lattice, int app, int spin_bytes, const PhaseArgs &a, cudaStream_t s,
                         int num_sms) {
  switch (spin_bytes) {
    case 1: return launch_phase_lat<int8_t>(lattice, app, a, s, num_sms);
    case 2: return launch_phase_lat<int16_t>(lattice, app, a, s, num_sms);
    case 4: return launch_phase_lat<int32_t>(lattice, app, a, s, num_sms);
  }
  return cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// mask clearing before a set is swept

template <int LAT>
__global__ void mask_clear_kernel(MaskClearArgs a) {
  constexpr int NN = Stencil<LAT>::NN;
  int64_t total = (int64_t)a.nxl * a.nyl * a.nzl;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    int x = a.xl[t % a.nxl];
    int64_t r = t / a.nxl;
    int y = a.yl[r % a.nyl];
    int z = a.zl[r / a.nyl];
    int64_t i = (int64_t)x + (int64_t)a.nx * ((int64_t)y + (int64_t)a.ny * z);
    if (a.color > 0) {
      if (Stencil<LAT>::color(x, y, z) == a.color) a.mask[i] = 0;
      continue;
    }
    int px = a.proc_x[x], py = a.proc_y[y], pz = a.proc_z[z];
    int hx = a.half_x[x], hy = a.half_y[y], hz = a.half_z[z];
    bool border = false;
#pragma unroll
    for (int j = 0; j < NN; j++) {
      int dx, dy, dz;
      Stencil<LAT>::offset(j, dx, dy, dz);
      int xn = x + dx, yn = y + dy, zn = z + dz;
      xn = xn < 0 ? xn + a.nx : (xn >= a.nx ? xn - a.nx : xn);
      yn = yn < 0 ? yn + a.ny : (yn >= a.ny ? yn - a.ny : yn);
      zn = Stencil<LAT>::k3d ? (zn < 0 ? zn + a.nz : (zn >= a.nz ? zn - a.nz : zn)) : 0;
      if (a.proc_x[xn] != px || a.proc_y[yn] != py || a.proc_z[zn] != pz || a.half_x[xn] != hx ||
          a.half_y[yn] != hy || a.half_z[zn] != hz)
        border = true;
    }
    if (border) a.mask[i] = 0;
  }
}

cudaError_t launch_mask_clear(int lattice, const MaskClearArgs &a, cudaStream_t s, int num_sms) {
  int64_t total = (int64_t)a.nxl * a.nyl * a.nzl;
  if (total <= 0) return cudaSuccess;
  int64_t blocks = (total + 255) / 256;
  if (blocks > (int64_t)num_sms * 8) blocks = (int64_t)num_sms * 8;
  switch (lattice) {
    case SPKGPU_SQ_4N: mask_clear_kernel<SPKGPU_SQ_4N><<<(unsigned)blocks, 256, 0, s>>>(a); break;
    case SPKGPU_SQ_8N: mask_clear_kernel<SPKGPU_SQ_8N><<<(unsigned)blocks, 256, 0, s>>>(a); break;
    case SPKGPU_SC_6N: mask_clear_kernel<SPKGPU_SC_6N><<<(unsigned)blocks, 256, 0, s>>>(a); break;
    case SPKGPU_SC_26N: mask_clear_kernel<SPKGPU_SC_26N><<<(unsigned)blocks, 256, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// total energy: sum over sites of the unlike-neighbour count
// (spparks_energy, src/library.cpp:140-146)

template <typename S, int LAT>
__global__ void energy_kernel(const S *spin, int nx, int ny, int nz, unsigned long long *out) {
  constexpr int NN = Stencil<LAT>::NN;
  int64_t n = (int64_t)nx * ny * nz;
  unsigned long long e = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int x = (int)(i % nx);
    int64_t r = i / nx;
    int y = (int)(r % ny);
    int z = (int)(r / ny);
    int own = spin[i];
#pragma unroll
    for (int j = 0; j < NN; j++) {
      int dx, dy, dz;
      Stencil<LAT>::offset(j, dx, dy, dz);
      e += (spin[wrap_index<LAT>(x, y, z, dx, dy, dz, nx, ny, nz)] != own);
    }
  }
  unsigned long long w = e;
  for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xFFFFFFFFu, w, o);
  if ((threadIdx.x & 31) == 0 && w) atomicAdd(out, w);
}

template <typename S>
static cudaError_t launch_energy_t(int lattice, const void *spin, int nx, int ny, int nz, unsigned long long *out,
                                   cudaStream_t s, int num_sms) {
  int64_t n = (int64_t)nx * ny * nz;
  int64_t blocks = (n + 255) / 256;
  if (blocks > (int64_t)num_sms * 8) blocks = (int64_t)num_sms * 8;
  const S *p = (const S *)spin;
  switch (lattice) {
    case SPKGPU_SQ_4N: energy_kernel<S, SPKGPU_SQ_4N><<<(unsigned)blocks, 256, 0, s>>>(p, nx, ny, nz, out); break;
    case SPKGPU_SQ_8N: energy_kernel<S, SPKGPU_SQ_8N><<<(unsigned)blocks, 256, 0, s>>>(p, nx, ny, nz, out); break;
    case SPKGPU_SC_6N: energy_kernel<S, SPKGPU_SC_6N><<<(unsigned)blocks, 256, 0, s>>>(p, nx, ny, nz, out); break;
    case SPKGPU_SC_26N: energy_kernel<S, SPKGPU_SC_26N><<<(unsigned)blocks, 256, 0, s>>>(p, nx, ny, nz, out); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_energy(int lattice, int spin_bytes, const void *spin, int nx, int ny, int nz,
                          unsigned long long *out, cudaStream_t s, int num_sms) {
  switch (spin_bytes) {
    case 1: return launch_energy_t<int8_t>(lattice, spin, nx, ny, nz, out, s, num_sms);
    case 2: return launch_energy_t<int16_t>(lattice, spin, nx, ny, nz, out, s, num_sms);
    case 4: return launch_energy_t<int32_t>(lattice, spin, nx, ny, nz, out, s, num_sms);
  }
  return cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// int32 <-> storage width, with the value check of AppIsing/AppPotts::init_app
// (src/app_ising.cpp:63-70, src/app_potts.cpp:78-84)

template <typename S>
__global__ void convert_in_kernel(const int32_t *src, S *dst, int64_t n, int nspins, int *bad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int v = src[i];
    if (v < 1 || v > nspins) *bad = 1;
    dst[i] = (S)v;
  }
}

template <typename S>
__global__ void convert_out_kernel(const S *src, int32_t *dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (int32_t)src[i];
}

// four sites per step, with 16-byte accesses on the int32 side: the int32
// side may be pinned host memory the kernel reads or writes directly
template <typename S>
__global__ void convert_in4_kernel(const int4 *src, S *dst, int64_t n4, int nspins, int *bad) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n4; q += (int64_t)gridDim.x * blockDim.x) {
    const int4 v = src[q];
    if (v.x < 1 || v.x > nspins || v.y < 1 || v.y > nspins || v.z < 1 || v.z > nspins || v.w < 1 || v.w > nspins)
      *bad = 1;
    if (sizeof(S) == 1) {
      ((uint32_t *)dst)[q] = (uint32_t)(uint8_t)v.x | ((uint32_t)(uint8_t)v.y << 8) |
                             ((uint32_t)(uint8_t)v.z << 16) | ((uint32_t)(uint8_t)v.w << 24);
    } else if (sizeof(S) == 2) {
      ((uint2 *)dst)[q] = make_uint2((uint32_t)(uint16_t)v.x | ((uint32_t)(uint16_t)v.y << 16),
                                     (uint32_t)(uint16_t)v.z | ((uint32_t)(uint16_t)v.w << 16));
    } else {
      ((int4 *)dst)[q] = v;
    }
  }
}

template <typename S>
__global__ void convert_out4_kernel(const S *src, int4 *dst, int64_t n4) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n4; q += (int64_t)gridDim.x * blockDim.x) {
    const S *p = src + 4 * q;
    dst[q] = make_int4((int)p[0], (int)p[1], (int)p[2], (int)p[3]);
  }
}

static unsigned convert_blocks(int64_t items) {
  int64_t b = (items + 255) / 256;
  return (unsigned)(b > 4096 ? 4096 : (b < 1 ? 1 : b));
}

cudaError_t launch_convert_in(int spin_bytes, const int32_t *src, void *dst, int64_t n, int nspins, int *bad,
                              cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (spin_bytes != 1 && spin_bytes != 2 && spin_bytes != 4) return cudaErrorInvalidValue;
  const int64_t n4 = (((uintptr_t)src & 15) == 0 && ((uintptr_t)dst & (4 * spin_bytes - 1)) == 0) ? n / 4 : 0;
  if (n4) {
    const int4 *s4 = (const int4 *)src;
    switch (spin_bytes) {
      case 1: convert_in4_kernel<int8_t><<<convert_blocks(n4), 256, 0, s>>>(s4, (int8_t *)dst, n4, nspins, bad); break;
      case 2: convert_in4_kernel<int16_t><<<convert_blocks(n4), 256, 0, s>>>(s4, (int16_t *)dst, n4, nspins, bad); break;
      case 4: convert_in4_kernel<int32_t><<<convert_blocks(n4), 256, 0, s>>>(s4, (int32_t *)dst, n4, nspins, bad); break;
    }
  }
  const int64_t r0 = 4 * n4, nr = n - r0;
  if (nr > 0) {
    const int32_t *sr = src + r0;
    char *dr = (char *)dst + r0 * spin_bytes;
    switch (spin_bytes) {
      case 1: convert_in_kernel<int8_t><<<convert_blocks(nr), 256, 0, s>>>(sr, (int8_t *)dr, nr, nspins, bad); break;
      case 2: convert_in_kernel<int16_t><<<convert_blocks(nr), 256, 0, s>>>(sr, (int16_t *)dr, nr, nspins, bad); break;
      case 4: convert_in_kernel<int32_t><<<convert_blocks(nr), 256, 0, s>>>(sr, (int32_t *)dr, nr, nspins, bad); break;
    }
  }
  return cudaGetLastError();
}

cudaError_t launch_convert_out(int spin_bytes, const void *src, int32_t *dst, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (spin_bytes != 1 && spin_bytes != 2 && spin_bytes != 4) return cudaErrorInvalidValue;
  const int64_t n4 = (((uintptr_t)dst & 15) == 0 && ((uintptr_t)src & (4 * spin_bytes - 1)) == 0) ? n / 4 : 0;
  if (n4) {
    int4 *d4 = (int4 *)dst;
    switch (spin_bytes) {
      case 1: convert_out4_kernel<int8_t><<<convert_blocks(n4), 256, 0, s>>>((const int8_t *)src, d4, n4); break;
      case 2: convert_out4_kernel<int16_t><<<convert_blocks(n4), 256, 0, s>>>((const int16_t *)src, d4, n4); break;
      case 4: convert_out4_kernel<int32_t><<<convert_blocks(n4), 256, 0, s>>>((const int32_t *)src, d4, n4); break;
    }
  }
  const int64_t r0 = 4 * n4, nr = n - r0;
  if (nr > 0) {
    const char *sr = (const char *)src + r0 * spin_bytes;
    int32_t *dr = dst + r0;
    switch (spin_bytes) {
      case 1: convert_out_kernel<int8_t><<<convert_blocks(nr), 256, 0, s>>>((const int8_t *)sr, dr, nr); break;
      case 2: convert_out_kernel<int16_t><<<convert_blocks(nr), 256, 0, s>>>((const int16_t *)sr, dr, nr); break;
      case 4: convert_out_kernel<int32_t><<<convert_blocks(nr), 256, 0, s>>>((const int32_t *)sr, dr, nr); break;
    }
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// seeded initial values: site s gets init_spin(seed, s, lo, hi), the Philox
// init stream (the role of `set site range lo hi`, src/set.cpp:582-760)

template <typename S>
__global__ void init_kernel(S *dst, int64_t n, uint32_t seed, int lo, int hi) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (S)init_spin(seed, (uint64_t)i, lo, hi);
}

__global__ void init_packed_kernel(uint64_t *dst, int64_t nwords, uint32_t seed) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nwords; t += (int64_t)gridDim.x * blockDim.x) {
    uint64_t v = 0;
    for (int b = 0; b < 64; b++) v |= (uint64_t)(init_spin(seed, (uint64_t)(t * 64 + b), 1, 2) == 2) << b;
    dst[t] = v;
  }
}

cudaError_t launch_init(int spin_bytes, void *dst, int64_t n, uint32_t seed, int lo, int hi, cudaStream_t s,
                        int num_sms) {
  int64_t blocks = std::min<int64_t>((n + 255) / 256, (int64_t)num_sms * 16);
  if (blocks < 1) blocks = 1;
  switch (spin_bytes) {
    case 1: init_kernel<int8_t><<<(unsigned)blocks, 256, 0, s>>>((int8_t *)dst, n, seed, lo, hi); break;
    case 2: init_kernel<int16_t><<<(unsigned)blocks, 256, 0, s>>>((int16_t *)dst, n, seed, lo, hi); break;
    case 4: init_kernel<int32_t><<<(unsigned)blocks, 256, 0, s>>>((int32_t *)dst, n, seed, lo, hi); break;
    case -1: init_packed_kernel<<<(unsigned)blocks, 256, 0, s>>>((uint64_t *)dst, n / 64, seed); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace spk
