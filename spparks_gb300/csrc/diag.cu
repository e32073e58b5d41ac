// Site diagnostics on the device, for the lattice a handle holds:
//
//   spkgpu_site_stats sum, minimum and maximum of the site values: `diag_style
//                     array i1 mean|sum|min|max` (DiagArray::compute,
//                     src/diag_array.cpp:107-200; mean = sum / nsites), Ising
//                     magnetisation m = 2 * mean - 3
//   spkgpu_clusters   `diag_style cluster` (DiagCluster::generate_clusters,
//                     src/diag_cluster.cpp:229-609): clusters are the
//                     connected components of equal site values over the
//                     lattice's neighbour list with periodic wrap
//                     (AppLattice::push_connected_neighbors,
//                     src/app_lattice.cpp:1187-1201); the reference prints
//                     Nclust, <N> = sum of volumes / Nclust and
//                     <R> = sum of volume^(1/dimension) / Nclust
//
// Clusters are labelled with a lock-free union-find: every site starts as
// its own root, each equal-valued neighbour pair (each unordered pair once,
// through the forward half of the stencil) is united by linking the larger
// root under the smaller with atomicMin, labels are flattened to their root,
// and roots are counted with their sizes.  Parents always have smaller
// indices than their children, so every walk ends within its start index;
// the walks still carry an explicit bound and report if it is ever hit.

#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <vector>

#include "counters.cuh"
#include "site_update.cuh"
#include "spk_internal.h"

namespace spk {

namespace {

template <typename S>
struct ByteSites {
  const S *p;
  __device__ int get(int64_t i) const { return (int)p[i]; }
};

// 64 Ising sites per word, bit = value - 1
struct PackedSites {
  const uint64_t *w;
  __device__ int get(int64_t i) const { return 1 + (int)((w[i >> 6] >> (i & 63)) & 1ull); }
};

inline unsigned grid_for(int64_t n, int num_sms) {
  int64_t b = (n + 255) / 256;
  int64_t cap = (int64_t)num_sms * 16;
  return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

template <class R>
__global__ void site_stats_kernel(R s, int64_t n, unsigned long long *sum, int *minmax) {
  unsigned long long acc = 0;
  int lo = 0x7FFFFFFF, hi = -0x7FFFFFFF - 1;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int v = s.get(i);
    acc += (unsigned long long)(long long)v;
    lo = v < lo ? v : lo;
    hi = v > hi ? v : hi;
  }
  for (int o = 16; o > 0; o >>= 1) {
    acc += __shfl_down_sync(0xFFFFFFFFu, acc, o);
    lo = min(lo, __shfl_down_sync(0xFFFFFFFFu, lo, o));
    hi = max(hi, __shfl_down_sync(0xFFFFFFFFu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    if (acc) atomicAdd(sum, acc);
    atomicMin(&minmax[0], lo);
    atomicMax(&minmax[1], hi);
  }
}

// root of x; a walk longer than `bound` sets *err and returns where it stopped
__device__ __forceinline__ int32_t uf_find(const int32_t *L, int32_t x, int64_t bound, int *err) {
  for (int64_t it = 0; it <= bound; it++) {
    int32_t p = *(const volatile int32_t *)&L[x];
    if (p == x) return x;
    x = p;
  }
  *err = 1;
  return x;
}

// link the clusters of a and b: the larger root goes under the smaller
__device__ __forceinline__ void uf_unite(int32_t *L, int32_t a, int32_t b, int64_t bound, int *err) {
  for (int64_t it = 0; it <= bound; it++) {
    a = uf_find(L, a, bound, err);
    b = uf_find(L, b, bound, err);
    if (a == b) return;
    if (a > b) {
      int32_t t = a;
      a = b;
      b = t;
    }
    // b is a root unless another thread linked it meanwhile: then retry from
    // what it points to now
    int32_t old = atomicMin(&L[b], a);
    if (old == b) return;
    b = old;
  }
  *err = 1;
}

__global__ void ccl_init_kernel(int32_t *L, int32_t *size, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    L[i] = (int32_t)i;
    size[i] = 0;
  }
}

// offsets j of the stencil that point "forward" (dz, dy, dx) > 0, so that
// every unordered neighbour pair is visited once
template <int LAT>
__device__ __forceinline__ bool forward(int j) {
  int dx, dy, dz;
  Stencil<LAT>::offset(j, dx, dy, dz);
  return dz > 0 || (dz == 0 && (dy > 0 || (dy == 0 && dx > 0)));
}

template <class R, int LAT>
__global__ void ccl_union_kernel(R s, int nx, int ny, int nz, int32_t *L, int *err) {
  constexpr int NN = Stencil<LAT>::NN;
  const int64_t n = (int64_t)nx * ny * nz;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % nx);
    const int64_t r = i / nx;
    const int y = (int)(r % ny);
    const int z = (int)(r / ny);
    const int own = s.get(i);
#pragma unroll
    for (int j = 0; j < NN; j++) {
      if (!forward<LAT>(j)) continue;
      int dx, dy, dz;
      Stencil<LAT>::offset(j, dx, dy, dz);
      const int64_t m = wrap_index<LAT>(x, y, z, dx, dy, dz, nx, ny, nz);
      if (m != i && s.get(m) == own) uf_unite(L, (int32_t)i, (int32_t)m, n, err);
    }
  }
}

// every label to its root, counting each cluster's sites at its root
__global__ void ccl_flatten_kernel(int32_t *L, int32_t *size, int64_t n, unsigned long long *nroot, int *err) {
  unsigned long long roots = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int32_t r = uf_find(L, (int32_t)i, n, err);
    atomicAdd(&size[r], 1);
    roots += (r == (int32_t)i);
  }
  for (int o = 16; o > 0; o >>= 1) roots += __shfl_down_sync(0xFFFFFFFFu, roots, o);
  if ((threadIdx.x & 31) == 0 && roots) atomicAdd(nroot, roots);
}

// per-block partial sums of size^invdim over the roots (the host adds the
// partials in block order, so the result does not depend on scheduling)
__global__ void ccl_radius_kernel(const int32_t *size, int64_t n, double invdim, double *partial) {
  __shared__ double red[8];
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int32_t v = size[i];
    if (v > 0) acc += invdim == 0.5 ? sqrt((double)v) : pow((double)v, invdim);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xFFFFFFFFu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += red[k];
    partial[blockIdx.x] = t;
  }
}

template <class R>
cudaError_t launch_union(int lattice, R s, int nx, int ny, int nz, int32_t *L, int *err, unsigned grid,
                         cudaStream_t st) {
  switch (lattice) {
    case SPKGPU_SQ_4N: ccl_union_kernel<R, SPKGPU_SQ_4N><<<grid, 256, 0, st>>>(s, nx, ny, nz, L, err); break;
    case SPKGPU_SQ_8N: ccl_union_kernel<R, SPKGPU_SQ_8N><<<grid, 256, 0, st>>>(s, nx, ny, nz, L, err); break;
    case SPKGPU_SC_6N: ccl_union_kernel<R, SPKGPU_SC_6N><<<grid, 256, 0, st>>>(s, nx, ny, nz, L, err); break;
    case SPKGPU_SC_26N: ccl_union_kernel<R, SPKGPU_SC_26N><<<grid, 256, 0, st>>>(s, nx, ny, nz, L, err); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace

}  // namespace spk

using namespace spk;

#define DIAG_CUDA(h, call)                                        \
  do {                                                            \
    cudaError_t c__ = (call);                                     \
    if (c__ != cudaSuccess) return spk_cuda_fail(h, c__, #call); \
  } while (0)

extern "C" {

int spkgpu_site_stats(spkgpu_lattice *h, int64_t *sum, int32_t *vmin, int32_t *vmax) {
  if (!h || !sum) return SPKGPU_ERR_ARG;
  // counter block: [3] sum, [6] {min, max} as two int32
  unsigned long long *acc = h->d_counters + 3;
  int *minmax = (int *)(h->d_counters + 6);
  DIAG_CUDA(h, cudaMemsetAsync(acc, 0, sizeof(unsigned long long), h->stream));
  DIAG_CUDA(h, cudaMemsetAsync(minmax, 0x7F, sizeof(int), h->stream));      // 0x7F7F7F7F
  DIAG_CUDA(h, cudaMemsetAsync(minmax + 1, 0x80, sizeof(int), h->stream));  // 0x80808080 < 0
  const unsigned g = grid_for(h->n, h->num_sms);
  if (h->packed)
    site_stats_kernel<<<g, 256, 0, h->stream>>>(PackedSites{(const uint64_t *)h->d_spin}, h->n, acc, minmax);
  else if (h->spin_bytes == 1)
    site_stats_kernel<<<g, 256, 0, h->stream>>>(ByteSites<int8_t>{(const int8_t *)h->d_spin}, h->n, acc, minmax);
  else if (h->spin_bytes == 2)
    site_stats_kernel<<<g, 256, 0, h->stream>>>(ByteSites<int16_t>{(const int16_t *)h->d_spin}, h->n, acc, minmax);
  else
    site_stats_kernel<<<g, 256, 0, h->stream>>>(ByteSites<int32_t>{(const int32_t *)h->d_spin}, h->n, acc, minmax);
  DIAG_CUDA(h, cudaGetLastError());
  h->launches++;
  unsigned long long v = 0;
  int mm[2] = {0, 0};
  DIAG_CUDA(h, cudaMemcpyAsync(&v, acc, sizeof(v), cudaMemcpyDeviceToHost, h->stream));
  DIAG_CUDA(h, cudaMemcpyAsync(mm, minmax, sizeof(mm), cudaMemcpyDeviceToHost, h->stream));
  DIAG_CUDA(h, cudaStreamSynchronize(h->stream));
  *sum = (int64_t)v;
  if (vmin) *vmin = mm[0];
  if (vmax) *vmax = mm[1];
  return SPKGPU_OK;
}

int spkgpu_clusters(spkgpu_lattice *h, int64_t *ncluster, double *mean_volume, double *mean_radius) {
  if (!h || !ncluster || !mean_volume || !mean_radius) return SPKGPU_ERR_ARG;
  if (h->n > 0x7FFFFFFFLL) return spk_fail(h, SPKGPU_ERR_TOO_LARGE, "cluster labels are 32-bit: at most 2^31-1 sites");
  const int64_t n = h->n;
  const unsigned g = grid_for(n, h->num_sms);
  // labels and sizes (2n int32), then one partial sum per block
  if (!h->d_labels) {
    const size_t words = ((size_t)n * 2 + 1) / 2;  // 8-byte words of the label area
    DIAG_CUDA(h, cudaMalloc(&h->d_labels, (words + (size_t)h->num_sms * 16) * 8));
  }
  int32_t *L = h->d_labels, *size = h->d_labels + n;
  double *partial = (double *)h->d_labels + ((size_t)n * 2 + 1) / 2;
  // scratch scalars of the counter block: [4] roots, [5] error flag
  unsigned long long *nroot = h->d_counters + 4;
  int *err = (int *)(h->d_counters + 5);
  DIAG_CUDA(h, cudaMemsetAsync(nroot, 0, 2 * sizeof(unsigned long long), h->stream));
  ccl_init_kernel<<<g, 256, 0, h->stream>>>(L, size, n);
  DIAG_CUDA(h, cudaGetLastError());
  const int nx = h->d.nx, ny = h->d.ny, nz = h->d.nz;
  cudaError_t e;
  if (h->packed)
    e = launch_union(h->d.lattice, PackedSites{(const uint64_t *)h->d_spin}, nx, ny, nz, L, err, g, h->stream);
  else if (h->spin_bytes == 1)
    e = launch_union(h->d.lattice, ByteSites<int8_t>{(const int8_t *)h->d_spin}, nx, ny, nz, L, err, g, h->stream);
  else if (h->spin_bytes == 2)
    e = launch_union(h->d.lattice, ByteSites<int16_t>{(const int16_t *)h->d_spin}, nx, ny, nz, L, err, g,
                     h->stream);
  else
    e = launch_union(h->d.lattice, ByteSites<int32_t>{(const int32_t *)h->d_spin}, nx, ny, nz, L, err, g,
                     h->stream);
  DIAG_CUDA(h, e);
  ccl_flatten_kernel<<<g, 256, 0, h->stream>>>(L, size, n, nroot, err);
  DIAG_CUDA(h, cudaGetLastError());
  const int dim = (h->d.lattice == SPKGPU_SC_6N || h->d.lattice == SPKGPU_SC_26N) ? 3 : 2;
  const double invdim = 1.0 / dim;  // DiagCluster: invdim = 1.0/domain->dimension
  ccl_radius_kernel<<<g, 256, 0, h->stream>>>(size, n, invdim, partial);
  DIAG_CUDA(h, cudaGetLastError());
  h->launches += 4;
  unsigned long long head[2] = {0, 0};
  std::vector<double> parts(g);
  DIAG_CUDA(h, cudaMemcpyAsync(head, nroot, sizeof(head), cudaMemcpyDeviceToHost, h->stream));
  DIAG_CUDA(h, cudaMemcpyAsync(parts.data(), partial, g * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  DIAG_CUDA(h, cudaStreamSynchronize(h->stream));
  int walk_err = 0;
  memcpy(&walk_err, &head[1], sizeof(walk_err));
  if (walk_err) return spk_fail(h, SPKGPU_ERR_DEVICE, "cluster labelling walk exceeded its bound");
  double rsum = 0.0;
  for (double p : parts) rsum += p;
  const int64_t nc = (int64_t)head[0];
  *ncluster = nc;
  *mean_volume = nc ? (double)n / (double)nc : 0.0;
  *mean_radius = nc ? rsum / (double)nc : 0.0;
  return SPKGPU_OK;
}

}  // extern "C"
