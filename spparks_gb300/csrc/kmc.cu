// Rejection-free KMC with the tree solver over sectors: the device form of
// AppLattice::setup (KMC part, src/app_lattice.cpp:340-377) and
// AppLattice::iterate_kmc_sector (src/app_lattice.cpp:517-626) driving
// SolveTree (src/solve_tree.cpp:70-224) and the apps' site_propensity /
// site_event (src/app_potts.cpp:153-244, src/app_ising.cpp:143-196).
//
// Sets ("chains") are the sectors of every processor sub-domain of the
// `processors` grid; chain c = proc * nsector + (sector-1).  In one sector
// phase the chains of that sector index on all processors touch disjoint
// sites, so they run concurrently, one warp each - the reference's own
// parallel schedule, with the serial 1x1x1 grid as the special case.
//
// Per pass and sector phase:
//   border refresh   kmc_prop_kernel over the border sites of the phase's
//                    chains (site_propensity -> tree leaf)
//   tree rebuild     kmc_build_kernel: every internal node = left + right,
//                    bottom-up, and the count of positive leaves.  This is
//                    bit-identical to the reference's sequence of
//                    SolveTree::set calls: the last set() touching a node
//                    adds the final values of its two children.
//   event loop       kmc_event_kernel, one warp per chain: pick a leaf with
//                    find(u0*sum), clock -1/sum*log(u1), stop when the
//                    sector time reaches dt_kmc (that event discarded), else
//                    perform site_event (event choice u2*propensity),
//                    recompute the propensity of the site and its in-chain
//                    neighbours and re-add their ancestor paths.
// Philox draws: event k of chain c uses block (c, k): words 0, 1, 2.
// Propensities are FP64 (exp from a host table, same as the reference's
// exp) or FP32; tree sums, the root and the clock are FP64 always.

#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "site_update.cuh"
#include "spk_internal.h"

namespace spk {

struct KmcArgs {
  void *spin;
  int nx, ny, nz;
  int nspins;
  int zero_t;
  double pexp[kMaxNeigh + 1];   // exp(-dE/T), FP64
  float pexpf[kMaxNeigh + 1];   // the same in FP32
  const int32_t *setof;         // chain of each site
  const int32_t *i2site;        // index of each site within its chain
  const int32_t *site2i;        // sites of all chains, chain after chain
  const int64_t *c_site_off;    // first entry of chain c in site2i
  const int32_t *c_nloc;        // sites of chain c
  const int64_t *c_tree_off;    // first node of chain c's tree
  const int32_t *c_leaf0;       // leaf offset (nround-1) of chain c's tree
  const int32_t *c_ntotal;      // nodes of chain c's tree (2*nround-1)
  int32_t *c_nactive;           // positive leaves of chain c
  unsigned long long *c_events; // Philox event counter of chain c
  double *trees;
  unsigned long long *pmax_bits;  // max over chains of sum/num_active (as bits)
  unsigned long long *naccept;
  int nsector;
  int nprocs;
  uint32_t seed;
  double dt_kmc;
  int fp64;
  int smem_trees;               // 1: the event kernel copies trees to shared memory
  const int32_t *c_box;         // chain c's box: x0, y0, z0, wx, wy, wz (6 per chain)
};

template <int LAT>
__device__ __forceinline__ void site_coords(int64_t i, int nx, int ny, int &x, int &y, int &z) {
  x = (int)(i % nx);
  int64_t r = i / nx;
  y = (int)(r % ny);
  z = (int)(r / ny);
}

template <int LAT>
__device__ __forceinline__ int64_t neighbor_of(int x, int y, int z, int j, int nx, int ny, int nz) {
  int dx, dy, dz;
  Stencil<LAT>::offset(j, dx, dy, dz);
  int xn = x + dx, yn = y + dy, zn = z + dz;
  xn = xn < 0 ? xn + nx : (xn >= nx ? xn - nx : xn);
  yn = yn < 0 ? yn + ny : (yn >= ny ? yn - ny : yn);
  if (Stencil<LAT>::k3d) zn = zn < 0 ? zn + nz : (zn >= nz ? zn - nz : zn);
  else zn = 0;
  return (int64_t)xn + (int64_t)nx * ((int64_t)yn + (int64_t)ny * zn);
}

template <typename S, int LAT>
__device__ __forceinline__ void load_neighbors(const S *spin, int64_t i, int nx, int ny, int nz,
                                               int (&nb)[Stencil<LAT>::NN]) {
  int x, y, z;
  site_coords<LAT>(i, nx, ny, x, y, z);
#pragma unroll
  for (int j = 0; j < Stencil<LAT>::NN; j++) nb[j] = (int)spin[neighbor_of<LAT>(x, y, z, j, nx, ny, nz)];
}

// site_propensity: Ising flip (src/app_ising.cpp:143-163) or the sum over
// distinct unlike neighbour values (src/app_potts.cpp:153-189), summed in the
// reference's order
template <typename S, int LAT, int APP>
__device__ double site_propensity(const KmcArgs &a, const S *spin, int64_t i) {
  constexpr int NN = Stencil<LAT>::NN;
  int nb[NN];
  load_neighbors<S, LAT>(spin, i, a.nx, a.ny, a.nz, nb);
  int own = (int)spin[i];
  int e0 = count_unlike<NN>(own, nb);
  if (APP == SPKGPU_ISING) {
    int e1 = count_unlike<NN>(own == 1 ? 2 : 1, nb);
    if (e1 <= e0) return 1.0;
    if (a.zero_t) return 0.0;
    return a.fp64 ? a.pexp[e1 - e0] : (double)a.pexpf[e1 - e0];
  }
  uint32_t first = first_appearance<NN>(own, nb);
  if (a.fp64) {
    double prob = 0.0;
#pragma unroll
    for (int j = 0; j < NN; j++) {
      if (!((first >> j) & 1u)) continue;
      int e1 = count_unlike<NN>(nb[j], nb);
      if (e1 <= e0) prob += 1.0;
      else if (!a.zero_t) prob += a.pexp[e1 - e0];
    }
    return prob;
  }
  float prob = 0.0f;
#pragma unroll
  for (int j = 0; j < NN; j++) {
    if (!((first >> j) & 1u)) continue;
    int e1 = count_unlike<NN>(nb[j], nb);
    if (e1 <= e0) prob += 1.0f;
    else if (!a.zero_t) prob += a.pexpf[e1 - e0];
  }
  return (double)prob;
}

// propensities of listed sites (or all sites) into their tree leaves
template <typename S, int LAT, int APP>
__global__ void kmc_prop_kernel(KmcArgs a, const int32_t *list, int64_t nlist) {
  const S *spin = (const S *)a.spin;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nlist; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = list ? (int64_t)list[t] : t;
    int c = a.setof[i];
    a.trees[a.c_tree_off[c] + a.c_leaf0[c] + a.i2site[i]] = site_propensity<S, LAT, APP>(a, spin, i);
  }
}

// per-chain total propensity from the current lattice (the shadow of an
// FP32 run): site_propensity with FP64 (fp64 = 1) or FP32 Boltzmann factors,
// summed per chain in FP64 (sites of sector iset only, or all for iset < 0)
template <typename S, int LAT, int APP>
__global__ void kmc_sum64_kernel(KmcArgs a, double *chain_sum, int iset, int fp64) {
  const S *spin = (const S *)a.spin;
  a.fp64 = fp64;
  const int64_t n = (int64_t)a.nx * a.ny * a.nz;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int c = a.setof[i];
    if (iset >= 0 && c % a.nsector != iset) continue;
    const double p = site_propensity<S, LAT, APP>(a, spin, i);
    if (p != 0.0) atomicAdd(&chain_sum[c], p);
  }
}

// the root (total propensity) of every chain's tree, gathered
__global__ void kmc_roots_kernel(KmcArgs a, int nchains, double *out) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nchains; c += gridDim.x * blockDim.x)
    out[c] = a.trees[a.c_tree_off[c]];
}

// max over the chains of sector iset (all chains for iset < 0) of
// sum/num_active, into *bits (non-negative doubles order as their bits)
__global__ void kmc_pmax64_kernel(KmcArgs a, const double *chain_sum, int iset, int nt, unsigned long long *bits) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
    const int c = iset < 0 ? t : t * a.nsector + iset;
    const int na = a.c_nactive[c];
    if (na <= 0) continue;
    const double v = chain_sum[c] / na;
    atomicMax(bits, (unsigned long long)__double_as_longlong(v));
  }
}

// bottom-up rebuild of the trees of chains (proc*nsector + iset), one CTA
// per chain (iset < 0: every chain), and the count of positive leaves
__global__ void kmc_build_kernel(KmcArgs a, int iset) {
  int c = (iset < 0) ? blockIdx.x : blockIdx.x * a.nsector + iset;
  double *T = a.trees + a.c_tree_off[c];
  int leaf0 = a.c_leaf0[c];
  int ntotal = a.c_ntotal[c];
  // levels: internal nodes of depth d are [2^d - 1, 2^(d+1) - 1)
  int depth = 0;
  while ((1 << depth) - 1 < leaf0) depth++;
  for (int d = depth - 1; d >= 0; d--) {
    int lo = (1 << d) - 1, hi = (1 << (d + 1)) - 1;
    for (int p = lo + threadIdx.x; p < hi; p += blockDim.x) T[p] = T[2 * p + 1] + T[2 * p + 2];
    __syncthreads();
  }
  int cnt = 0;
  for (int p = leaf0 + threadIdx.x; p < ntotal; p += blockDim.x) cnt += T[p] > 0.0;
  cnt = __reduce_add_sync(0xFFFFFFFFu, cnt);
  __shared__ int red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int tot = 0;
    for (int w = 0; w < (int)(blockDim.x + 31) / 32; w++) tot += red[w];
    a.c_nactive[c] = tot;
  }
}

// a <= b for doubles that are both >= +0 (propensities, their sums, times):
// their bit patterns order as integers, and an integer compare keeps the
// scarce FP64 pipe for the arithmetic
__device__ __forceinline__ bool nonneg_le(double a, double b) {
  return __double_as_longlong(a) <= __double_as_longlong(b);
}

// SolveTree::find (src/solve_tree.cpp:207-224); value and the tree are >= 0
__device__ __forceinline__ int tree_find(const double *T, int leaf0, double value) {
  int i = 0;
  while (i < leaf0) {
    int left = 2 * i + 1;
    double tl = T[left];
    if (nonneg_le(value, tl)) i = left;
    else {
      value -= tl;
      i = left + 1;
    }
  }
  return i - leaf0;
}

// one warp per chain of sector iset: the event loop of iterate_kmc_sector
template <typename S, int LAT, int APP>
__global__ void __launch_bounds__(32) kmc_event_kernel(KmcArgs a, int iset) {
  constexpr int NN = Stencil<LAT>::NN;
  extern __shared__ double smem_tree[];
  const int lane = threadIdx.x;
  const int c = blockIdx.x * a.nsector + iset;
  S *spin = (S *)a.spin;
  double *G = a.trees + a.c_tree_off[c];
  const int leaf0 = a.c_leaf0[c];
  const int ntotal = a.c_ntotal[c];
  double *T = G;
  if (a.smem_trees) {
    for (int p = lane; p < ntotal; p += 32) smem_tree[p] = G[p];
    T = smem_tree;
    __syncwarp();
  }
  const int32_t *site2i = a.site2i + a.c_site_off[c];
  int nactive = a.c_nactive[c];
  unsigned long long k = a.c_events[c];
  double sum = T[0];
  // pmax = maximum sector propensity per active site (src/app_lattice.cpp:563-573)
  if (lane == 0 && nactive > 0) {
    double ptmp = sum / nactive;
    atomicMax(a.pmax_bits, (unsigned long long)__double_as_longlong(ptmp));
  }
  double timesector = 0.0;
  unsigned int done_events = 0;
  // the draws of the next 32 events, one per lane: the Philox block's pick
  // and event words and the clock's log(u), computed in one pass (the FP64
  // log is the costliest step of an event on this GPU)
  double pre_ux = 0.0, pre_uz = 0.0, pre_log = 0.0;
  int pre_left = 0;
  while (__double_as_longlong(sum) != 0) {  // sum >= 0
    if (pre_left == 0) {
      const U4 pw = kmc_block(a.seed, (uint32_t)c, k + (unsigned long long)lane);
      pre_ux = word_to_uniform(pw.x);
      pre_uz = word_to_uniform(pw.z);
      pre_log = log(word_to_uniform(pw.y));
      pre_left = 32;
    }
    const int slot = 32 - pre_left;
    pre_left--;
    const double ux = __shfl_sync(0xFFFFFFFFu, pre_ux, slot);
    const double uz = __shfl_sync(0xFFFFFFFFu, pre_uz, slot);
    const double lu = __shfl_sync(0xFFFFFFFFu, pre_log, slot);
    k++;
    int m = 0;
    if (lane == 0) m = tree_find(T, leaf0, ux * sum);
    m = __shfl_sync(0xFFFFFFFFu, m, 0);
    double dt = -1.0 / sum * lu;
    timesector += dt;
    if (nonneg_le(a.dt_kmc, timesector)) break;  // timesector >= dt_kmc
    int64_t i = site2i[m];
    int x, y, z;
    site_coords<LAT>(i, a.nx, a.ny, x, y, z);
    // site_event
    if (lane == 0) {
      int own = (int)spin[i];
      if (APP == SPKGPU_ISING) {
        spin[i] = (S)(own == 1 ? 2 : 1);
      } else {
        int nb[NN];
        load_neighbors<S, LAT>(spin, i, a.nx, a.ny, a.nz, nb);
        double threshhold = uz * T[leaf0 + m];
        int e0 = count_unlike<NN>(own, nb);
        uint32_t first = first_appearance<NN>(own, nb);
        int value = own;
        if (a.fp64) {
          double prob = 0.0;
          for (int j = 0; j < NN; j++) {
            if (!((first >> j) & 1u)) continue;
            value = nb[j];
            int e1 = count_unlike<NN>(value, nb);
            if (e1 <= e0) prob += 1.0;
            else if (!a.zero_t) prob += a.pexp[e1 - e0];
            if (nonneg_le(threshhold, prob)) break;  // prob >= threshhold
          }
        } else {
          float prob = 0.0f;
          for (int j = 0; j < NN; j++) {
            if (!((first >> j) & 1u)) continue;
            value = nb[j];
            int e1 = count_unlike<NN>(value, nb);
            if (e1 <= e0) prob += 1.0f;
            else if (!a.zero_t) prob += a.pexpf[e1 - e0];
            if (nonneg_le(threshhold, (double)prob)) break;
          }
        }
        spin[i] = (S)value;
      }
    }
    __syncwarp();
    // propensity of the site (entry 0) and its in-chain neighbours (1..NN)
    int64_t s = -1;
    if (lane == 0) s = i;
    else if (lane <= NN) {
      int64_t nbi = neighbor_of<LAT>(x, y, z, lane - 1, a.nx, a.ny, a.nz);
      if (a.setof[nbi] == c) s = nbi;
    }
    double p = 0.0;
    int leaf = -1;
    if (s >= 0) {
      p = site_propensity<S, LAT, APP>(a, spin, s);
      leaf = a.i2site[s];
    }
    // leaves in the reference's order (self, then neighbours in order);
    // num_active as SolveTree::set counts it
    for (int j = 0; j <= NN; j++) {
      int lj = __shfl_sync(0xFFFFFFFFu, leaf, j);
      double pj = __shfl_sync(0xFFFFFFFFu, p, j);
      if (lj < 0) continue;
      if (lane == 0) {
        // propensities are >= 0: positive <=> non-zero bits
        const double old = T[leaf0 + lj];
        nactive += (__double_as_longlong(pj) != 0) - (__double_as_longlong(old) != 0);
        T[leaf0 + lj] = pj;
      }
      __syncwarp();
    }
    // re-add the ancestor paths, level by level (lanes that share a node
    // write the same value)
    int node = leaf >= 0 ? leaf0 + leaf : -1;
    while (__any_sync(0xFFFFFFFFu, node > 0)) {
      if (node > 0) {
        int parent = (node - 1) >> 1;
        T[parent] = T[2 * parent + 1] + T[2 * parent + 2];
        node = parent;
      }
      __syncwarp();
    }
    sum = T[0];
    done_events++;
  }
  if (lane == 0) {
    a.c_events[c] = k;
    a.c_nactive[c] = nactive;
    if (done_events) atomicAdd(a.naccept, (unsigned long long)done_events);
  }
  if (a.smem_trees) {
    __syncwarp();
    for (int p = lane; p < ntotal; p += 32) G[p] = T[p];
  }
}


// ---------------------------------------------------------------------------
// Event loop with the tree in shared memory.
//
// The same events as kmc_event_kernel, with the memory round trips of an
// event cut from about forty dependent global loads to two:
//   * the top 14 levels of the chain's tree (16383 nodes, 128 KB) live in
//     shared memory for the whole sector phase (the whole tree when it has
//     at most 14 levels) and are written back at the end;
//   * below them, the descendants of the level-13 node the pick's walk
//     reaches (levels 14..D, a "slot") are fetched in one round trip; for
//     the changed leaves, each lane fetches its leaf's path below level 14
//     and the path's siblings (all that re-adding the path reads), together
//     with the site values the event reads;
//   * a site's chain and leaf index come from its coordinates: a chain is a
//     box (a processor sub-domain's sector half along each axis) and its
//     leaves follow ascending site order, so the leaf of (x, y, z) is its
//     rank in the box (AppLattice::create_set, src/app_lattice.cpp:954-1070);
//   * the site values within two steps of the event site (every value the
//     event and the 1 + NN propensities read) are fetched at once into
//     shared memory.
// Node values stay bit-identical: each changed leaf's ancestors are re-added
// as parent = left + right bottom-up (src/solve_tree.cpp:174-200), in shared
// memory, and written through to the global tree below level 14.
// Slot layout: a node n at depth j >= 1 below the level-13 node A sits at
// t = n - (A << j) - 1 (depth j holds 2^j nodes from t = 2^j - 2).

constexpr int kTopLevels = 14;
constexpr int kTopNodes = (1 << kTopLevels) - 1;  // levels 0..13

// shared memory (bytes) of kmc_tree_event_kernel for a tree of ntotal nodes
// on a lattice of NN neighbours and dim dimensions; 0 if it does not fit
inline size_t kmc_tree_smem_bytes(int ntotal, int nn, bool k3d, size_t limit) {
  const int blk = k3d ? 125 : 25;
  size_t top, slots = 0;
  if (ntotal <= kTopNodes) {
    top = (size_t)ntotal;
  } else {
    int nround = (ntotal + 1) / 2, depth = 0;
    while ((1 << depth) < nround) depth++;
    const int hb = depth - (kTopLevels - 1);
    top = (size_t)kTopNodes;
    slots = (size_t)(nn + 2) * (size_t)((2 << hb) - 2);
  }
  const size_t bytes = (top + slots) * 8 + (size_t)blk * 4;
  return bytes <= limit ? bytes : 0;
}

// 8-byte asynchronous copy global -> shared (no register round trip, so a
// lane's copies all fly at once); completed by cp_async_wait_all
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// issue the copy of the descendants of the level-13 node A (depths 1..hb)
// from the global tree G into slot S, all lanes
__device__ __forceinline__ void load_slot(const double *G, double *S, int A, int slotn, int lane) {
  for (int t = lane; t < slotn; t += 32) {
    const int j = 31 - __clz(t + 2);
    cp_async8(S + t, G + ((int64_t)A << j) + t + 1);
  }
}

// SolveTree::find (src/solve_tree.cpp:207-224) over `levels` levels of the
// heap T rooted at index 0 (children of u at 2u+1, 2u+2): returns the index
// reached and leaves the remaining value in `value`, bit for bit as the
// reference's walk.  Two levels per step: the left child and both
// grandchildren that can come next are read together, then the two
// decisions are taken in turn.  The walk is the same on every lane (no
// divergence, no broadcast afterwards).  Branch-free forms (the subtraction
// always issued, the compare selecting) and FP64 compares measured slower.
__device__ __forceinline__ int heap_walk(const double *T, int levels, double &value) {
  int u = 0;
  for (; levels >= 2; levels -= 2) {
    const int l = 2 * u + 1;
    const double tl = T[l], tll = T[2 * l + 1], trl = T[2 * l + 3];
    if (nonneg_le(value, tl)) {
      u = l;
      if (nonneg_le(value, tll)) u = 2 * l + 1;
      else {
        value -= tll;
        u = 2 * l + 2;
      }
    } else {
      value -= tl;
      u = l + 1;
      if (nonneg_le(value, trl)) u = 2 * l + 3;
      else {
        value -= trl;
        u = 2 * l + 4;
      }
    }
  }
  if (levels) {
    const int l = 2 * u + 1;
    const double tl = T[l];
    if (nonneg_le(value, tl)) u = l;
    else {
      value -= tl;
      u = l + 1;
    }
  }
  return u;
}

template <typename S, int LAT, int APP>
__global__ void __launch_bounds__(32) kmc_tree_event_kernel(KmcArgs a, int iset) {
  using St = Stencil<LAT>;
  constexpr int NN = St::NN;
  constexpr int BW = 5;                             // block edge: offsets -2..2
  constexpr int BLK = St::k3d ? BW * BW * BW : BW * BW;
  constexpr int NQ = (BLK + 31) / 32;               // block entries per lane
  constexpr int CTR = St::k3d ? 62 : 12;            // block index of offset (0,0,0)
  constexpr int NSLOT = NN + 2;                     // one per changed leaf, one for the pick
  constexpr unsigned FULL = 0xFFFFFFFFu;
  extern __shared__ double kmc_smem[];
  const int lane = threadIdx.x;
  const int c = blockIdx.x * a.nsector + iset;
  S *spin = (S *)a.spin;
  double *G = a.trees + a.c_tree_off[c];
  const int leaf0 = a.c_leaf0[c];
  const int ntotal = a.c_ntotal[c];
  const int depth = 31 - __clz(leaf0 + 1);          // leaves at level depth
  const bool whole = ntotal <= kTopNodes;
  const int ntop = whole ? ntotal : kTopNodes;
  const int hb = whole ? 0 : depth - (kTopLevels - 1);  // leaf depth below a level-13 node
  const int slotn = whole ? 0 : (2 << hb) - 2;
  double *top = kmc_smem;
  double *slots = top + ntop;
  int *blk = (int *)(slots + (size_t)NSLOT * slotn);
  const int *box = a.c_box + 6 * c;
  const int bx = box[0], by = box[1], bz = box[2], wx = box[3], wy = box[4], wz = box[5];
  // power-of-two box sides: a rank's coordinates by shifts and masks
  const bool pow2 = ((wx & (wx - 1)) == 0) && ((wy & (wy - 1)) == 0);
  const int lwx = __ffs(wx) - 1, lwy = __ffs(wy) - 1;

  for (int p = lane; p < ntop; p += 32) cp_async8(top + p, G + p);
  // the Boltzmann factors in shared memory: lanes index them with different
  // energy changes, which an indexed parameter load would serialise
  __shared__ double s_pexp[kMaxNeigh + 1];
  __shared__ float s_pexpf[kMaxNeigh + 1];
  if (lane <= kMaxNeigh) {
    s_pexp[lane] = a.zero_t ? 0.0 : a.pexp[lane];
    s_pexpf[lane] = a.zero_t ? 0.0f : a.pexpf[lane];
  }
  // this lane's changed site: 0 = the event site, j = neighbour j-1
  int odx = 0, ody = 0, odz = 0;
  if (lane >= 1 && lane <= NN) St::offset(lane - 1, odx, ody, odz);
  const int my_bo = odx + BW * ody + BW * BW * odz;  // its block offset from the centre
  // this lane's block entries t = lane + 32 q as offsets from the centre
  int bdx[NQ], bdy[NQ], bdz[NQ];
#pragma unroll
  for (int q = 0; q < NQ; q++) {
    const int t = lane + 32 * q;
    bdx[q] = t % BW - 2;
    bdy[q] = (t / BW) % BW - 2;
    bdz[q] = St::k3d ? t / (BW * BW) - 2 : 0;
  }
  cp_async_wait_all();
  __syncwarp();

  int nactive = a.c_nactive[c];
  unsigned long long k = a.c_events[c];
  double sum = top[0];
  if (lane == 0 && nactive > 0) {
    double ptmp = sum / nactive;
    atomicMax(a.pmax_bits, (unsigned long long)__double_as_longlong(ptmp));
  }
  double timesector = 0.0;
  unsigned int done_events = 0;
  double pre_ux = 0.0, pre_uz = 0.0, pre_log = 0.0;
  int pre_left = 0;
  while (__double_as_longlong(sum) != 0) {  // sum >= 0
    if (pre_left == 0) {
      const U4 pw = kmc_block(a.seed, (uint32_t)c, k + (unsigned long long)lane);
      pre_ux = word_to_uniform(pw.x);
      pre_uz = word_to_uniform(pw.z);
      pre_log = log(word_to_uniform(pw.y));
      pre_left = 32;
    }
    const int slot_no = 32 - pre_left;
    pre_left--;
    const double ux = __shfl_sync(FULL, pre_ux, slot_no);
    const double uz = __shfl_sync(FULL, pre_uz, slot_no);
    const double lu = __shfl_sync(FULL, pre_log, slot_no);
    k++;
    // the clock step does not depend on the pick (SolveTree::event,
    // src/solve_tree.cpp:130-143)
    const double dt = -1.0 / sum * lu;
    // SolveTree::find (src/solve_tree.cpp:207-224): through the cached
    // levels, then (below level 13) through the picked level-13 node's
    // descendants, fetched in one round trip; every lane walks
    double value = ux * sum;
    int node = heap_walk(top, whole ? depth : kTopLevels - 1, value);
    double *SF = slots + (size_t)(NSLOT - 1) * slotn;  // the pick's slot
    if (!whole) {
      load_slot(G, SF, node, slotn, lane);
      cp_async_wait_all();
      __syncwarp();
      // slot t holds the descendant at local heap index t + 1
      node = heap_walk(SF - 1, hb, value) + (node << hb);
    }
    const int m = node - leaf0;
    timesector += dt;
    if (nonneg_le(a.dt_kmc, timesector)) break;  // timesector >= dt_kmc
    const int pA = whole ? 0 : ((node + 1) >> hb) - 1;  // the pick's level-13 node
    // the site of leaf m: its rank in the chain's box
    int x, y, z;
    if (pow2) {
      x = bx + (m & (wx - 1));
      y = by + ((m >> lwx) & (wy - 1));
      z = bz + (m >> (lwx + lwy));
    } else {
      x = bx + m % wx;
      const int r = m / wx;
      y = by + r % wy;
      z = bz + r / wy;
    }
    const int64_t i = (int64_t)x + (int64_t)a.nx * ((int64_t)y + (int64_t)a.ny * z);
    // site values within two steps (wrapped): loads first, stores after
    int64_t bidx[NQ];
    int bval[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      bidx[q] = -1;
      if (lane + 32 * q < BLK) {
        bidx[q] = wrap_index<LAT>(x, y, z, bdx[q], bdy[q], bdz[q], a.nx, a.ny, a.nz);
        bval[q] = (int)spin[bidx[q]];
      }
    }
    // this lane's changed site: in the chain? its leaf, and its level-13 node
    bool mine = false;
    int leaf = -1, A = -1;
    if (lane <= NN) {
      int xs = x + odx, ys = y + ody, zs = z + odz;
      xs = xs < 0 ? xs + a.nx : (xs >= a.nx ? xs - a.nx : xs);
      ys = ys < 0 ? ys + a.ny : (ys >= a.ny ? ys - a.ny : ys);
      if (St::k3d) zs = zs < 0 ? zs + a.nz : (zs >= a.nz ? zs - a.nz : zs);
      else zs = 0;
      const unsigned ux_ = (unsigned)(xs - bx), uy_ = (unsigned)(ys - by), uz_ = (unsigned)(zs - bz);
      if (ux_ < (unsigned)wx && uy_ < (unsigned)wy && uz_ < (unsigned)wz) {
        mine = true;
        leaf = (int)((uz_ * (unsigned)wy + uy_) * (unsigned)wx + ux_);
        A = whole ? 0 : ((leaf0 + leaf + 1) >> hb) - 1;
      }
    }
    const int lnode = leaf0 + leaf;
    // one slot per distinct level-13 node, held by its lowest lane; each
    // lane fetches its own path below that node and the path's siblings
    // while the event is picked
    double *MS = slots;
    if (!whole) {
      const unsigned grp = __match_any_sync(FULL, mine ? A : -1);
      const int sl = mine ? __ffs(grp) - 1 : 0;  // a lane <= NN
      MS = slots + (size_t)sl * slotn;
      if (mine) {
        int nd = lnode;
        for (int j = hb; j >= 1; j--) {
          const int sib = (nd & 1) ? nd + 1 : nd - 1;
          cp_async8(MS + (nd - (A << j) - 1), G + nd);
          cp_async8(MS + (sib - (A << j) - 1), G + sib);
          nd = (nd - 1) >> 1;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < NQ; q++)
      if (bidx[q] >= 0) blk[lane + 32 * q] = bval[q];
    __syncwarp();
    // site_event (src/app_potts.cpp:196-244, src/app_ising.cpp:170-196):
    // lane j < NN computes the weight of neighbour j's value; the running
    // sum then takes the first appearances of values other than the site's
    // own in neighbour order, as the reference adds them, and stops at the
    // first that reaches the threshold
    int newv = 0;
    {
      const int own = blk[CTR];
      if (APP == SPKGPU_ISING) {
        newv = own == 1 ? 2 : 1;
      } else {
        int nb[NN];
#pragma unroll
        for (int j = 0; j < NN; j++) {
          int dx, dy, dz;
          St::offset(j, dx, dy, dz);
          nb[j] = blk[CTR + dx + BW * dy + BW * BW * dz];
        }
        const double pm = whole ? top[node] : SF[node - (pA << hb) - 1];
        const double threshhold = uz * pm;
        const int e0 = count_unlike<NN>(own, nb);
        const uint32_t first = first_appearance<NN>(own, nb);
        const int mv = lane < NN ? pick_value<NN>(nb, lane) : own;
        const int e1 = count_unlike<NN>(mv, nb);
        const bool live = lane < NN && ((first >> lane) & 1u);
        int val = own;
        // the running sum stops at the first value that reaches the
        // threshold (the same on every lane: a uniform branch)
        if (a.fp64) {
          const double term = !live ? 0.0 : (e1 <= e0 ? 1.0 : s_pexp[e1 - e0]);
          double tj[NN];
#pragma unroll
          for (int j = 0; j < NN; j++) tj[j] = __shfl_sync(FULL, term, j);
          double prob = 0.0;
#pragma unroll
          for (int j = 0; j < NN; j++) {
            if ((first >> j) & 1u) {
              prob += tj[j];
              val = nb[j];
              if (nonneg_le(threshhold, prob)) break;  // prob >= threshhold
            }
          }
        } else {
          const float term = !live ? 0.0f : (e1 <= e0 ? 1.0f : s_pexpf[e1 - e0]);
          float tj[NN];
#pragma unroll
          for (int j = 0; j < NN; j++) tj[j] = __shfl_sync(FULL, term, j);
          float prob = 0.0f;
#pragma unroll
          for (int j = 0; j < NN; j++) {
            if ((first >> j) & 1u) {
              prob += tj[j];
              val = nb[j];
              if (nonneg_le(threshhold, (double)prob)) break;
            }
          }
        }
        newv = val;
      }
      if (lane == 0) spin[i] = (S)newv;
    }
    // every block entry holding site i (more than one on periodic extents < 5)
#pragma unroll
    for (int q = 0; q < NQ; q++)
      if (bidx[q] == i) blk[lane + 32 * q] = newv;
    cp_async_wait_all();
    __syncwarp();
    // the propensity of this lane's site from the block
    double p = 0.0;
    if (mine) {
      const int cb = CTR + my_bo;
      const int own = blk[cb];
      int nb[NN];
#pragma unroll
      for (int j = 0; j < NN; j++) {
        int dx, dy, dz;
        St::offset(j, dx, dy, dz);
        nb[j] = blk[cb + dx + BW * dy + BW * BW * dz];
      }
      const int e0 = count_unlike<NN>(own, nb);
      if (APP == SPKGPU_ISING) {
        const int e1 = count_unlike<NN>(own == 1 ? 2 : 1, nb);
        p = e1 <= e0 ? 1.0 : (a.fp64 ? s_pexp[e1 - e0] : (double)s_pexpf[e1 - e0]);
      } else {
        // one pass over the neighbour pairs gives the first appearances and
        // each value's multiplicity (its unlike count is NN minus that);
        // the terms are then added in neighbour order, a value that is not a
        // first appearance adding 0 (p + 0 == p for p >= 0)
        uint32_t first = 0;
        int mult[NN];
#pragma unroll
        for (int j = 0; j < NN; j++) mult[j] = 1;
#pragma unroll
        for (int j = 0; j < NN; j++) {
          bool f = nb[j] != own;
#pragma unroll
          for (int q = 0; q < j; q++) {
            const bool eq = nb[q] == nb[j];
            f = f && !eq;
            mult[j] += eq;
            mult[q] += eq;
          }
          first |= (f ? 1u : 0u) << j;
        }
        if (a.fp64) {
          double t[NN];
#pragma unroll
          for (int j = 0; j < NN; j++) {
            const int e1 = NN - mult[j];
            t[j] = !((first >> j) & 1u) ? 0.0 : (e1 <= e0 ? 1.0 : s_pexp[max(e1 - e0, 0)]);
          }
#pragma unroll
          for (int j = 0; j < NN; j++) p += t[j];
        } else {
          float t[NN];
#pragma unroll
          for (int j = 0; j < NN; j++) {
            const int e1 = NN - mult[j];
            t[j] = !((first >> j) & 1u) ? 0.0f : (e1 <= e0 ? 1.0f : s_pexpf[max(e1 - e0, 0)]);
          }
          float pf = 0.0f;
#pragma unroll
          for (int j = 0; j < NN; j++) pf += t[j];
          p = (double)pf;
        }
      }
    }
    // the leaves (a leaf reached by several lanes is set once: the values
    // agree), num_active as SolveTree::set counts it
    const unsigned lgrp = __match_any_sync(FULL, mine ? leaf : -1);
    const bool setter = mine && (__ffs(lgrp) - 1) == lane;
    int dact = 0;
    if (setter) {
      double *lp = whole ? &top[lnode] : &MS[lnode - (A << hb) - 1];
      dact = (__double_as_longlong(p) != 0) - (__double_as_longlong(*lp) != 0);
      *lp = p;
      if (!whole) G[lnode] = p;
    }
    nactive += __reduce_add_sync(FULL, dact);
    __syncwarp();
    // ancestors: below level 14 in the slots (written through to G), then
    // the cached levels; lanes on a shared path write equal values
    int nd = lnode;
    if (!whole) {
      for (int j = hb - 1; j >= 1; j--) {
        if (mine) {
          nd = (nd - 1) >> 1;
          const int tl = 2 * nd + 1 - (A << (j + 1)) - 1;
          const double v = MS[tl] + MS[tl + 1];
          MS[nd - (A << j) - 1] = v;
          G[nd] = v;
        }
        __syncwarp();
      }
      if (mine) {
        nd = A;
        top[A] = MS[0] + MS[1];
      }
      __syncwarp();
    }
    // cached levels: in step up to the lowest common ancestor of the changed
    // leaves (kmerge levels above the leaves), then lane 0 (whose path every
    // other path has joined) alone, with the siblings fetched first
    const unsigned lmin = __reduce_min_sync(FULL, mine ? (unsigned)leaf : 0xFFFFFFFFu);
    const unsigned lmax = __reduce_max_sync(FULL, mine ? (unsigned)leaf : 0u);
    const int kmerge = lmin == lmax ? 0 : 32 - __clz(lmin ^ lmax);
    const int steps = whole ? kmerge : max(0, kmerge - hb);
    for (int q = 0; q < steps; q++) {
      if (mine) {
        nd = (nd - 1) >> 1;
        top[nd] = top[2 * nd + 1] + top[2 * nd + 2];
      }
      __syncwarp();
    }
    // the single path above the common ancestor: lane q fetches the sibling
    // q levels up, then every lane adds them in turn (the same sums on every
    // lane, lane 0 stores them); lane 0 is always on the path
    const int top_nd = __shfl_sync(FULL, nd, 0);
    const int lev = 31 - __clz(top_nd + 1);  // levels above it, the same on every lane
    double sib = 0.0;
    if (lane < lev) {
      const int anc = ((top_nd + 1) >> lane) - 1;
      sib = top[(anc & 1) ? anc + 1 : anc - 1];
    }
    double v = top[top_nd];
    int n = top_nd;
#pragma unroll
    for (int q = 0; q < kTopLevels; q++) {
      if (q < lev) {
        const double sq = __shfl_sync(FULL, sib, q);
        const bool left = n & 1;
        n = (n - 1) >> 1;
        v = left ? v + sq : sq + v;
        if (lane == 0) top[n] = v;
      }
    }
    sum = v;
    __syncwarp();
    done_events++;
  }
  __syncwarp();
  for (int p = lane; p < ntop; p += 32) G[p] = top[p];
  if (lane == 0) {
    a.c_events[c] = k;
    a.c_nactive[c] = nactive;
    if (done_events) atomicAdd(a.naccept, (unsigned long long)done_events);
  }
}

}  // namespace spk

using namespace spk;

struct KmcState {
  int ready = 0;
  int adapt = 1;
  double nstop = 1.0, tstop = 0.0;
  int fp64 = 1;
  int nchains = 0;
  int64_t nsites = 0;
  double dt_kmc = 0.0;
  int64_t naccept_base = 0;
  int64_t npass = 0;
  int max_ntotal = 0;
  std::vector<int64_t> border_off;  // per sector: offset into border list (nsector+1)
  int32_t *d_setof = nullptr, *d_i2site = nullptr, *d_site2i = nullptr, *d_border = nullptr;
  int32_t *d_box = nullptr;         // chain boxes (6 per chain)
  bool boxes = false;               // every chain is a box in ascending site order
  size_t tree_smem = 0;             // shared memory of kmc_tree_event_kernel (0: global-tree kernel)
  int64_t *d_site_off = nullptr, *d_tree_off = nullptr;
  int32_t *d_nloc = nullptr, *d_leaf0 = nullptr, *d_ntotal = nullptr, *d_nactive = nullptr;
  unsigned long long *d_events = nullptr;
  double *d_trees = nullptr;
  unsigned long long *d_scalars = nullptr;  // [0] pmax bits, [1] naccept
  std::vector<int32_t> h_nactive;
  // FP32 runs with the FP64 shadow (fp64 == 0): per-chain FP64 sums
  int shadow = 0;
  int in_run = 0;             // a run paused at an output time can continue
  double *d_sum64 = nullptr;
  double dt_rel_err = 0.0;    // max relative error of dt_kmc = nstop/pmax against FP64, last run
};

void spk_kmc_free(spkgpu_lattice *h) {
  if (!h || !h->kmc) return;
  KmcState *k = h->kmc;
  cudaFree(k->d_setof);
  cudaFree(k->d_i2site);
  cudaFree(k->d_site2i);
  cudaFree(k->d_border);
  cudaFree(k->d_box);
  cudaFree(k->d_site_off);
  cudaFree(k->d_tree_off);
  cudaFree(k->d_nloc);
  cudaFree(k->d_leaf0);
  cudaFree(k->d_ntotal);
  cudaFree(k->d_nactive);
  cudaFree(k->d_events);
  cudaFree(k->d_trees);
  cudaFree(k->d_scalars);
  cudaFree(k->d_sum64);
  delete k;
  h->kmc = nullptr;
}

#define KMC_CUDA(h, call)                                   \
  do {                                                      \
    cudaError_t e__ = (call);                               \
    if (e__ != cudaSuccess) return spk_cuda_fail(h, e__, #call); \
  } while (0)

static KmcArgs kmc_args(spkgpu_lattice *h) {
  KmcState *k = h->kmc;
  KmcArgs a;
  memset(&a, 0, sizeof(a));
  a.spin = h->d_spin;
  a.nx = h->d.nx;
  a.ny = h->d.ny;
  a.nz = h->d.nz;
  a.nspins = h->d.nspins;
  a.zero_t = h->acc.zero_t;
  for (int d = 0; d <= kMaxNeigh; d++) {
    a.pexp[d] = h->acc.pexp[d];
    a.pexpf[d] = (float)h->acc.pexp[d];
  }
  a.setof = k->d_setof;
  a.i2site = k->d_i2site;
  a.site2i = k->d_site2i;
  a.c_site_off = k->d_site_off;
  a.c_nloc = k->d_nloc;
  a.c_tree_off = k->d_tree_off;
  a.c_leaf0 = k->d_leaf0;
  a.c_ntotal = k->d_ntotal;
  a.c_nactive = k->d_nactive;
  a.c_events = k->d_events;
  a.trees = k->d_trees;
  a.pmax_bits = k->d_scalars;
  a.naccept = k->d_scalars + 1;
  a.nsector = h->d.nsector;
  a.nprocs = k->nchains / h->d.nsector;
  a.seed = h->d.seed;
  a.dt_kmc = k->dt_kmc;
  a.fp64 = k->fp64;
  a.smem_trees = ((size_t)k->max_ntotal * 8 <= 48 * 1024) ? 1 : 0;
  a.c_box = k->d_box;
  return a;
}

template <typename S, int LAT>
static cudaError_t launch_prop_t(int app, const KmcArgs &a, const int32_t *list, int64_t n, cudaStream_t s, int sms) {
  if (n <= 0) return cudaSuccess;
  int64_t blocks = std::min<int64_t>((n + 127) / 128, (int64_t)sms * 16);
  if (app == SPKGPU_ISING) kmc_prop_kernel<S, LAT, SPKGPU_ISING><<<(unsigned)blocks, 128, 0, s>>>(a, list, n);
  else kmc_prop_kernel<S, LAT, SPKGPU_POTTS><<<(unsigned)blocks, 128, 0, s>>>(a, list, n);
  return cudaGetLastError();
}

template <typename S, int LAT>
static cudaError_t launch_sum64_t(int app, const KmcArgs &a, double *chain_sum, int iset, int fp64, int64_t n,
                                  cudaStream_t s, int sms) {
  int64_t blocks = std::min<int64_t>((n + 255) / 256, (int64_t)sms * 16);
  if (app == SPKGPU_ISING)
    kmc_sum64_kernel<S, LAT, SPKGPU_ISING><<<(unsigned)blocks, 256, 0, s>>>(a, chain_sum, iset, fp64);
  else
    kmc_sum64_kernel<S, LAT, SPKGPU_POTTS><<<(unsigned)blocks, 256, 0, s>>>(a, chain_sum, iset, fp64);
  return cudaGetLastError();
}

template <typename S, int LAT>
static cudaError_t launch_events_t(int app, const KmcArgs &a, int iset, int nprocs, size_t smem, size_t tree_smem,
                                   cudaStream_t s) {
  if (tree_smem) {
    auto f = app == SPKGPU_ISING ? kmc_tree_event_kernel<S, LAT, SPKGPU_ISING> : kmc_tree_event_kernel<S, LAT, SPKGPU_POTTS>;
    if (tree_smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tree_smem);
      if (e != cudaSuccess) return e;
    }
    f<<<nprocs, 32, tree_smem, s>>>(a, iset);
    return cudaGetLastError();
  }
  if (app == SPKGPU_ISING) {
    auto f = kmc_event_kernel<S, LAT, SPKGPU_ISING>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    f<<<nprocs, 32, smem, s>>>(a, iset);
  } else {
    auto f = kmc_event_kernel<S, LAT, SPKGPU_POTTS>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    f<<<nprocs, 32, smem, s>>>(a, iset);
  }
  return cudaGetLastError();
}

template <typename S>
static cudaError_t dispatch_lat(int lattice, int app, int what, const KmcArgs &a, const int32_t *list, int64_t n,
                                int iset, int nprocs, size_t smem, size_t tree_smem, cudaStream_t s, int sms) {
#define SPK_KMC_CASE(LATV)                                                                   \
  case LATV:                                                                                 \
    return what == 0 ? launch_prop_t<S, LATV>(app, a, list, n, s, sms)                       \
                     : launch_events_t<S, LATV>(app, a, iset, nprocs, smem, tree_smem, s);
  switch (lattice) {
    SPK_KMC_CASE(SPKGPU_SQ_4N)
    SPK_KMC_CASE(SPKGPU_SQ_8N)
    SPK_KMC_CASE(SPKGPU_SC_6N)
    SPK_KMC_CASE(SPKGPU_SC_26N)
  }
#undef SPK_KMC_CASE
  return cudaErrorInvalidValue;
}

template <typename S>
static cudaError_t sum64_lat(int lattice, int app, const KmcArgs &a, double *chain_sum, int iset, int fp64,
                             int64_t n, cudaStream_t s, int sms) {
  switch (lattice) {
    case SPKGPU_SQ_4N: return launch_sum64_t<S, SPKGPU_SQ_4N>(app, a, chain_sum, iset, fp64, n, s, sms);
    case SPKGPU_SQ_8N: return launch_sum64_t<S, SPKGPU_SQ_8N>(app, a, chain_sum, iset, fp64, n, s, sms);
    case SPKGPU_SC_6N: return launch_sum64_t<S, SPKGPU_SC_6N>(app, a, chain_sum, iset, fp64, n, s, sms);
    case SPKGPU_SC_26N: return launch_sum64_t<S, SPKGPU_SC_26N>(app, a, chain_sum, iset, fp64, n, s, sms);
  }
  return cudaErrorInvalidValue;
}

// the all-FP64 shadow of the propensity sums of the chains of sector iset
// (every chain for iset < 0) at this point of the run: their sums into
// k->d_sum64 and max(sum/num_active) into k->d_scalars[2] (bits, max-ed)
static cudaError_t kmc_shadow64(spkgpu_lattice *h, const KmcArgs &a, int iset, int fp64 = 1) {
  KmcState *k = h->kmc;
  const int nprocs = k->nchains / h->d.nsector;
  cudaError_t e = cudaErrorInvalidValue;
  double *cs = k->d_sum64;
  switch (h->spin_bytes) {
    case 1: e = sum64_lat<int8_t>(h->d.lattice, h->d.app, a, cs, iset, fp64, h->n, h->stream, h->num_sms); break;
    case 2: e = sum64_lat<int16_t>(h->d.lattice, h->d.app, a, cs, iset, fp64, h->n, h->stream, h->num_sms); break;
    case 4: e = sum64_lat<int32_t>(h->d.lattice, h->d.app, a, cs, iset, fp64, h->n, h->stream, h->num_sms); break;
  }
  if (e != cudaSuccess) return e;
  const int nt = iset < 0 ? k->nchains : nprocs;
  kmc_pmax64_kernel<<<(nt + 255) / 256, 256, 0, h->stream>>>(a, k->d_sum64, iset, nt, k->d_scalars + 2);
  h->launches += 2;
  return cudaGetLastError();
}

// the chains' roots in chain order (through the shadow buffer as scratch)
static int kmc_roots(spkgpu_lattice *h, const KmcArgs &a, std::vector<double> &roots) {
  KmcState *k = h->kmc;
  roots.resize(k->nchains);
  kmc_roots_kernel<<<(k->nchains + 255) / 256, 256, 0, h->stream>>>(a, k->nchains, k->d_sum64);
  h->launches++;
  KMC_CUDA(h, cudaGetLastError());
  KMC_CUDA(h, cudaMemcpyAsync(roots.data(), k->d_sum64, k->nchains * sizeof(double), cudaMemcpyDeviceToHost,
                              h->stream));
  KMC_CUDA(h, cudaStreamSynchronize(h->stream));
  return SPKGPU_OK;
}

// the shadow's pmax (as max-ed since the last clear) and the sum of the
// per-chain sums
static int kmc_shadow_read(spkgpu_lattice *h, double *pmax64, double *total64) {
  KmcState *k = h->kmc;
  unsigned long long bits = 0;
  std::vector<double> sums(k->nchains);
  KMC_CUDA(h, cudaMemcpyAsync(&bits, k->d_scalars + 2, 8, cudaMemcpyDeviceToHost, h->stream));
  KMC_CUDA(h, cudaMemcpyAsync(sums.data(), k->d_sum64, k->nchains * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  KMC_CUDA(h, cudaStreamSynchronize(h->stream));
  memcpy(pmax64, &bits, 8);
  double tot = 0.0;
  for (double v : sums) tot += v;
  *total64 = tot;
  return SPKGPU_OK;
}

static cudaError_t kmc_launch(spkgpu_lattice *h, int what, const KmcArgs &a, const int32_t *list, int64_t n,
                              int iset) {
  KmcState *k = h->kmc;
  int nprocs = k->nchains / h->d.nsector;
  size_t smem = a.smem_trees ? (size_t)k->max_ntotal * 8 : 0;
  h->launches++;
  const size_t ts = k->tree_smem;
  switch (h->spin_bytes) {
    case 1: return dispatch_lat<int8_t>(h->d.lattice, h->d.app, what, a, list, n, iset, nprocs, smem, ts, h->stream, h->num_sms);
    case 2: return dispatch_lat<int16_t>(h->d.lattice, h->d.app, what, a, list, n, iset, nprocs, smem, ts, h->stream, h->num_sms);
    case 4: return dispatch_lat<int32_t>(h->d.lattice, h->d.app, what, a, list, n, iset, nprocs, smem, ts, h->stream, h->num_sms);
  }
  return cudaErrorInvalidValue;
}

extern "C" int spkgpu_kmc_setup(spkgpu_lattice *h, int32_t adapt, double nstop, double tstop, int32_t fp64) {
  if (!h) return SPKGPU_ERR_ARG;
  const spkgpu_desc &d = h->d;
  if (d.nsector < 2) return spk_fail(h, SPKGPU_ERR_UNSUPPORTED, "KMC on the GPU needs sectors (sector yes|2|4|8)");
  if (h->packed) return spk_fail(h, SPKGPU_ERR_UNSUPPORTED, "KMC needs one value per site (spin_bytes 1, 2 or 4)");
  if (d.rng != SPKGPU_RNG_PHILOX) return spk_fail(h, SPKGPU_ERR_ARG, "KMC uses Philox draws");
  if (adapt && !(nstop > 0.0)) return spk_fail(h, SPKGPU_ERR_ARG, "nstop must be > 0");
  if (!adapt && !(tstop > 0.0)) return spk_fail(h, SPKGPU_ERR_ARG, "tstop must be > 0");
  if (h->n >= (1LL << 31)) return spk_fail(h, SPKGPU_ERR_UNSUPPORTED, "KMC lattices are limited to 2^31 sites");
  spk_kmc_free(h);
  KmcState *k = new (std::nothrow) KmcState();
  if (!k) return SPKGPU_ERR_NOMEM;
  h->kmc = k;
  k->adapt = adapt ? 1 : 0;
  k->nstop = nstop;
  k->tstop = tstop;
  if (fp64 < 0 || fp64 > 2) return spk_fail(h, SPKGPU_ERR_ARG, "fp64 must be 0, 1 or 2");
  k->fp64 = (fp64 == 1) ? 1 : 0;
  k->shadow = (fp64 == 0) ? 1 : 0;
  // chain membership from the handle's processor and sector-half tables
  std::vector<int32_t> blob_proc[3], blob_half[3];
  int dims[3] = {d.nx, d.ny, d.nz};
  for (int ax = 0; ax < 3; ax++) {
    blob_proc[ax].resize(dims[ax]);
    blob_half[ax].resize(dims[ax]);
    KMC_CUDA(h, cudaMemcpy(blob_proc[ax].data(), h->d_axis + h->proc_off[ax], dims[ax] * 4, cudaMemcpyDeviceToHost));
    KMC_CUDA(h, cudaMemcpy(blob_half[ax].data(), h->d_axis + h->half_off[ax], dims[ax] * 4, cudaMemcpyDeviceToHost));
  }
  int nsec = d.nsector;
  int nprocs = d.procs[0] * d.procs[1] * d.procs[2];
  k->nchains = nprocs * nsec;
  int64_t n = h->n;
  k->nsites = n;
  std::vector<int32_t> setof(n), i2site(n), nloc(k->nchains, 0);
  for (int64_t i = 0; i < n; i++) {
    int x = (int)(i % d.nx);
    int64_t r = i / d.nx;
    int y = (int)(r % d.ny);
    int z = (int)(r / d.ny);
    int proc = blob_proc[0][x] + d.procs[0] * (blob_proc[1][y] + d.procs[1] * blob_proc[2][z]);
    int iw = blob_half[0][x], jw = blob_half[1][y], kw = blob_half[2][z];
    int msector = (nsec == 2) ? iw : (nsec == 4 ? 2 * jw + iw : 4 * kw + 2 * jw + iw);
    int c = proc * nsec + msector;
    setof[i] = c;
    i2site[i] = nloc[c]++;
  }
  std::vector<int64_t> site_off(k->nchains + 1, 0), tree_off(k->nchains + 1, 0);
  std::vector<int32_t> leaf0(k->nchains), ntotal(k->nchains);
  for (int c = 0; c < k->nchains; c++) {
    site_off[c + 1] = site_off[c] + nloc[c];
    int64_t nround = 1;
    while (nround < nloc[c]) nround *= 2;
    leaf0[c] = (int32_t)(nround - 1);
    ntotal[c] = (int32_t)(2 * nround - 1);
    tree_off[c + 1] = tree_off[c] + ntotal[c];
    k->max_ntotal = std::max(k->max_ntotal, ntotal[c]);
  }
  std::vector<int32_t> site2i(n);
  for (int64_t i = 0; i < n; i++) site2i[site_off[setof[i]] + i2site[i]] = (int32_t)i;
  // chain boxes: along each axis a chain takes the coordinates of its
  // processor (and of its sector half where the sectors split that axis);
  // each must be one run of coordinates and the box must hold the chain
  std::vector<int32_t> box((size_t)k->nchains * 6);
  k->boxes = true;
  {
    const int split[3] = {1, nsec >= 4 ? 1 : 0, nsec == 8 ? 1 : 0};
    for (int c = 0; c < k->nchains && k->boxes; c++) {
      const int proc = c / nsec, msec = c % nsec;
      const int pc[3] = {proc % d.procs[0], (proc / d.procs[0]) % d.procs[1], proc / (d.procs[0] * d.procs[1])};
      const int hc[3] = {msec & 1, (msec >> 1) & 1, (msec >> 2) & 1};
      int64_t vol = 1;
      for (int ax = 0; ax < 3; ax++) {
        int lo = -1, hi = -2, cnt = 0;
        for (int v = 0; v < dims[ax]; v++) {
          if (blob_proc[ax][v] != pc[ax] || (split[ax] && blob_half[ax][v] != hc[ax])) continue;
          if (lo < 0) lo = v;
          hi = v;
          cnt++;
        }
        if (cnt == 0 || cnt != hi - lo + 1) k->boxes = false;
        box[6 * c + ax] = lo;
        box[6 * c + 3 + ax] = cnt;
        vol *= cnt;
      }
      if (vol != nloc[c]) k->boxes = false;
    }
  }
  // border sites (a neighbour in another chain), grouped by sector index in
  // the order chains of that sector appear (find_border_sites,
  // src/app_lattice.cpp:1094-1149)
  int nn = h->maxneigh;
  std::vector<std::vector<int32_t>> border_by_sec(nsec);
  for (int c = 0; c < k->nchains; c++) {
    int sec = c % nsec;
    for (int64_t m = site_off[c]; m < site_off[c + 1]; m++) {
      int64_t i = site2i[m];
      int x = (int)(i % d.nx);
      int64_t r = i / d.nx;
      int y = (int)(r % d.ny);
      int z = (int)(r / d.ny);
      bool border = false;
      for (int j = 0; j < nn && !border; j++) {
        int dx = 0, dy = 0, dz = 0;
        switch (d.lattice) {
          case SPKGPU_SQ_4N: Stencil<SPKGPU_SQ_4N>::offset(j, dx, dy, dz); break;
          case SPKGPU_SQ_8N: Stencil<SPKGPU_SQ_8N>::offset(j, dx, dy, dz); break;
          case SPKGPU_SC_6N: Stencil<SPKGPU_SC_6N>::offset(j, dx, dy, dz); break;
          default: Stencil<SPKGPU_SC_26N>::offset(j, dx, dy, dz); break;
        }
        int xn = (x + dx + d.nx) % d.nx, yn = (y + dy + d.ny) % d.ny, zn = (z + dz + d.nz) % d.nz;
        int64_t nbi = xn + (int64_t)d.nx * (yn + (int64_t)d.ny * zn);
        if (setof[nbi] != c) border = true;
      }
      if (border) border_by_sec[sec].push_back((int32_t)i);
    }
  }
  std::vector<int32_t> border;
  k->border_off.assign(nsec + 1, 0);
  for (int s = 0; s < nsec; s++) {
    border.insert(border.end(), border_by_sec[s].begin(), border_by_sec[s].end());
    k->border_off[s + 1] = (int64_t)border.size();
  }
  auto dm = [&](void **p, size_t bytes) { return cudaMalloc(p, bytes ? bytes : 16) == cudaSuccess; };
  if (!dm((void **)&k->d_setof, n * 4) || !dm((void **)&k->d_i2site, n * 4) || !dm((void **)&k->d_site2i, n * 4) ||
      !dm((void **)&k->d_border, border.size() * 4) || !dm((void **)&k->d_site_off, (k->nchains + 1) * 8) ||
      !dm((void **)&k->d_tree_off, (k->nchains + 1) * 8) || !dm((void **)&k->d_nloc, k->nchains * 4) ||
      !dm((void **)&k->d_leaf0, k->nchains * 4) || !dm((void **)&k->d_ntotal, k->nchains * 4) ||
      !dm((void **)&k->d_nactive, k->nchains * 4) || !dm((void **)&k->d_events, k->nchains * 8) ||
      !dm((void **)&k->d_trees, tree_off[k->nchains] * 8) || !dm((void **)&k->d_scalars, 4 * 8) ||
      !dm((void **)&k->d_sum64, k->nchains * 8) || !dm((void **)&k->d_box, box.size() * 4)) {
    spk_kmc_free(h);
    return spk_fail(h, SPKGPU_ERR_NOMEM, "KMC allocation failed");
  }
  KMC_CUDA(h, cudaMemcpy(k->d_setof, setof.data(), n * 4, cudaMemcpyHostToDevice));
  KMC_CUDA(h, cudaMemcpy(k->d_i2site, i2site.data(), n * 4, cudaMemcpyHostToDevice));
  KMC_CUDA(h, cudaMemcpy(k->d_site2i, site2i.data(), n * 4, cudaMemcpyHostToDevice));
  if (!border.empty()) KMC_CUDA(h, cudaMemcpy(k->d_border, border.data(), border.size() * 4, cudaMemcpyHostToDevice));
  KMC_CUDA(h, cudaMemcpy(k->d_site_off, site_off.data(), (k->nchains + 1) * 8, cudaMemcpyHostToDevice));
  KMC_CUDA(h, cudaMemcpy(k->d_tree_off, tree_off.data(), (k->nchains + 1) * 8, cudaMemcpyHostToDevice));
  KMC_CUDA(h, cudaMemcpy(k->d_nloc, nloc.data(), k->nchains * 4, cudaMemcpyHostToDevice));
  KMC_CUDA(h, cudaMemcpy(k->d_leaf0, leaf0.data(), k->nchains * 4, cudaMemcpyHostToDevice));
  KMC_CUDA(h, cudaMemcpy(k->d_ntotal, ntotal.data(), k->nchains * 4, cudaMemcpyHostToDevice));
  KMC_CUDA(h, cudaMemcpy(k->d_box, box.data(), box.size() * 4, cudaMemcpyHostToDevice));
  // the shared-memory tree kernel where the chains are boxes and the tree
  // fits; the global-tree kernel otherwise
  k->tree_smem = 0;
  if (k->boxes) {
    int optin = 0;
    KMC_CUDA(h, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->d.device));
    k->tree_smem = kmc_tree_smem_bytes(k->max_ntotal, nn, d.lattice == SPKGPU_SC_6N || d.lattice == SPKGPU_SC_26N,
                                       (size_t)optin);
  }
  KMC_CUDA(h, cudaMemset(k->d_events, 0, k->nchains * 8));
  KMC_CUDA(h, cudaMemset(k->d_trees, 0, tree_off[k->nchains] * 8));
  KMC_CUDA(h, cudaMemset(k->d_scalars, 0, 4 * 8));
  k->ready = 1;
  return SPKGPU_OK;
}

// pmax over all chains of sum/num_active after a full rebuild
static int kmc_pmax(spkgpu_lattice *h, double *pmax) {
  unsigned long long bits = 0;
  KMC_CUDA(h, cudaMemcpyAsync(&bits, h->kmc->d_scalars, 8, cudaMemcpyDeviceToHost, h->stream));
  KMC_CUDA(h, cudaStreamSynchronize(h->stream));
  double v;
  memcpy(&v, &bits, 8);
  *pmax = v;
  return SPKGPU_OK;
}

extern "C" int spkgpu_kmc_run_until(spkgpu_lattice *h, double *ptime, double stoptime, double until, int32_t first,
                                    spkgpu_kmc_stats *out) {
  if (!h || !ptime) return SPKGPU_ERR_ARG;
  KmcState *k = h->kmc;
  if (!k || !k->ready) return spk_fail(h, SPKGPU_ERR_STATE, "spkgpu_kmc_setup has not been called");
  if (!h->have_temperature) return spk_fail(h, SPKGPU_ERR_STATE, "temperature has not been set");
  if (!first && !k->in_run) return spk_fail(h, SPKGPU_ERR_STATE, "no KMC run to continue");
  const int nsec = h->d.nsector;
  double time = *ptime;
  KmcArgs a = kmc_args(h);
  // FP32 propensities with the FP64 shadow: pmax of the same chains at the
  // same moments from all-FP64 propensities, and the relative error of the
  // adaptive time step nstop/pmax it gives
  auto shadow_err = [&](double pmax32) -> int {
    double pmax64 = 0.0, tot64 = 0.0;
    int rc = kmc_shadow_read(h, &pmax64, &tot64);
    if (rc) return rc;
    if (pmax32 > 0.0 && pmax64 > 0.0)
      k->dt_rel_err = std::max(k->dt_rel_err, fabs(pmax64 / pmax32 - 1.0));  // (1/p32 - 1/p64) / (1/p64)
    return SPKGPU_OK;
  };
  auto shadow_clear = [&]() -> cudaError_t {
    cudaError_t e = cudaMemsetAsync(k->d_sum64, 0, k->nchains * sizeof(double), h->stream);
    return e == cudaSuccess ? cudaMemsetAsync(k->d_scalars + 2, 0, 8, h->stream) : e;
  };
  if (first) {
    // setup(): every propensity, every tree (src/app_lattice.cpp:340-347)
    KMC_CUDA(h, kmc_launch(h, 0, a, nullptr, h->n, 0));
    kmc_build_kernel<<<k->nchains, 256, 0, h->stream>>>(a, -1);
    h->launches++;
    KMC_CUDA(h, cudaGetLastError());
    if (k->tstop > 0.0 && !k->adapt) k->dt_kmc = k->tstop;
    if (k->adapt) {
      // max over sets of sum/num_active (src/app_lattice.cpp:356-371)
      std::vector<double> roots;
      std::vector<int32_t> nact(k->nchains);
      int rc = kmc_roots(h, a, roots);
      if (rc) return rc;
      KMC_CUDA(h, cudaMemcpy(nact.data(), k->d_nactive, k->nchains * 4, cudaMemcpyDeviceToHost));
      double pmax = 0.0;
      for (int c = 0; c < k->nchains; c++)
        if (nact[c] > 0) pmax = std::max(pmax, roots[c] / nact[c]);
      k->dt_kmc = (pmax > 0.0) ? k->nstop / pmax : stoptime - time;
    }
    k->dt_rel_err = 0.0;
    if (k->shadow && k->adapt) {
      KMC_CUDA(h, shadow_clear());
      KMC_CUDA(h, kmc_shadow64(h, a, -1));
      int rc = shadow_err(k->nstop / k->dt_kmc);
      if (rc) return rc;
    }
    k->dt_kmc = std::min(k->dt_kmc, stoptime - time);
    k->in_run = 1;
  }
  if (stoptime > time) {
    bool alldone = false;
    while (!alldone) {
      KMC_CUDA(h, cudaMemsetAsync(k->d_scalars, 0, 8, h->stream));
      if (k->shadow) KMC_CUDA(h, shadow_clear());
      a.dt_kmc = k->dt_kmc;
      for (int iset = 0; iset < nsec; iset++) {
        int64_t b0 = k->border_off[iset], b1 = k->border_off[iset + 1];
        KMC_CUDA(h, kmc_launch(h, 0, a, k->d_border + b0, b1 - b0, iset));
        kmc_build_kernel<<<k->nchains / nsec, 256, 0, h->stream>>>(a, iset);
        h->launches++;
        KMC_CUDA(h, cudaGetLastError());
        // pmax is taken here, before the sector's events (src/app_lattice.cpp:564-571)
        if (k->shadow) KMC_CUDA(h, kmc_shadow64(h, a, iset));
        KMC_CUDA(h, kmc_launch(h, 1, a, nullptr, 0, iset));
      }
      k->npass++;
      time += k->dt_kmc;
      if (time >= stoptime) alldone = true;
      if (k->adapt) {
        double pmax = 0.0;
        int rc = kmc_pmax(h, &pmax);
        if (rc) return rc;
        if (k->shadow) {
          rc = shadow_err(pmax);
          if (rc) return rc;
        }
        k->dt_kmc = (pmax > 0.0) ? k->nstop / pmax : stoptime - time;
        k->dt_kmc = std::min(k->dt_kmc, stoptime - time);
      }
      // an output time: return to the caller, which continues the run
      // with first = 0 (src/app_lattice.cpp:606-609)
      if (!alldone && time >= until) break;
    }
  }
  if (time >= stoptime) k->in_run = 0;
  *ptime = time;
  if (out) {
    unsigned long long na = 0;
    KMC_CUDA(h, cudaMemcpyAsync(&na, k->d_scalars + 1, 8, cudaMemcpyDeviceToHost, h->stream));
    std::vector<double> roots;
    int rc = kmc_roots(h, a, roots);
    if (rc) return rc;
    double total = 0.0;
    for (double r : roots) total += r;
    out->time = time;
    out->naccept = (int64_t)na;
    out->npass = k->npass;
    out->dt_kmc = k->dt_kmc;
    out->total_propensity = total;
    out->prop_rel_err = 0.0;
    out->dt_rel_err = 0.0;
    if (k->shadow) {
      // the final lattice's total propensity from FP32 and from FP64 site
      // propensities (both summed in FP64)
      double pm = 0.0, tot32 = 0.0, tot64 = 0.0;
      KMC_CUDA(h, shadow_clear());
      KMC_CUDA(h, kmc_shadow64(h, a, -1, 0));
      rc = kmc_shadow_read(h, &pm, &tot32);
      if (rc) return rc;
      KMC_CUDA(h, shadow_clear());
      KMC_CUDA(h, kmc_shadow64(h, a, -1, 1));
      rc = kmc_shadow_read(h, &pm, &tot64);
      if (rc) return rc;
      out->prop_rel_err = tot64 > 0.0 ? fabs(tot32 - tot64) / tot64 : 0.0;
      out->dt_rel_err = k->dt_rel_err;
    }
  }
  return SPKGPU_OK;
}

extern "C" int spkgpu_kmc_run(spkgpu_lattice *h, double *ptime, double stoptime, spkgpu_kmc_stats *out) {
  return spkgpu_kmc_run_until(h, ptime, stoptime, stoptime, 1, out);
}
