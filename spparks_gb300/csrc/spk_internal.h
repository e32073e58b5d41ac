// Internal declarations shared by the spkgpu translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/spkgpu.h"

namespace spk {

constexpr int kMaxNeigh = 26;

inline int maxneigh_of(int lattice) {
  switch (lattice) {
    case SPKGPU_SQ_4N: return 4;
    case SPKGPU_SQ_8N: return 8;
    case SPKGPU_SC_6N: return 6;
    case SPKGPU_SC_26N: return 26;
  }
  return 0;
}

inline int ncolors_of(int lattice) {
  switch (lattice) {
    case SPKGPU_SQ_4N: return 2;
    case SPKGPU_SQ_8N: return 4;
    case SPKGPU_SC_6N: return 2;
    case SPKGPU_SC_26N: return 8;
  }
  return 0;
}

inline bool is2d(int lattice) { return lattice == SPKGPU_SQ_4N || lattice == SPKGPU_SQ_8N; }

// Boltzmann acceptance tables for one temperature: for an energy increase
// dE > 0 the reference rejects when u > exp((einitial-efinal)*t_inverse)
// (src/app_ising.cpp:120); thr[dE] = floor(exp(-dE*t_inverse) * 2^32) turns
// that into "accept iff x < thr[dE]" on the Philox word (for ising,
// floor(exp(-dE*t_inverse) * 2^31) against the word's low 31 bits), pexp[dE]
// is the double itself for the Park-Miller (strict) path.
struct AcceptTable {
  uint64_t thr[kMaxNeigh + 1];
  double pexp[kMaxNeigh + 1];
  int zero_t;  // temperature == 0: every uphill move is rejected
};

void build_accept_table(double temperature, int app, AcceptTable *t);

// one set of sites swept in one launch: the sites of colour `color` whose
// coordinates lie in the per-axis lists.  Every lattice colour fixes the
// parity of x given y and z, so x comes from a parity-split list: xl[q]
// holds the set's x coordinates of parity q, and q = (color-1+y+z)&1 when
// xpar_fixed = 0 (sq/4n, sc/6n) or xl[0] is already the right list.
struct PhaseArgs {
  void *spin;
  int nx, ny, nz;
  const int32_t *xl[2];
  int nxl[2];
  int xpar_fixed;
  const int32_t *yl, *zl;
  int nyl, nzl;
  int color;
  uint32_t seed, sweep, pass;
  int nspins;
  int rng;
  int mask_on;
  int32_t *siteseeds;
  uint8_t *mask;
  unsigned long long *naccept;
  AcceptTable acc;
};

// clears AppLattice::mask before a set is swept (boundary_clear_mask,
// src/app_lattice.cpp:1157-1163): for a colour set every site of the colour
// (each borders other sets), for a sector set the sites with a neighbour in
// another (processor, sector) set
struct MaskClearArgs {
  uint8_t *mask;
  int nx, ny, nz;
  const int32_t *xl, *yl, *zl;   // coordinates of the set (any parity)
  int nxl, nyl, nzl;
  int color;                     // > 0: colour-set mode
  const int32_t *proc_x, *proc_y, *proc_z;  // processor index per coordinate
  const int32_t *half_x, *half_y, *half_z;  // sector half per coordinate
};

// launchers (return cudaError_t of the launch)
cudaError_t launch_phase(int lattice, int app, int spin_bytes, const PhaseArgs &a, cudaStream_t s,
                         int num_sms);
cudaError_t launch_mask_clear(int lattice, const MaskClearArgs &a, cudaStream_t s, int num_sms);
cudaError_t launch_energy(int lattice, int spin_bytes, const void *spin, int nx, int ny, int nz,
                          unsigned long long *out, cudaStream_t s, int num_sms);
// The device address of host memory that kernels may read and write
// directly (page-locked and registered with CUDA: cudaHostAlloc,
// cudaMallocHost, cudaHostRegister), or nullptr for any other pointer.
inline void *mapped_host_ptr(const void *p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return (at.type == cudaMemoryTypeHost && at.devicePointer) ? at.devicePointer : nullptr;
}

cudaError_t launch_convert_in(int spin_bytes, const int32_t *src, void *dst, int64_t n, int nspins,
                              int *bad, cudaStream_t s);
cudaError_t launch_convert_out(int spin_bytes, const void *src, int32_t *dst, int64_t n,
                               cudaStream_t s);
cudaError_t launch_init(int spin_bytes, void *dst, int64_t n, uint32_t seed, int lo, int hi, cudaStream_t s,
                        int num_sms);

// fused whole-sweep tile kernel for 2d lattices without sectors
// (returns cudaErrorNotSupported when the configuration is not covered)
struct FusedArgs {
  const void *src;
  void *dst;
  int nx, ny;
  uint32_t seed, sweep;
  int nspins;
  unsigned long long *naccept;
  AcceptTable acc;
};
bool fused2d_supported(int lattice, int app, int spin_bytes, int nx, int ny);
cudaError_t launch_fused2d(int lattice, int app, int spin_bytes, const FusedArgs &a, cudaStream_t s,
                           int num_sms);

// all sweeps of one call for an sq/4n lattice that fits one CTA's shared
// memory (sweep_resident.cu); same eligibility as the fused sweep otherwise
bool resident_supported(int lattice, int app, int spin_bytes, int nx, int ny);
cudaError_t launch_resident_sweeps(int app, int spin_bytes, void *spin, int nx, int ny, uint32_t seed,
                                   uint32_t sweep0, int nsweeps, int nspins, unsigned long long *naccept,
                                   const AcceptTable &acc, cudaStream_t s);

// row-pair sweep for sq/8n and sc/26n without sectors (sweep_rows.cu)
bool rows_supported(int lattice, int spin_bytes, int nx, int nspins);
cudaError_t launch_rows_sweep(int lattice, int app, int spin_bytes, void *spin, int nx, int ny, int nz,
                              uint32_t seed, uint32_t sweep, int nspins, unsigned long long *naccept,
                              const AcceptTable &acc, cudaStream_t st, int *launches);

// bit-packed Ising on sc/6n (packed.cu)
struct PackedArgs {
  void *words;                 // nx/64 * ny * nz uint64
  void *decisions;             // 4 uint64 per word
  int nx, ny, nz;
  int64_t nwords;
  uint32_t seed, sweep;
  uint64_t thr2, thr4, thr6;   // Boltzmann thresholds for dE = 2, 4, 6
  unsigned long long *naccept;
};
cudaError_t launch_packed_sweep(const PackedArgs &a, cudaStream_t s, int num_sms);
cudaError_t launch_packed_pack(const int32_t *src, uint64_t *dst, int64_t nwords, int *bad, cudaStream_t s,
                               int num_sms);
cudaError_t launch_packed_unpack(const uint64_t *src, int32_t *dst, int64_t nwords, cudaStream_t s, int num_sms);
cudaError_t launch_packed_energy(const uint64_t *W, int nx, int ny, int nz, unsigned long long *out, cudaStream_t s,
                                 int num_sms);

}  // namespace spk

// per-axis coordinate lists of the handle: list (axis a, sector half h,
// parity q) starts at d_axis + off[a][h][q] and holds len[a][h][q] entries;
// h = 2 and q = 2 mean "any"
struct spkgpu_axes_store {
  int64_t off[3][3][3];
  int len[3][3][3];
};

// the handle behind the C ABI
struct spkgpu_lattice {
  spkgpu_desc d;
  int64_t n = 0;
  int spin_bytes = 4;
  int ncolors = 0;
  int maxneigh = 0;
  int num_sms = 0;
  void *d_spin = nullptr;
  void *d_spin_alt = nullptr;   // second buffer of the fused double-buffered sweep
  void *d_decisions = nullptr;  // bit-packed path: per-word decision masks of a sweep
  bool packed = false;          // spin_bytes == -1: 64 Ising sites per uint64
  int32_t *d_seeds = nullptr;
  uint8_t *d_mask = nullptr;
  unsigned long long *d_counters = nullptr;  // [1] energy, [2] bad-value flag, [3..5] diagnostics
  int32_t *d_labels = nullptr;  // diagnostics: cluster labels and sizes (2n int32) + partial sums
  int32_t *d_stage = nullptr;   // int32 staging for upload/download
  int64_t stage_n = 0;
  int32_t *d_axis = nullptr;    // per-axis coordinate lists and tables
  spkgpu_axes_store *axes = nullptr;
  int64_t proc_off[3] = {0, 0, 0};  // processor index per coordinate
  int64_t half_off[3] = {0, 0, 0};  // sector half per coordinate
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double temperature = 0.0;
  bool have_temperature = false;
  spk::AcceptTable acc;
  int64_t sweep = 0;
  int64_t nsweeps_done = 0;
  int64_t nattempt = 0;
  int64_t launches = 0;
  bool fused_ok = false;         // sq/4n fused tile sweep
  bool resident_ok = false;      // sq/4n lattice in one CTA's shared memory
  bool rows_ok = false;          // sq/8n, sc/26n row-pair sweep
  std::string err;
  // KMC state (kmc.cu)
  struct KmcState *kmc = nullptr;
};

int spk_fail(spkgpu_lattice *h, int code, const std::string &msg);
void spk_kmc_free(spkgpu_lattice *h);
int spk_cuda_fail(spkgpu_lattice *h, cudaError_t e, const char *what);
