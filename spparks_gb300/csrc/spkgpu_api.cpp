// The spkgpu C ABI (include/spkgpu.h): handle lifecycle, host<->device site
// values, and the sweep driver that reproduces the set ordering of
// AppLattice::iterate_rejection (src/app_lattice.cpp:632-711):
//   for each sweep:  for each sector (1 if none):  [clear mask on the
//   sector border]  for each colour: [clear colour mask] for each pass
//   (nloop): one phase launch over that (sector, colour) set.
// Sector membership follows AppLattice::create_set (src/app_lattice.cpp:
// 956-985): within each processor sub-domain (Domain::procs2domain_*,
// src/domain.cpp:174-330) a site is in the lower half of an axis when its
// coordinate is below the sub-domain midpoint.

#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>
#include <map>
#include <mutex>
#include <vector>

#include "counters.cuh"
#include "spk_internal.h"

using spk::AcceptTable;

// d_counters layout: [0,8) scalars ([1] energy, [2] bad-value flag, [3..5]
// site diagnostics),
// [8, 8+256) Naccept slots
static const int kNacceptSlots = 8;
static const int kCounterWords = kNacceptSlots + spk::kCounterSlots;

int spk_fail(spkgpu_lattice *h, int code, const std::string &msg) {
  if (h) h->err = msg;
  return code;
}

int spk_cuda_fail(spkgpu_lattice *h, cudaError_t e, const char *what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  return spk_fail(h, SPKGPU_ERR_CUDA, m);
}

#define SPK_CUDA(h, call)                                   \
  do {                                                      \
    cudaError_t e__ = (call);                               \
    if (e__ != cudaSuccess) return spk_cuda_fail(h, e__, #call); \
  } while (0)

namespace spk {

void build_accept_table(double temperature, int app, AcceptTable *t) {
  // the Boltzmann draw has 31 bits for ising, 32 for the other apps
  const double scale = (app == SPKGPU_ISING) ? 2147483648.0 : 4294967296.0;
  t->zero_t = (temperature == 0.0) ? 1 : 0;
  double t_inverse = (temperature != 0.0) ? 1.0 / temperature : 0.0;
  for (int de = 0; de <= kMaxNeigh; de++) {
    // the reference evaluates exp((einitial-efinal)*t_inverse) with
    // einitial-efinal = -dE exactly (integer-valued doubles)
    double p = exp((double)(-de) * t_inverse);
    t->pexp[de] = p;
    double scaled = p * scale;  // exact: power-of-two scaling
    double fl = floor(scaled);
    t->thr[de] = (fl >= scale) ? (uint64_t)scale : (uint64_t)fl;
  }
  if (t->zero_t) {
    for (int de = 0; de <= kMaxNeigh; de++) {
      t->thr[de] = 0;
      t->pexp[de] = 0.0;
    }
  }
}

}  // namespace spk

namespace {

// processor of coordinate c along an axis of n sites split over P procs:
// proc p owns [p*n/P, (p+1)*n/P) in box units (Domain::procs2domain_*)
int proc_of(int c, int n, int P) {
  double prd = (double)n;
  for (int p = 0; p < P; p++) {
    double lo = p * prd / P;
    double hi = (p < P - 1) ? (p + 1) * prd / P : prd;
    if ((double)c >= lo && (double)c < hi) return p;
  }
  return P - 1;
}

double mid_of(int p, int n, int P) {
  double prd = (double)n;
  double lo = p * prd / P;
  double hi = (p < P - 1) ? (p + 1) * prd / P : prd;
  return 0.5 * (lo + hi);
}

struct AxisTables {
  // lists[h][q]: coords with sector half h (2 = any) and parity q (2 = any)
  std::vector<int32_t> lists[3][3];
  std::vector<int32_t> proc, half;
};

AxisTables make_axis(int n, int P, bool split_z2d) {
  AxisTables t;
  t.proc.resize(n);
  t.half.resize(n);
  for (int c = 0; c < n; c++) {
    int p = proc_of(c, n, P);
    t.proc[c] = p;
    // 2d boxes span z in -0.5..0.5 (midpoint 0): the single layer is "upper"
    t.half[c] = split_z2d ? 1 : (((double)c < mid_of(p, n, P)) ? 0 : 1);
  }
  for (int h = 0; h < 3; h++)
    for (int q = 0; q < 3; q++)
      for (int c = 0; c < n; c++)
        if ((h == 2 || t.half[c] == h) && (q == 2 || (c & 1) == q)) t.lists[h][q].push_back(c);
  return t;
}

int sector_half(int nsector, int sector, int axis) {
  // sector numbering of create_set: msector = 4*kw + 2*jw + iw + 1
  int s = sector - 1;
  if (nsector <= 1) return 2;
  if (nsector == 2) return axis == 0 ? s : 2;
  if (nsector == 4) return axis == 0 ? (s & 1) : (axis == 1 ? (s >> 1) & 1 : 2);
  return axis == 0 ? (s & 1) : (axis == 1 ? (s >> 1) & 1 : (s >> 2) & 1);
}

}  // namespace

// Where an sq/4n lattice fits one cluster, both the cluster-resident sweep
// (every sweep of a call in one launch) and the tile kernel (one launch per
// sweep) apply; they give the same lattice.  The first handle of each
// (device, app, width, nx, ny) times four sweeps of each on a scratch copy
// (Philox initial values, temperature 1) and keeps the faster for every
// later handle of that shape in the process.
static bool resident_is_faster(spkgpu_lattice *h) {
  static std::mutex mu;
  static std::map<std::vector<int>, bool> cache;
  const spkgpu_desc &d = h->d;
  const std::vector<int> key{d.device, d.app, h->spin_bytes, d.nx, d.ny};
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  const size_t bytes = (size_t)h->n * h->spin_bytes;
  void *a = nullptr, *b = nullptr;
  unsigned long long *cnt = nullptr;
  bool resident = false;  // the tile kernel, should a timing step fail
  if (cudaMalloc(&a, bytes) == cudaSuccess && cudaMalloc(&b, bytes) == cudaSuccess &&
      cudaMalloc(&cnt, spk::kCounterSlots * sizeof(unsigned long long)) == cudaSuccess) {
    spk::AcceptTable acc;
    spk::build_accept_table(1.0, d.app, &acc);
    cudaStream_t st = h->stream;
    const int nsw = 4;
    float ms[2] = {0.0f, 0.0f};
    bool ok = spk::launch_init(h->spin_bytes, a, h->n, d.seed, 1, d.nspins, st, h->num_sms) == cudaSuccess;
    for (int form = 0; form < 2 && ok; form++) {
      for (int rep = 0; rep < 2 && ok; rep++) {  // the first pass warms up
        ok = cudaEventRecord(h->ev0, st) == cudaSuccess;
        if (form == 0) {
          ok = ok && spk::launch_resident_sweeps(d.app, h->spin_bytes, a, d.nx, d.ny, d.seed, 0, nsw, d.nspins, cnt,
                                                 acc, st) == cudaSuccess;
        } else {
          for (int k = 0; k < nsw && ok; k++) {
            spk::FusedArgs f;
            f.src = (k & 1) ? b : a;
            f.dst = (k & 1) ? a : b;
            f.nx = d.nx;
            f.ny = d.ny;
            f.seed = d.seed;
            f.sweep = (uint32_t)k;
            f.nspins = d.nspins;
            f.naccept = cnt;
            f.acc = acc;
            ok = spk::launch_fused2d(d.lattice, d.app, h->spin_bytes, f, st, h->num_sms) == cudaSuccess;
          }
        }
        ok = ok && cudaEventRecord(h->ev1, st) == cudaSuccess && cudaEventSynchronize(h->ev1) == cudaSuccess &&
             cudaEventElapsedTime(&ms[form], h->ev0, h->ev1) == cudaSuccess;
      }
    }
    if (ok) resident = ms[0] <= ms[1];
    cudaGetLastError();
  }
  cudaFree(a);
  cudaFree(b);
  cudaFree(cnt);
  std::lock_guard<std::mutex> lock(mu);
  cache[key] = resident;
  return resident;
}

extern "C" {

int spkgpu_version(void) { return 1; }

const char *spkgpu_last_error(const spkgpu_lattice *h) { return h ? h->err.c_str() : "null handle"; }

int spkgpu_create(const spkgpu_desc *desc, spkgpu_lattice **out) {
  if (!desc || !out) return SPKGPU_ERR_ARG;
  *out = nullptr;
  const spkgpu_desc &d = *desc;
  if (d.lattice < SPKGPU_SQ_4N || d.lattice > SPKGPU_SC_26N) return SPKGPU_ERR_ARG;
  if (d.app < SPKGPU_ISING || d.app > SPKGPU_POTTS_NEIGH) return SPKGPU_ERR_ARG;
  if (d.nx <= 0 || d.ny <= 0 || d.nz <= 0) return SPKGPU_ERR_ARG;
  if (spk::is2d(d.lattice) && d.nz != 1) return SPKGPU_ERR_ARG;
  if (d.app == SPKGPU_ISING && d.nspins != 2) return SPKGPU_ERR_ARG;
  if (d.nspins < 1 || d.nspins >= (1 << 21)) return SPKGPU_ERR_ARG;
  if (!(d.nsector == 1 || d.nsector == 2 || d.nsector == 4 || d.nsector == 8)) return SPKGPU_ERR_ARG;
  if (spk::is2d(d.lattice) && d.nsector == 8) return SPKGPU_ERR_ARG;  // src/app_lattice.cpp:176-177
  if (d.nloop < 1) return SPKGPU_ERR_ARG;
  if (d.procs[0] < 1 || d.procs[1] < 1 || d.procs[2] < 1) return SPKGPU_ERR_ARG;
  if (spk::is2d(d.lattice) && d.procs[2] != 1) return SPKGPU_ERR_ARG;
  if (d.procs[0] > d.nx || d.procs[1] > d.ny || d.procs[2] > d.nz) return SPKGPU_ERR_ARG;
  if (!spk::is2d(d.lattice)) {  // src/app_lattice.cpp:167-173
    if (d.nsector == 2 && (d.procs[1] != 1 || d.procs[2] != 1)) return SPKGPU_ERR_ARG;
    if (d.nsector == 4 && d.procs[2] != 1) return SPKGPU_ERR_ARG;
  } else if (d.nsector == 2 && d.procs[1] != 1) {
    return SPKGPU_ERR_ARG;
  }
  if (d.rng != SPKGPU_RNG_PHILOX && d.rng != SPKGPU_RNG_STRICT) return SPKGPU_ERR_ARG;
  if (d.variant < 0 || d.variant > 2) return SPKGPU_ERR_ARG;
  if (d.rng == SPKGPU_RNG_STRICT && d.nsector > 1) return SPKGPU_ERR_ARG;  // src/app_lattice.cpp:155-156
  // colouring needs even extents (Lattice::ncolors, src/lattice.cpp:187-228)
  if (d.nx % 2 || d.ny % 2 || (!spk::is2d(d.lattice) && d.nz % 2)) return SPKGPU_ERR_ARG;
  int sb = d.spin_bytes;
  if (sb == 0) sb = d.nspins <= 127 ? 1 : (d.nspins <= 32767 ? 2 : 4);
  bool packed = (sb == -1);
  if (packed) {  // multispin Ising: sc/6n, 64 sites of x per word, plain colour sweeps
    if (d.lattice != SPKGPU_SC_6N || d.app != SPKGPU_ISING || d.nx % 64 || d.nsector != 1 || d.nloop != 1 ||
        d.rng != SPKGPU_RNG_PHILOX || d.mask || d.variant != 0)
      return SPKGPU_ERR_ARG;
  } else if (!(sb == 1 || sb == 2 || sb == 4)) {
    return SPKGPU_ERR_ARG;
  }
  if ((sb == 1 && d.nspins > 127) || (sb == 2 && d.nspins > 32767)) return SPKGPU_ERR_ARG;

  spkgpu_lattice *h = new (std::nothrow) spkgpu_lattice();
  if (!h) return SPKGPU_ERR_NOMEM;
  h->d = d;
  h->spin_bytes = sb;
  h->packed = packed;
  h->n = (int64_t)d.nx * d.ny * d.nz;
  h->ncolors = spk::ncolors_of(d.lattice);
  h->maxneigh = spk::maxneigh_of(d.lattice);
  spk::build_accept_table(0.0, d.app, &h->acc);
  int code = SPKGPU_OK;
  auto fail = [&](int c) {
    code = c;
    spkgpu_destroy(h);
    return c;
  };
  cudaError_t e = cudaSetDevice(d.device);
  if (e != cudaSuccess) return fail(spk_cuda_fail(h, e, "cudaSetDevice"));
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d.device);
  h->num_sms = sms > 0 ? sms : 1;
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(SPKGPU_ERR_CUDA);
  if (cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess)
    return fail(SPKGPU_ERR_CUDA);
  size_t spin_alloc = packed ? (size_t)h->n / 8 : (size_t)h->n * sb;
  if (cudaMalloc(&h->d_spin, spin_alloc) != cudaSuccess) return fail(SPKGPU_ERR_NOMEM);
  if (cudaMemsetAsync(h->d_spin, 0, spin_alloc, h->stream) != cudaSuccess) return fail(SPKGPU_ERR_CUDA);
  if (packed && cudaMalloc(&h->d_decisions, (size_t)h->n / 64 * 32) != cudaSuccess) return fail(SPKGPU_ERR_NOMEM);
  if (cudaMalloc(&h->d_counters, kCounterWords * sizeof(unsigned long long)) != cudaSuccess)
    return fail(SPKGPU_ERR_NOMEM);
  cudaMemsetAsync(h->d_counters, 0, kCounterWords * sizeof(unsigned long long), h->stream);
  if (d.rng == SPKGPU_RNG_STRICT) {
    if (cudaMalloc(&h->d_seeds, (size_t)h->n * 4) != cudaSuccess) return fail(SPKGPU_ERR_NOMEM);
    cudaMemsetAsync(h->d_seeds, 0, (size_t)h->n * 4, h->stream);
  }
  if (d.mask) {
    if (cudaMalloc(&h->d_mask, (size_t)h->n) != cudaSuccess) return fail(SPKGPU_ERR_NOMEM);
    cudaMemsetAsync(h->d_mask, 0, (size_t)h->n, h->stream);
  }
  // axis tables
  int dims[3] = {d.nx, d.ny, d.nz};
  std::vector<int32_t> blob;
  spkgpu_axes_store *ax = new (std::nothrow) spkgpu_axes_store();
  if (!ax) return fail(SPKGPU_ERR_NOMEM);
  h->kmc = nullptr;
  for (int a = 0; a < 3; a++) {
    bool z2d = (a == 2 && spk::is2d(d.lattice));
    AxisTables t = make_axis(dims[a], d.procs[a], z2d);
    for (int hh = 0; hh < 3; hh++)
      for (int q = 0; q < 3; q++) {
        ax->off[a][hh][q] = (int64_t)blob.size();
        ax->len[a][hh][q] = (int)t.lists[hh][q].size();
        blob.insert(blob.end(), t.lists[hh][q].begin(), t.lists[hh][q].end());
      }
    h->proc_off[a] = (int64_t)blob.size();
    blob.insert(blob.end(), t.proc.begin(), t.proc.end());
    h->half_off[a] = (int64_t)blob.size();
    blob.insert(blob.end(), t.half.begin(), t.half.end());
  }
  if (cudaMalloc(&h->d_axis, blob.size() * 4) != cudaSuccess) {
    delete ax;
    return fail(SPKGPU_ERR_NOMEM);
  }
  if (cudaMemcpy(h->d_axis, blob.data(), blob.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
    delete ax;
    return fail(SPKGPU_ERR_CUDA);
  }
  h->axes = ax;
  h->fused_ok = (!packed && (d.variant == 0 || d.variant == 2) && d.nsector == 1 && d.nloop == 1 &&
                 d.rng == SPKGPU_RNG_PHILOX && !d.mask &&
                 spk::fused2d_supported(d.lattice, d.app, sb, d.nx, d.ny));
  h->resident_ok = h->fused_ok && d.variant == 0 && spk::resident_supported(d.lattice, d.app, sb, d.nx, d.ny) &&
                   resident_is_faster(h);
  if (h->fused_ok) {
    if (cudaMalloc(&h->d_spin_alt, (size_t)h->n * sb) != cudaSuccess) return fail(SPKGPU_ERR_NOMEM);
  }
  h->rows_ok = (!packed && d.variant == 0 && d.nsector == 1 && d.nloop == 1 && d.rng == SPKGPU_RNG_PHILOX &&
                !d.mask && spk::rows_supported(d.lattice, sb, d.nx, d.nspins));
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return fail(SPKGPU_ERR_CUDA);
  *out = h;
  return code;
}

int spkgpu_destroy(spkgpu_lattice *h) {
  if (!h) return SPKGPU_ERR_ARG;
  if (h->stream) cudaStreamSynchronize(h->stream);
  spk_kmc_free(h);
  cudaFree(h->d_spin);
  cudaFree(h->d_spin_alt);
  cudaFree(h->d_decisions);
  cudaFree(h->d_seeds);
  cudaFree(h->d_mask);
  cudaFree(h->d_counters);
  cudaFree(h->d_labels);
  cudaFree(h->d_stage);
  cudaFree(h->d_axis);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h->axes;
  delete h;
  return SPKGPU_OK;
}

int spkgpu_set_temperature(spkgpu_lattice *h, double temperature) {
  if (!h) return SPKGPU_ERR_ARG;
  if (!(temperature >= 0.0) || isinf(temperature))
    return spk_fail(h, SPKGPU_ERR_ARG, "temperature must be finite and >= 0");
  h->temperature = temperature;
  h->have_temperature = true;
  spk::build_accept_table(temperature, h->d.app, &h->acc);
  return SPKGPU_OK;
}

static int ensure_stage(spkgpu_lattice *h, int64_t want) {
  if (h->stage_n >= want) return SPKGPU_OK;
  cudaFree(h->d_stage);
  h->d_stage = nullptr;
  h->stage_n = 0;
  if (cudaMalloc(&h->d_stage, (size_t)want * 4) != cudaSuccess)
    return spk_fail(h, SPKGPU_ERR_NOMEM, "staging buffer allocation failed");
  h->stage_n = want;
  return SPKGPU_OK;
}

static const int64_t kStageChunk = (int64_t)1 << 24;  // 16 Mi sites (64 MiB) per staging pass

int spkgpu_upload_spins(spkgpu_lattice *h, const int32_t *spin, int64_t n) {
  if (!h || !spin) return SPKGPU_ERR_ARG;
  if (n != h->n) return spk_fail(h, SPKGPU_ERR_ARG, "site count mismatch");
  int *bad = (int *)(h->d_counters + 2);
  SPK_CUDA(h, cudaMemsetAsync(bad, 0, sizeof(int), h->stream));
  // registered pinned host memory: the conversion kernel reads it directly
  // (one pass over NVLink-C2C or PCIe, no staging copy)
  const int32_t *mapped = (const int32_t *)spk::mapped_host_ptr(spin);
  if (mapped) {
    if (h->packed)
      SPK_CUDA(h, spk::launch_packed_pack(mapped, (uint64_t *)h->d_spin, n / 64, bad, h->stream, h->num_sms));
    else
      SPK_CUDA(h, spk::launch_convert_in(h->spin_bytes, mapped, h->d_spin, n, h->d.nspins, bad, h->stream));
    h->launches++;
  }
  int rc = mapped ? SPKGPU_OK : ensure_stage(h, std::min(n, kStageChunk) + 1);
  if (rc) return rc;
  for (int64_t off = 0; !mapped && off < n; off += kStageChunk) {
    int64_t m = std::min(kStageChunk, n - off);
    SPK_CUDA(h, cudaMemcpyAsync(h->d_stage, spin + off, (size_t)m * 4, cudaMemcpyHostToDevice, h->stream));
    if (h->packed)
      SPK_CUDA(h, spk::launch_packed_pack(h->d_stage, (uint64_t *)h->d_spin + off / 64, m / 64, bad, h->stream,
                                          h->num_sms));
    else
      SPK_CUDA(h, spk::launch_convert_in(h->spin_bytes, h->d_stage, (char *)h->d_spin + off * h->spin_bytes, m,
                                         h->d.nspins, bad, h->stream));
    h->launches++;
  }
  int badh = 0;
  SPK_CUDA(h, cudaMemcpyAsync(&badh, bad, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  SPK_CUDA(h, cudaStreamSynchronize(h->stream));
  if (badh) return spk_fail(h, SPKGPU_ERR_INVALID_SPIN, "One or more sites have invalid values");
  return SPKGPU_OK;
}

int spkgpu_init_spins(spkgpu_lattice *h, int32_t lo, int32_t hi) {
  if (!h) return SPKGPU_ERR_ARG;
  if (lo < 1 || hi < lo || hi > h->d.nspins) return spk_fail(h, SPKGPU_ERR_ARG, "values must lie in 1..nspins");
  if (h->packed && (lo != 1 || hi != 2)) return spk_fail(h, SPKGPU_ERR_ARG, "packed lattices take 1..2");
  SPK_CUDA(h, spk::launch_init(h->packed ? -1 : h->spin_bytes, h->d_spin, h->n, h->d.seed, lo, hi, h->stream,
                               h->num_sms));
  h->launches++;
  SPK_CUDA(h, cudaStreamSynchronize(h->stream));
  return SPKGPU_OK;
}

int spkgpu_download_spins(spkgpu_lattice *h, int32_t *spin, int64_t n) {
  if (!h || !spin) return SPKGPU_ERR_ARG;
  if (n != h->n) return spk_fail(h, SPKGPU_ERR_ARG, "site count mismatch");
  // registered pinned host memory: the conversion kernel writes it directly
  int32_t *mapped = (int32_t *)spk::mapped_host_ptr(spin);
  if (mapped) {
    if (h->packed)
      SPK_CUDA(h, spk::launch_packed_unpack((const uint64_t *)h->d_spin, mapped, n / 64, h->stream, h->num_sms));
    else
      SPK_CUDA(h, spk::launch_convert_out(h->spin_bytes, h->d_spin, mapped, n, h->stream));
    h->launches++;
    SPK_CUDA(h, cudaStreamSynchronize(h->stream));
    return SPKGPU_OK;
  }
  int rc = ensure_stage(h, std::min(n, kStageChunk) + 1);
  if (rc) return rc;
  for (int64_t off = 0; off < n; off += kStageChunk) {
    int64_t m = std::min(kStageChunk, n - off);
    if (h->packed)
      SPK_CUDA(h, spk::launch_packed_unpack((const uint64_t *)h->d_spin + off / 64, h->d_stage, m / 64, h->stream,
                                            h->num_sms));
    else
      SPK_CUDA(h, spk::launch_convert_out(h->spin_bytes, (const char *)h->d_spin + off * h->spin_bytes, h->d_stage,
                                          m, h->stream));
    h->launches++;
    SPK_CUDA(h, cudaMemcpyAsync(spin + off, h->d_stage, (size_t)m * 4, cudaMemcpyDeviceToHost, h->stream));
  }
  SPK_CUDA(h, cudaStreamSynchronize(h->stream));
  return SPKGPU_OK;
}

int spkgpu_upload_siteseeds(spkgpu_lattice *h, const int32_t *seeds, int64_t n) {
  if (!h || !seeds) return SPKGPU_ERR_ARG;
  if (!h->d_seeds) return spk_fail(h, SPKGPU_ERR_STATE, "handle is not in strict RNG mode");
  if (n != h->n) return spk_fail(h, SPKGPU_ERR_ARG, "site count mismatch");
  SPK_CUDA(h, cudaMemcpyAsync(h->d_seeds, seeds, (size_t)n * 4, cudaMemcpyHostToDevice, h->stream));
  SPK_CUDA(h, cudaStreamSynchronize(h->stream));
  return SPKGPU_OK;
}

int spkgpu_download_siteseeds(spkgpu_lattice *h, int32_t *seeds, int64_t n) {
  if (!h || !seeds) return SPKGPU_ERR_ARG;
  if (!h->d_seeds) return spk_fail(h, SPKGPU_ERR_STATE, "handle is not in strict RNG mode");
  if (n != h->n) return spk_fail(h, SPKGPU_ERR_ARG, "site count mismatch");
  SPK_CUDA(h, cudaMemcpyAsync(seeds, h->d_seeds, (size_t)n * 4, cudaMemcpyDeviceToHost, h->stream));
  SPK_CUDA(h, cudaStreamSynchronize(h->stream));
  return SPKGPU_OK;
}

int spkgpu_upload_mask(spkgpu_lattice *h, const uint8_t *mask, int64_t n) {
  if (!h || !mask) return SPKGPU_ERR_ARG;
  if (!h->d_mask) return spk_fail(h, SPKGPU_ERR_STATE, "handle has no mask");
  if (n != h->n) return spk_fail(h, SPKGPU_ERR_ARG, "site count mismatch");
  SPK_CUDA(h, cudaMemcpyAsync(h->d_mask, mask, (size_t)n, cudaMemcpyHostToDevice, h->stream));
  SPK_CUDA(h, cudaStreamSynchronize(h->stream));
  return SPKGPU_OK;
}

int spkgpu_download_mask(spkgpu_lattice *h, uint8_t *mask, int64_t n) {
  if (!h || !mask) return SPKGPU_ERR_ARG;
  if (!h->d_mask) return spk_fail(h, SPKGPU_ERR_STATE, "handle has no mask");
  if (n != h->n) return spk_fail(h, SPKGPU_ERR_ARG, "site count mismatch");
  SPK_CUDA(h, cudaMemcpyAsync(mask, h->d_mask, (size_t)n, cudaMemcpyDeviceToHost, h->stream));
  SPK_CUDA(h, cudaStreamSynchronize(h->stream));
  return SPKGPU_OK;
}

int spkgpu_set_sweep_index(spkgpu_lattice *h, int64_t sweep) {
  if (!h || sweep < 0) return SPKGPU_ERR_ARG;
  h->sweep = sweep;
  return SPKGPU_OK;
}

static int enqueue_sweeps(spkgpu_lattice *h, int32_t nsweeps) {
  const spkgpu_desc &d = h->d;
  spkgpu_axes_store *ax = h->axes;
  const int32_t *A = h->d_axis;
  unsigned long long *nacc = h->d_counters + kNacceptSlots;
  bool z3 = !spk::is2d(d.lattice);
  int nsec = d.nsector;
  if (h->resident_ok && nsweeps > 0) {
    // every sweep of the call in one launch, in place
    SPK_CUDA(h, spk::launch_resident_sweeps(d.app, h->spin_bytes, h->d_spin, d.nx, d.ny, d.seed, (uint32_t)h->sweep,
                                            nsweeps, d.nspins, nacc, h->acc, h->stream));
    h->launches++;
    h->sweep += nsweeps;
    h->nsweeps_done += nsweeps;
    h->nattempt += h->n * (int64_t)nsweeps;
    return SPKGPU_OK;
  }
  for (int32_t s = 0; s < nsweeps; s++) {
    uint32_t sweep = (uint32_t)h->sweep;
    if (h->packed) {
      spk::PackedArgs pa;
      pa.words = h->d_spin;
      pa.decisions = h->d_decisions;
      pa.nx = d.nx;
      pa.ny = d.ny;
      pa.nz = d.nz;
      pa.nwords = h->n / 64;
      pa.seed = d.seed;
      pa.sweep = sweep;
      pa.thr2 = h->acc.thr[2];
      pa.thr4 = h->acc.thr[4];
      pa.thr6 = h->acc.thr[6];
      pa.naccept = nacc;
      SPK_CUDA(h, spk::launch_packed_sweep(pa, h->stream, h->num_sms));
      h->launches += 3;
    } else if (h->rows_ok) {
      int nl = 0;
      SPK_CUDA(h, spk::launch_rows_sweep(d.lattice, d.app, h->spin_bytes, h->d_spin, d.nx, d.ny, d.nz, d.seed,
                                         sweep, d.nspins, nacc, h->acc, h->stream, &nl));
      h->launches += nl;
    } else if (h->fused_ok) {
      spk::FusedArgs f;
      f.src = h->d_spin;
      f.dst = h->d_spin_alt;
      f.nx = d.nx;
      f.ny = d.ny;
      f.seed = d.seed;
      f.sweep = sweep;
      f.nspins = d.nspins;
      f.naccept = nacc;
      f.acc = h->acc;
      SPK_CUDA(h, spk::launch_fused2d(d.lattice, d.app, h->spin_bytes, f, h->stream, h->num_sms));
      h->launches++;
      std::swap(h->d_spin, h->d_spin_alt);
    } else {
      for (int isec = 1; isec <= nsec; isec++) {
        int hx = sector_half(nsec, isec, 0), hy = sector_half(nsec, isec, 1), hz = z3 ? sector_half(nsec, isec, 2) : 2;
        if (d.mask && nsec > 1) {
          spk::MaskClearArgs m;
          m.mask = h->d_mask;
          m.nx = d.nx;
          m.ny = d.ny;
          m.nz = d.nz;
          m.xl = A + ax->off[0][hx][2];
          m.nxl = ax->len[0][hx][2];
          m.yl = A + ax->off[1][hy][2];
          m.nyl = ax->len[1][hy][2];
          m.zl = A + ax->off[2][hz][2];
          m.nzl = ax->len[2][hz][2];
          m.color = 0;
          m.proc_x = A + h->proc_off[0];
          m.proc_y = A + h->proc_off[1];
          m.proc_z = A + h->proc_off[2];
          m.half_x = A + h->half_off[0];
          m.half_y = A + h->half_off[1];
          m.half_z = A + h->half_off[2];
          SPK_CUDA(h, spk::launch_mask_clear(d.lattice, m, h->stream, h->num_sms));
          h->launches++;
        }
        for (int c = 1; c <= h->ncolors; c++) {
          if (d.mask && nsec == 1) {
            spk::MaskClearArgs m;
            memset(&m, 0, sizeof(m));
            m.mask = h->d_mask;
            m.nx = d.nx;
            m.ny = d.ny;
            m.nz = d.nz;
            m.xl = A + ax->off[0][2][2];
            m.nxl = ax->len[0][2][2];
            m.yl = A + ax->off[1][2][2];
            m.nyl = ax->len[1][2][2];
            m.zl = A + ax->off[2][2][2];
            m.nzl = ax->len[2][2][2];
            m.color = c;
            SPK_CUDA(h, spk::launch_mask_clear(d.lattice, m, h->stream, h->num_sms));
            h->launches++;
          }
          spk::PhaseArgs p;
          memset(&p, 0, sizeof(p));
          p.spin = h->d_spin;
          p.nx = d.nx;
          p.ny = d.ny;
          p.nz = d.nz;
          int cm = c - 1;
          int qx = 2, qy = 2, qz = 2;
          if (d.lattice == SPKGPU_SQ_8N) {
            qx = cm & 1;
            qy = (cm >> 1) & 1;
          } else if (d.lattice == SPKGPU_SC_26N) {
            qx = cm & 1;
            qy = (cm >> 1) & 1;
            qz = (cm >> 2) & 1;
          }
          if (qx == 2) {
            p.xpar_fixed = 0;
            p.xl[0] = A + ax->off[0][hx][0];
            p.nxl[0] = ax->len[0][hx][0];
            p.xl[1] = A + ax->off[0][hx][1];
            p.nxl[1] = ax->len[0][hx][1];
          } else {
            p.xpar_fixed = 1;
            p.xl[0] = p.xl[1] = A + ax->off[0][hx][qx];
            p.nxl[0] = p.nxl[1] = ax->len[0][hx][qx];
          }
          p.yl = A + ax->off[1][hy][qy];
          p.nyl = ax->len[1][hy][qy];
          p.zl = A + ax->off[2][hz][qz];
          p.nzl = ax->len[2][hz][qz];
          p.color = c;
          p.seed = d.seed;
          p.sweep = sweep;
          p.nspins = d.nspins;
          p.rng = d.rng;
          p.mask_on = d.mask;
          p.siteseeds = h->d_seeds;
          p.mask = h->d_mask;
          p.naccept = nacc;
          p.acc = h->acc;
          for (int pass = 0; pass < d.nloop; pass++) {
            p.pass = (uint32_t)pass;
            SPK_CUDA(h, spk::launch_phase(d.lattice, d.app, h->spin_bytes, p, h->stream, h->num_sms));
            h->launches++;
          }
        }
      }
    }
    h->sweep++;
    h->nsweeps_done++;
    h->nattempt += h->n * d.nloop;
  }
  return SPKGPU_OK;
}

int spkgpu_sweep(spkgpu_lattice *h, int32_t nsweeps) {
  if (!h || nsweeps < 0) return SPKGPU_ERR_ARG;
  if (!h->have_temperature) return spk_fail(h, SPKGPU_ERR_STATE, "temperature has not been set");
  return enqueue_sweeps(h, nsweeps);
}

int spkgpu_timed_sweeps(spkgpu_lattice *h, int32_t nsweeps, float *ms) {
  if (!h || !ms || nsweeps < 0) return SPKGPU_ERR_ARG;
  if (!h->have_temperature) return spk_fail(h, SPKGPU_ERR_STATE, "temperature has not been set");
  SPK_CUDA(h, cudaEventRecord(h->ev0, h->stream));
  int rc = enqueue_sweeps(h, nsweeps);
  if (rc) return rc;
  SPK_CUDA(h, cudaEventRecord(h->ev1, h->stream));
  SPK_CUDA(h, cudaEventSynchronize(h->ev1));
  SPK_CUDA(h, cudaEventElapsedTime(ms, h->ev0, h->ev1));
  return SPKGPU_OK;
}

int spkgpu_get_stats(spkgpu_lattice *h, spkgpu_stats *out) {
  if (!h || !out) return SPKGPU_ERR_ARG;
  unsigned long long slots[spk::kCounterSlots];
  SPK_CUDA(h, cudaMemcpyAsync(slots, h->d_counters + kNacceptSlots, sizeof(slots), cudaMemcpyDeviceToHost,
                              h->stream));
  SPK_CUDA(h, cudaStreamSynchronize(h->stream));
  unsigned long long na = 0;
  for (int k = 0; k < spk::kCounterSlots; k++) na += slots[k];
  out->naccept = (int64_t)na;
  out->nattempt = h->nattempt;
  out->nsweeps = h->nsweeps_done;
  return SPKGPU_OK;
}

int spkgpu_energy(spkgpu_lattice *h, double *energy) {
  if (!h || !energy) return SPKGPU_ERR_ARG;
  unsigned long long *acc = h->d_counters + 1;
  SPK_CUDA(h, cudaMemsetAsync(acc, 0, sizeof(unsigned long long), h->stream));
  if (h->packed)
    SPK_CUDA(h, spk::launch_packed_energy((const uint64_t *)h->d_spin, h->d.nx, h->d.ny, h->d.nz, acc, h->stream,
                                          h->num_sms));
  else
    SPK_CUDA(h, spk::launch_energy(h->d.lattice, h->spin_bytes, h->d_spin, h->d.nx, h->d.ny, h->d.nz, acc,
                                   h->stream, h->num_sms));
  h->launches++;
  unsigned long long e = 0;
  SPK_CUDA(h, cudaMemcpyAsync(&e, acc, sizeof(e), cudaMemcpyDeviceToHost, h->stream));
  SPK_CUDA(h, cudaStreamSynchronize(h->stream));
  *energy = (double)e;
  return SPKGPU_OK;
}

int spkgpu_synchronize(spkgpu_lattice *h) {
  if (!h) return SPKGPU_ERR_ARG;
  SPK_CUDA(h, cudaStreamSynchronize(h->stream));
  return SPKGPU_OK;
}

int spkgpu_stream(spkgpu_lattice *h, void **stream) {
  if (!h || !stream) return SPKGPU_ERR_ARG;
  *stream = (void *)h->stream;
  return SPKGPU_OK;
}

int spkgpu_device_spins(spkgpu_lattice *h, void **dptr, int64_t *bytes) {
  if (!h || !dptr || !bytes) return SPKGPU_ERR_ARG;
  *dptr = h->d_spin;
  *bytes = h->packed ? h->n / 8 : h->n * h->spin_bytes;
  return SPKGPU_OK;
}

int spkgpu_launch_count(const spkgpu_lattice *h, int64_t *count) {
  if (!h || !count) return SPKGPU_ERR_ARG;
  *count = h->launches;
  return SPKGPU_OK;
}

}  // extern "C"
