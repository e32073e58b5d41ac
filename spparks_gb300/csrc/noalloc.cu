// spkgpu_sweep_sq4_noalloc: the fused sq/4n colour sweep (sweep_fused2d.cu)
// on a lattice the caller already holds in device memory, without any device
// allocation by this library.
//
// Who needs it: a caller that owns every byte of device memory through its
// own pool (for example a framework's caching allocator carved up at start),
// or one that must not pay the device-wide synchronisation that cudaMalloc
// and cudaFree may imply while other streams of the application are running.
// Such a caller passes the lattice (input and output, updated in place) and
// gets the change count back; the only extra memory is the fixed array below.
//
// The fused sweep is double-buffered: it reads the lattice and writes a
// second buffer, then the roles swap.  Here the second buffer and the change
// counter live in g_noalloc_scratch, a file-scope device array of fixed size
// that every GPU loading this library holds until the process exits.  Lattices
// larger than SPKGPU_NOALLOC_MAX_BYTES are rejected with SPKGPU_ERR_TOO_LARGE.
//
// The array is shared by every call on a device and keeps the contents of the
// last call; the counter is cleared at the start of each call.  Two calls
// whose work overlaps on the GPU (different streams, or different host
// threads) race on the array: serialise them.
//
// Host code cannot use the array's name as a device address (it names a host
// shadow), so the first call on each device looks the address up with
// cudaGetSymbolAddress while that device is current and caches it together
// with the device's current context.  That first call therefore does set-up
// work and should be made before any stream capture.  When the context
// changes (after cudaDeviceReset the runtime makes a new primary context and
// reloads the module), the next call looks the address up again, so a reset
// never leaves a stale address behind.
//
// With naccept set, the call reads the counter back and waits for the
// stream; that cannot be part of a stream capture, so such a call on a
// capturing stream is refused (SPKGPU_ERR_ARG) before anything is enqueued.

#include <cuda.h>
#include <cuda_runtime.h>
#include <math.h>

#include <mutex>

#include "counters.cuh"
#include "spk_internal.h"

namespace {

// change-counter slots (spk::kCounterSlots of 8 bytes), then the buffer
constexpr size_t kCounterBytes = 2048;
__device__ __align__(256) unsigned char g_noalloc_scratch[kCounterBytes + SPKGPU_NOALLOC_MAX_BYTES];

constexpr int kMaxDevices = 64;
void *g_scratch_ptr[kMaxDevices] = {nullptr};
CUcontext g_scratch_ctx[kMaxDevices] = {nullptr};
std::mutex g_scratch_mutex;

// the calling thread's current context (driver entry point reached through
// the runtime, so the library does not link the driver library itself)
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
int current_context(CUcontext *ctx) {
  // looked up once (thread-safe static initialisation)
  static const CtxGetCurrentFn fn = []() -> CtxGetCurrentFn {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return nullptr;
    return (CtxGetCurrentFn)p;
  }();
  if (!fn) return SPKGPU_ERR_CUDA;
  return fn(ctx) == CUDA_SUCCESS && *ctx ? SPKGPU_OK : SPKGPU_ERR_CUDA;
}

// address of the scratch array on the current device, looked up once per
// device and context
int scratch_on_current_device(unsigned char **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SPKGPU_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return SPKGPU_ERR_UNSUPPORTED;
  CUcontext ctx = nullptr;
  if (current_context(&ctx) != SPKGPU_OK) {
    // no context bound to this thread yet: bind the device's primary context
    if (cudaSetDevice(dev) != cudaSuccess) return SPKGPU_ERR_CUDA;
    int rc = current_context(&ctx);
    if (rc) return rc;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[dev] || g_scratch_ctx[dev] != ctx) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return SPKGPU_ERR_CUDA;
    g_scratch_ptr[dev] = p;
    g_scratch_ctx[dev] = ctx;
  }
  *out = (unsigned char *)g_scratch_ptr[dev];
  return SPKGPU_OK;
}

}  // namespace

extern "C" int spkgpu_sweep_sq4_noalloc(void *spin, int32_t nx, int32_t ny, int32_t spin_bytes, int32_t app,
                                        int32_t nspins, double temperature, uint32_t seed, int64_t sweep0,
                                        int32_t nsweeps, void *stream, int64_t *naccept) {
  if (!spin || nx <= 0 || ny <= 0 || nsweeps < 0 || sweep0 < 0) return SPKGPU_ERR_ARG;
  // the tile kernel moves site values in 8-byte chunks
  if ((uintptr_t)spin % 8 != 0) return SPKGPU_ERR_ARG;
  if (app < SPKGPU_ISING || app > SPKGPU_POTTS_NEIGH) return SPKGPU_ERR_ARG;
  if (app == SPKGPU_ISING && nspins != 2) return SPKGPU_ERR_ARG;
  if (nspins < 1 || nspins >= (1 << 21)) return SPKGPU_ERR_ARG;
  if ((spin_bytes == 1 && nspins > 127) || (spin_bytes == 2 && nspins > 32767)) return SPKGPU_ERR_ARG;
  if (!(temperature >= 0.0) || isinf(temperature)) return SPKGPU_ERR_ARG;
  if (!spk::fused2d_supported(SPKGPU_SQ_4N, app, spin_bytes, nx, ny)) return SPKGPU_ERR_ARG;
  size_t bytes = (size_t)nx * (size_t)ny * (size_t)spin_bytes;
  if (bytes > (size_t)SPKGPU_NOALLOC_MAX_BYTES) return SPKGPU_ERR_TOO_LARGE;

  cudaStream_t s = (cudaStream_t)stream;
  if (naccept) {
    // reading the counter back waits for the stream: not possible in a capture
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) return SPKGPU_ERR_CUDA;
    if (cap != cudaStreamCaptureStatusNone) return SPKGPU_ERR_ARG;
  }
  unsigned char *scratch = nullptr;
  int rc = scratch_on_current_device(&scratch);
  if (rc) return rc;
  unsigned long long *counter = (unsigned long long *)scratch;
  void *other = scratch + kCounterBytes;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);

  static_assert(kCounterBytes == spk::kCounterSlots * sizeof(unsigned long long), "counter slots");
  if (cudaMemsetAsync(counter, 0, kCounterBytes, s) != cudaSuccess) return SPKGPU_ERR_CUDA;
  spk::FusedArgs f;
  f.nx = nx;
  f.ny = ny;
  f.seed = seed;
  f.nspins = nspins;
  f.naccept = counter;
  spk::build_accept_table(temperature, app, &f.acc);
  for (int32_t k = 0; k < nsweeps; k++) {
    f.src = (k & 1) ? other : spin;
    f.dst = (k & 1) ? spin : other;
    f.sweep = (uint32_t)(sweep0 + k);
    if (spk::launch_fused2d(SPKGPU_SQ_4N, app, spin_bytes, f, s, sms) != cudaSuccess) return SPKGPU_ERR_CUDA;
  }
  // an odd number of sweeps leaves the result in the scratch buffer
  if (nsweeps & 1) {
    if (cudaMemcpyAsync(spin, other, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess) return SPKGPU_ERR_CUDA;
  }
  if (naccept) {
    unsigned long long v[spk::kCounterSlots];
    if (cudaMemcpyAsync(v, counter, sizeof(v), cudaMemcpyDeviceToHost, s) != cudaSuccess) return SPKGPU_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return SPKGPU_ERR_CUDA;
    unsigned long long tot = 0;
    for (int k = 0; k < spk::kCounterSlots; k++) tot += v[k];
    *naccept = (int64_t)tot;
  }
  return SPKGPU_OK;
}
