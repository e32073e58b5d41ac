// Calibration of the integer-issue ceiling of the sweep kernels: how many
// Philox4x32-10 blocks per second this device computes with the sweeps' own
// Philox code (hoisted round keys, four independent blocks per thread in
// flight), with nothing else in the loop.  An Ising sweep of the Philox draw
// contract spends one block per four sites and the other apps one per x-pair,
// so four (ising) or two times this rate bounds a sweep from above.  No
// counterpart in the reference.

#include <cuda_runtime.h>

#include "../../include/spkgpu.h"
#include "spk_philox.cuh"

namespace spk {
namespace {

constexpr int kCalibThreads = 128;
constexpr int kCalibIlp = 4;

__global__ void __launch_bounds__(kCalibThreads, 8) philox_rate_kernel(uint32_t seed, int iters, uint32_t *out) {
  const RoundKeys rk = round_keys(seed, kStreamSweep);
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t acc = 0;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < kCalibIlp; k++) {
      U4 w = philox4x32_10_rk(U4{t * kCalibIlp + k, (uint32_t)i, 7u, 0u}, rk);
      acc ^= w.x ^ w.y ^ w.z ^ w.w;
    }
  }
  out[t] = acc;  // keeps the blocks live
}

}  // namespace
}  // namespace spk

extern "C" int spkgpu_philox_rate(int32_t device, int32_t iters, double *blocks_per_s) {
  if (!blocks_per_s || iters <= 0) return SPKGPU_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return SPKGPU_ERR_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms <= 0)
    return SPKGPU_ERR_CUDA;
  const int grid = sms * 8;
  uint32_t *out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = SPKGPU_OK;
  if (cudaMalloc(&out, (size_t)grid * spk::kCalibThreads * 4) != cudaSuccess) return SPKGPU_ERR_NOMEM;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = SPKGPU_ERR_CUDA;
  // best of three timed launches after three warm-up launches
  float ms = 0.0f;
  if (rc == SPKGPU_OK) {
    for (int w = 0; w < 3; w++) spk::philox_rate_kernel<<<grid, spk::kCalibThreads>>>(12345u, iters, out);
    for (int r = 0; r < 3 && rc == SPKGPU_OK; r++) {
      float t = 0.0f;
      cudaEventRecord(e0);
      spk::philox_rate_kernel<<<grid, spk::kCalibThreads>>>(12345u, iters, out);
      cudaEventRecord(e1);
      if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&t, e0, e1) != cudaSuccess || t <= 0.0f)
        rc = SPKGPU_ERR_CUDA;
      else if (ms == 0.0f || t < ms)
        ms = t;
    }
  }
  if (rc == SPKGPU_OK)
    *blocks_per_s = (double)grid * spk::kCalibThreads * (double)iters * spk::kCalibIlp / (ms * 1e-3);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(out);
  return rc;
}
