// Change counters (Naccept) without same-address contention: a CTA sums its
// threads' counts in shared memory and adds the total with one atomic into
// one of kCounterSlots slots (chosen by block index); readers sum the slots.
#pragma once

#include <stdint.h>

namespace spk {

constexpr int kCounterSlots = 256;

#ifdef __CUDACC__
// every thread of the block must call it (it synchronises the block)
__device__ __forceinline__ void block_count_add(unsigned long long *slots, unsigned long long v) {
  __shared__ unsigned long long block_total;
  if (threadIdx.x == 0) block_total = 0;
  __syncthreads();
  unsigned long long w = v;
  for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xFFFFFFFFu, w, o);
  if ((threadIdx.x & 31) == 0 && w) atomicAdd(&block_total, w);
  __syncthreads();
  if (threadIdx.x == 0 && block_total) atomicAdd(&slots[blockIdx.x & (kCounterSlots - 1)], block_total);
}
#endif

}  // namespace spk
