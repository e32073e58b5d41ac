// Rejection-free KMC with the tree solver over sectors (filled in below).
#include "spk_internal.h"

void spk_kmc_free(spkgpu_lattice *) {}

extern "C" int spkgpu_kmc_setup(spkgpu_lattice *h, int32_t, double, double, int32_t) {
  return spk_fail(h, SPKGPU_ERR_UNSUPPORTED, "KMC not built yet");
}
extern "C" int spkgpu_kmc_run(spkgpu_lattice *h, double *, double, spkgpu_kmc_stats *) {
  return spk_fail(h, SPKGPU_ERR_UNSUPPORTED, "KMC not built yet");
}
