/* app_style ising/gpu: AppIsing (src/app_ising.h) with its sweeps and tree
   KMC on the GB300 path (app_gpu.h). */
#ifdef APP_CLASS
AppStyle(ising/gpu,AppIsingGPU)
#else
#ifndef SPK_APP_ISING_GPU_H
#define SPK_APP_ISING_GPU_H

#include "app_gpu.h"
#include "app_ising.h"

namespace SPPARKS_NS {

class AppIsingGPU : public AppGPU<AppIsing> {
 public:
  AppIsingGPU(class SPPARKS *spk, int narg, char **arg) : AppGPU<AppIsing>(spk, narg, arg) {}
};

}  // namespace SPPARKS_NS

#endif
#endif
