/* app_style potts/neighonly/gpu Q: AppPottsNeighOnly
   (src/app_potts_neighonly.h) with its sweeps and tree KMC on the GB300 path
   (app_gpu.h); its arguments are read as AppPottsNeighOnly reads them
   (src/app_potts_neighonly.cpp:34-41). */
#ifdef APP_CLASS
AppStyle(potts/neighonly/gpu,AppPottsNeighOnlyGPU)
#else
#ifndef SPK_APP_POTTS_NEIGHONLY_GPU_H
#define SPK_APP_POTTS_NEIGHONLY_GPU_H

#include <stdlib.h>

#include "app_gpu.h"
#include "app_potts_neighonly.h"

namespace SPPARKS_NS {

class AppPottsNeighOnlyGPU : public AppGPU<AppPottsNeighOnly> {
 public:
  AppPottsNeighOnlyGPU(class SPPARKS *spk, int narg, char **arg) : AppGPU<AppPottsNeighOnly>(spk, narg, arg) {
    if (narg != 2) error->all(FLERR, "Illegal app_style command");
    nspins = atoi(arg[1]);
    if (nspins <= 0) error->all(FLERR, "Illegal app_style command");
  }

 protected:
  int nspins_of() const override { return nspins; }
};

}  // namespace SPPARKS_NS

#endif
#endif
