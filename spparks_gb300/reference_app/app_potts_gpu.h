/* app_style potts/gpu Q: AppPotts (src/app_potts.h) with its sweeps and
   tree KMC on the GB300 path (app_gpu.h).  AppPotts reads its arguments only
   under its own style name (src/app_potts.cpp:45-52), so they are read here
   the same way. */
#ifdef APP_CLASS
AppStyle(potts/gpu,AppPottsGPU)
#else
#ifndef SPK_APP_POTTS_GPU_H
#define SPK_APP_POTTS_GPU_H

#include <stdlib.h>

#include "app_gpu.h"
#include "app_potts.h"

namespace SPPARKS_NS {

class AppPottsGPU : public AppGPU<AppPotts> {
 public:
  AppPottsGPU(class SPPARKS *spk, int narg, char **arg) : AppGPU<AppPotts>(spk, narg, arg) {
    if (narg != 2) error->all(FLERR, "Illegal app_style command");
    nspins = atoi(arg[1]);
    if (nspins <= 0) error->all(FLERR, "Illegal app_style command");
    dt_sweep = 1.0 / nspins;
  }

 protected:
  int nspins_of() const override { return nspins; }
};

}  // namespace SPPARKS_NS

#endif
#endif
