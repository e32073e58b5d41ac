/* The one non-template piece of the GPU app styles (app_gpu.h): the call
   of Output::compute, kept in its own file because output.h has no include
   guard and the style headers are included next to it. */

#include "app_gpu.h"
#include "output.h"

namespace SPPARKS_NS {

double spk_gpu_output_compute(SPPARKS *spk, double time, int done) { return spk->output->compute(time, done); }

}  // namespace SPPARKS_NS
