/* Oracle shim (test infrastructure only): the Philox draw context shared by
   the RandomPark shim and the oracle app/solver subclasses. */
#ifndef SPK_SHIM_CTX_H
#define SPK_SHIM_CTX_H

#include <stdint.h>

namespace spk_shim {

struct DrawCtx {
  int active;      // 1 while a site update or KMC event is being drawn
  uint32_t w[4];   // one Philox4x32-10 block
  int base;        // first word this context may hand out
  int next;        // draws handed out so far
  int limit;       // draws allowed
  int ising;       // 1: both draws come from word `base` (ising sweeps)
};

extern DrawCtx ctx;
extern uint32_t philox_seed;
// high bits of the Philox key's stream word (replica r of an ensemble: (r+1) << 8)
extern uint32_t stream_base;

}  // namespace spk_shim

#endif
