/* Oracle (test infrastructure only): the reference's SolveTree
   (src/solve_tree.cpp) with a Philox draw context opened around event()
   (src/solve_tree.cpp:130-143).  Each clone owns one event chain (one KMC
   set, i.e. one sector); event k of chain c draws its tree pick and clock
   from words 0 and 1 of the Philox block (c, k), and the app's site_event
   draws word 2 of the same block. */

#ifdef SOLVE_CLASS
SolveStyle(tree,SolveTreePhilox)
#else

#ifndef SPK_ORACLE_SOLVE_H
#define SPK_ORACLE_SOLVE_H

#include <stdint.h>
#include "solve_tree.h"

namespace spk_oracle {
extern uint32_t last_event_words[4];
extern int last_event_valid;
}

namespace SPPARKS_NS {

class SolveTreePhilox : public SolveTree {
 public:
  SolveTreePhilox(class SPPARKS *, int, char **);
  SolveTreePhilox *clone();
  int event(double *);

 private:
  uint32_t chain;
  uint64_t nevent;
  uint32_t nclones;
};

}  // namespace SPPARKS_NS

#endif
#endif
