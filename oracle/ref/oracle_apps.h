/* Oracle (test infrastructure only): subclasses of the reference's own apps
   and tree solver, registered under the reference's style names in the
   Philox build of the reference (oracle/ref/Makefile).  They change no
   physics: each one opens a Philox draw context around the reference's own
   per-site or per-event routine and then calls it.

     site_event_rejection  src/app_ising.cpp:104-136, src/app_potts.cpp:112-146,
                           src/app_potts_neighonly.cpp:71-117,
                           src/app_potts_neigh.cpp:71-116
     site_event            src/app_potts.cpp:196-244 (word 2 of the event block)
     SolveTree::event      src/solve_tree.cpp:130-143 (words 0 and 1)
     app_update            called once per pass by src/app_lattice.cpp:700 and
                           :600; used here to record the lattice after each sweep
*/

#ifdef APP_CLASS
AppStyle(ising,AppIsingPhilox)
AppStyle(potts,AppPottsPhilox)
AppStyle(potts/neighonly,AppPottsNeighOnlyPhilox)
AppStyle(potts/neigh,AppPottsNeighPhilox)
#else

#ifndef SPK_ORACLE_APPS_H
#define SPK_ORACLE_APPS_H

#include <vector>
#include <stdint.h>

#include "app_ising.h"
#include "app_potts.h"
#include "app_potts_neighonly.h"
#include "app_potts_neigh.h"

namespace spk_oracle {

struct SweepRecord {
  int sweep;
  long long naccept;
  long long nattempt;
  uint64_t hash;
  double time;
};

extern int record_on;
extern std::vector<SweepRecord> records;
uint64_t hash_spins(const int *spin, int n);

}  // namespace spk_oracle

namespace SPPARKS_NS {

template <class Base>
class PhiloxApp : public Base {
 public:
  PhiloxApp(class SPPARKS *spk, int narg, char **arg);
  void site_event_rejection(int, class RandomPark *);
  void site_event(int, class RandomPark *);
  void app_update(double);

 private:
  std::vector<int> visits;
  int visits_sweep;
};

typedef PhiloxApp<AppIsing> AppIsingPhilox;
typedef PhiloxApp<AppPotts> AppPottsPhilox;
typedef PhiloxApp<AppPottsNeighOnly> AppPottsNeighOnlyPhilox;
typedef PhiloxApp<AppPottsNeigh> AppPottsNeighPhilox;

}  // namespace SPPARKS_NS

#endif
#endif
