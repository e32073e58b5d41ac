/* Oracle (test infrastructure only): implementation of the Philox-context
   subclasses declared in oracle_apps.h and oracle_solve.h.  See those
   headers for the reference routines each one wraps. */

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "oracle_apps.h"
#include "oracle_solve.h"
#include "shim_ctx.h"
#include "../philox_oracle.h"

namespace spk_oracle {
int record_on = 0;
std::vector<SweepRecord> records;
uint32_t last_event_words[4] = {0, 0, 0, 0};
int last_event_valid = 0;

uint64_t hash_spins(const int *spin, int n) {
  uint64_t h = 1469598103934665603ULL;
  for (int i = 0; i < n; i++) {
    uint32_t v = (uint32_t)spin[i];
    for (int b = 0; b < 4; b++) {
      h ^= (v >> (8 * b)) & 0xFFu;
      h *= 1099511628211ULL;
    }
  }
  return h;
}
}  // namespace spk_oracle

using namespace SPPARKS_NS;

template <class Base>
PhiloxApp<Base>::PhiloxApp(SPPARKS *spk, int narg, char **arg)
    : Base(spk, narg, arg), visits_sweep(-1) {
  this->allow_app_update = 1;
}

template <class Base>
void PhiloxApp<Base>::site_event_rejection(int i, RandomPark *random) {
  // pass index = how many times this site was already visited in this sweep
  // (non-zero only when sector nstop > 1 loops a set several times)
  if (visits_sweep != this->nsweeps || (int)visits.size() != this->nlocal) {
    visits.assign(this->nlocal, 0);
    visits_sweep = this->nsweeps;
  }
  // ising: one word per site, four sites per block; the other apps: two
  // words per site, two sites per block
  const bool ising = std::is_same<Base, AppIsing>::value;
  uint64_t s = (uint64_t)(this->id[i] - 1);
  const int sh = ising ? 2 : 1;
  uint32_t ctr[4] = {(uint32_t)(s >> sh), (uint32_t)(s >> (32 + sh)), (uint32_t)this->nsweeps,
                     (uint32_t)visits[i]};
  uint32_t key[2] = {spk_shim::philox_seed, spk_shim::stream_base | SPKO_STREAM_SWEEP};
  spk_shim::DrawCtx &c = spk_shim::ctx;
  spko_philox4x32_10(ctr, key, c.w);
  c.base = ising ? (int)(s & 3) : (int)(s & 1) * 2;
  c.ising = ising ? 1 : 0;
  c.next = 0;
  c.limit = 2;
  c.active = 1;
  Base::site_event_rejection(i, random);
  c.active = 0;
  visits[i]++;
}

template <class Base>
void PhiloxApp<Base>::site_event(int i, RandomPark *random) {
  if (!spk_oracle::last_event_valid) {
    fprintf(stderr, "oracle: site_event without a preceding solver event\n");
    exit(3);
  }
  spk_shim::DrawCtx &c = spk_shim::ctx;
  memcpy(c.w, spk_oracle::last_event_words, sizeof(c.w));
  c.base = 2;
  c.ising = 0;
  c.next = 0;
  c.limit = 1;
  c.active = 1;
  Base::site_event(i, random);
  c.active = 0;
  spk_oracle::last_event_valid = 0;
}

template <class Base>
void PhiloxApp<Base>::app_update(double dt) {
  if (!spk_oracle::record_on) return;
  spk_oracle::SweepRecord r;
  r.sweep = this->nsweeps;
  r.naccept = (long long)this->naccept;
  r.nattempt = (long long)this->nattempt;
  r.hash = spk_oracle::hash_spins(this->iarray[0], this->nlocal);
  r.time = this->time + dt;
  spk_oracle::records.push_back(r);
}

template class SPPARKS_NS::PhiloxApp<AppIsing>;
template class SPPARKS_NS::PhiloxApp<AppPotts>;
template class SPPARKS_NS::PhiloxApp<AppPottsNeighOnly>;
template class SPPARKS_NS::PhiloxApp<AppPottsNeigh>;

/* ---------------------------------------------------------------------- */

SolveTreePhilox::SolveTreePhilox(SPPARKS *spk, int narg, char **arg)
    : SolveTree(spk, narg, arg), chain(0), nevent(0), nclones(0) {}

SolveTreePhilox *SolveTreePhilox::clone() {
  char *arg[1];
  arg[0] = style;
  SolveTreePhilox *p = new SolveTreePhilox(spk, 1, arg);
  p->chain = nclones++;
  return p;
}

int SolveTreePhilox::event(double *pdt) {
  if (get_total_propensity() == 0.0) return SolveTree::event(pdt);
  spk_shim::DrawCtx &c = spk_shim::ctx;
  spko_kmc_draws(spk_shim::philox_seed, chain, nevent, c.w);
  nevent++;
  c.base = 0;
  c.ising = 0;
  c.next = 0;
  c.limit = 2;
  c.active = 1;
  int m = SolveTree::event(pdt);
  c.active = 0;
  memcpy(spk_oracle::last_event_words, c.w, sizeof(c.w));
  spk_oracle::last_event_valid = 1;
  return m;
}
