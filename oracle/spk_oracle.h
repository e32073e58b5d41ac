/* Oracle (test infrastructure only; never part of the product path).
   A plain-C restatement of the SPPARKS on-lattice hot path, used by the
   tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the
   checker for the GPU kernels.  Every routine cites the reference routine it
   restates.  It is pinned by tests against (a) the reference's own example
   logs and (b) fixtures produced by the reference itself built with a
   Philox RandomPark shim (oracle/ref). */
#ifndef SPK_ORACLE_H
#define SPK_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { SPKO_SQ4 = 0, SPKO_SQ8 = 1, SPKO_SC6 = 2, SPKO_SC26 = 3 };
enum { SPKO_ISING = 0, SPKO_POTTS = 1, SPKO_NEIGHONLY = 2, SPKO_NEIGH = 3 };
enum { SPKO_RNG_PHILOX = 0, SPKO_RNG_STRICT = 1 };

typedef struct {
  int lattice;          /* SPKO_SQ4 ... */
  int nx, ny, nz;       /* nz = 1 for 2d lattices */
  int app;              /* SPKO_ISING ... */
  int nspins;           /* Q (2 for Ising) */
  double temperature;   /* reference units, as typed in `temperature` */
  int nsector;          /* 1 (no sectors), 2, 4, 8 */
  int nloop;            /* passes over each set per sweep (sector nstop) */
  int rng;              /* SPKO_RNG_PHILOX or SPKO_RNG_STRICT */
  uint32_t seed;        /* Philox key word 0 */
  int mask;             /* sweep ... mask yes */
  int px, py, pz;       /* processor grid (1 1 1 = serial) */
  uint32_t stream_base; /* Philox key word 1 = stream_base | stream; replica r
                           of an ensemble uses (r+1) << 8 */
} spko_cfg;

int spko_maxneigh(int lattice);
int spko_ncolors(int lattice);
int spko_neighbors(const spko_cfg *c, int64_t i, int64_t *out);
int spko_color(const spko_cfg *c, int64_t i);
int spko_sector(const spko_cfg *c, int64_t i);
double spko_energy(const spko_cfg *c, const int32_t *spin);
int spko_clusters(const spko_cfg *c, const int32_t *spin, int64_t *ncluster, double *vav, double *rav);
uint64_t spko_hash(const int32_t *spin, int64_t n);
void spko_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void spko_init_spins(uint32_t seed, int64_t n, int lo, int hi, int32_t *spin);
/* the initial values of the sites ids[0..n-1] alone (as spko_init_spins) */
void spko_init_values(uint32_t seed, int64_t n, const int64_t *ids, int lo, int hi, int32_t *out);

/* Rejection (rKMC) colour sweeps.  Runs nsweeps sweeps starting at sweep
   index sweep0.  naccept/nattempt accumulate; hashes (optional) receive the
   lattice hash after each sweep.  siteseeds is the per-site Park-Miller
   state for SPKO_RNG_STRICT, mask the per-site mask bytes when c->mask. */
int spko_color_sweeps(const spko_cfg *c, int32_t *spin, int64_t sweep0, int nsweeps,
                      int64_t *naccept, int64_t *nattempt, uint64_t *hashes,
                      int32_t *siteseeds, uint8_t *mask);

/* Single site updates for lattices too large for a full oracle run: site
   ids[k] with value self[k] and its neighbours' values nbv[k*nn .. k*nn+nn-1]
   (nn = maxneigh, in spko_neighbors order) as the site sees them at its turn
   in colour sweep `sweep`, pass `pass` (Philox draws); out[k] = its value
   after its site_event_rejection.  Returns the number of changed sites. */
int64_t spko_site_updates(const spko_cfg *c, int64_t n, const int64_t *ids, const int32_t *self,
                          const int32_t *nbv, uint32_t sweep, uint32_t pass, int32_t *out);
/* neighbour ids of n sites, nn = maxneigh per site (spko_neighbors order) */
void spko_neighbors_many(const spko_cfg *c, int64_t n, const int64_t *ids, int64_t *out);

/* Park-Miller / Marsaglia restatements for the reference's own seeding */
typedef struct {
  double u[98];
  double c, cd, cm;
  int i97, j97;
} spko_ranmars;
void spko_ranmars_init(spko_ranmars *r, int seed);
double spko_ranmars_uniform(spko_ranmars *r);
double spko_park_uniform(int32_t *seed);
int32_t spko_park_seed_from_double(double rseed);
int32_t spko_park_reset(double rseed, int64_t offset, int warmup);
/* `set site range lo hi` with the default loop option */
void spko_set_range(int32_t park_seed, int64_t n, int lo, int hi, int32_t *spin);

/* `sweep random` with sectors (serial; reproduces the reference example
   logs).  Runs nsweeps passes with one Park-Miller stream (*ranapp). */
int spko_random_sector_sweeps(const spko_cfg *c, int32_t *spin, int32_t *ranapp, int nsweeps,
                              int64_t *naccept, int64_t *nattempt);

/* Rejection-free KMC with the tree solver over sectors (and an optional
   processor grid), Philox draws.  State persists in an opaque object so
   that consecutive runs equal one continuous run. */
typedef struct spko_kmc spko_kmc;
spko_kmc *spko_kmc_create(const spko_cfg *c, int nstop_mode, double nstop, double tstop);
void spko_kmc_destroy(spko_kmc *k);
/* one `run dt` command: returns number of passes done, updates *time */
int spko_kmc_run(spko_kmc *k, int32_t *spin, double *time, double stoptime, int64_t *naccept,
                 uint64_t *hashes, double *pass_times, int maxrec);
double spko_kmc_total_propensity(spko_kmc *k);
int spko_kmc_nchains(spko_kmc *k);
uint64_t spko_kmc_chain_events(spko_kmc *k, int chain);

#ifdef __cplusplus
}
#endif
#endif
