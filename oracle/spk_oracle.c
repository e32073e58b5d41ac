/* Oracle (test infrastructure only; never part of the product path).
   Plain-C restatement of the SPPARKS on-lattice hot path.  See spk_oracle.h.
   Lattice layout: site index i = x + nx*(y + ny*z) = id-1, the order in which
   create_sites numbers a structured lattice (src/create_sites.cpp:345-351). */

#include "spk_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "philox_oracle.h"

/* ---------------------------------------------------------------------- */
/* lattice geometry                                                        */
/* ---------------------------------------------------------------------- */

/* maxneigh per lattice style: src/create_sites.cpp:536-545 */
int spko_maxneigh(int lattice) {
  switch (lattice) {
    case SPKO_SQ4: return 4;
    case SPKO_SQ8: return 8;
    case SPKO_SC6: return 6;
    case SPKO_SC26: return 26;
  }
  return 0;
}

/* Lattice::ncolors with delcolor = 1: src/lattice.cpp:187-228 */
int spko_ncolors(int lattice) {
  switch (lattice) {
    case SPKO_SQ4: return 2;
    case SPKO_SQ8: return 4;
    case SPKO_SC6: return 2;
    case SPKO_SC26: return 8;
  }
  return 0;
}

/* neighbour offsets in the order of CreateSites::offsets_2d/3d
   (src/create_sites.cpp:1303-1371): dx outer, dy, dz inner, each -1..1,
   keeping those inside the distance window of the style */
static int offsets(int lattice, int off[26][3]) {
  int n = 0;
  int is3d = (lattice == SPKO_SC6 || lattice == SPKO_SC26);
  for (int dx = -1; dx <= 1; dx++)
    for (int dy = -1; dy <= 1; dy++)
      for (int dz = (is3d ? -1 : 0); dz <= (is3d ? 1 : 0); dz++) {
        int r2 = dx * dx + dy * dy + dz * dz;
        int keep = 0;
        if (lattice == SPKO_SQ4 || lattice == SPKO_SC6) keep = (r2 == 1);
        else keep = (r2 >= 1);
        if (!keep) continue;
        off[n][0] = dx;
        off[n][1] = dy;
        off[n][2] = dz;
        n++;
      }
  return n;
}

/* periodic remap of structured_connectivity (src/create_sites.cpp:589-621) */
int spko_neighbors(const spko_cfg *c, int64_t i, int64_t *out) {
  int off[26][3];
  int n = offsets(c->lattice, off);
  int64_t x = i % c->nx;
  int64_t y = (i / c->nx) % c->ny;
  int64_t z = i / ((int64_t)c->nx * c->ny);
  for (int j = 0; j < n; j++) {
    int64_t xn = (x + off[j][0] + c->nx) % c->nx;
    int64_t yn = (y + off[j][1] + c->ny) % c->ny;
    int64_t zn = (z + off[j][2] + c->nz) % c->nz;
    out[j] = xn + (int64_t)c->nx * (yn + (int64_t)c->ny * zn);
  }
  return n;
}

/* Lattice::id2color (src/lattice.cpp:234-283), returns 1..ncolors */
int spko_color(const spko_cfg *c, int64_t i) {
  int64_t x = i % c->nx;
  int64_t y = (i / c->nx) % c->ny;
  int64_t z = i / ((int64_t)c->nx * c->ny);
  switch (c->lattice) {
    case SPKO_SQ4: return (int)((x + y) % 2) + 1;
    case SPKO_SQ8: return (int)(2 * (y % 2) + x % 2) + 1;
    case SPKO_SC6: return (int)((x + y + z) % 2) + 1;
    case SPKO_SC26: return (int)(4 * (z % 2) + 2 * (y % 2) + x % 2) + 1;
  }
  return 0;
}

/* processor sub-domain along one axis (Domain::procs2domain_*,
   src/domain.cpp:174-330): proc p of P owns coordinates in
   [lo + p*prd/P, lo + (p+1)*prd/P); site coordinate = lattice index */
static int proc_of(int64_t x, int n, int P, double lo) {
  double prd = (double)n;
  for (int p = 0; p < P; p++) {
    double sublo = lo + p * prd / P;
    double subhi = (p < P - 1) ? lo + (p + 1) * prd / P : lo + prd;
    if ((double)x >= sublo && (double)x < subhi) return p;
  }
  return P - 1;
}

static double mid_of(int p, int n, int P, double lo) {
  double prd = (double)n;
  double sublo = lo + p * prd / P;
  double subhi = (p < P - 1) ? lo + (p + 1) * prd / P : lo + prd;
  return 0.5 * (sublo + subhi);
}

static int is2d(const spko_cfg *c) { return c->lattice == SPKO_SQ4 || c->lattice == SPKO_SQ8; }

/* box z bounds: 2d boxes are -0.5..0.5 (examples/ising/in.ising:10),
   3d boxes 0..nz */
static double zlo_of(const spko_cfg *c) { return is2d(c) ? -0.5 : 0.0; }

static int proc_index(const spko_cfg *c, int64_t i) {
  int64_t x = i % c->nx;
  int64_t y = (i / c->nx) % c->ny;
  int64_t z = i / ((int64_t)c->nx * c->ny);
  int px = c->px > 0 ? c->px : 1, py = c->py > 0 ? c->py : 1, pz = c->pz > 0 ? c->pz : 1;
  int ax = proc_of(x, c->nx, px, 0.0);
  int ay = proc_of(y, c->ny, py, 0.0);
  int az = is2d(c) ? 0 : proc_of(z, c->nz, pz, 0.0);
  return ax + px * (ay + py * az);
}

/* sector of a site within its processor sub-domain, AppLattice::create_set
   (src/app_lattice.cpp:972-985), returns 1..nsector */
int spko_sector(const spko_cfg *c, int64_t i) {
  if (c->nsector <= 1) return 1;
  int64_t x = i % c->nx;
  int64_t y = (i / c->nx) % c->ny;
  int64_t z = i / ((int64_t)c->nx * c->ny);
  int px = c->px > 0 ? c->px : 1, py = c->py > 0 ? c->py : 1, pz = c->pz > 0 ? c->pz : 1;
  int ax = proc_of(x, c->nx, px, 0.0);
  int ay = proc_of(y, c->ny, py, 0.0);
  double xmid = mid_of(ax, c->nx, px, 0.0);
  double ymid = mid_of(ay, c->ny, py, 0.0);
  double zmid;
  double zc = (double)z;
  if (is2d(c)) {
    zmid = 0.0; /* box -0.5..0.5 */
  } else {
    int az = proc_of(z, c->nz, pz, 0.0);
    zmid = mid_of(az, c->nz, pz, 0.0);
  }
  int iw = ((double)x < xmid) ? 0 : 1;
  int jw = ((double)y < ymid) ? 0 : 1;
  int kw = (zc < zmid) ? 0 : 1;
  if (c->nsector == 2) return iw + 1;
  if (c->nsector == 4) return 2 * jw + iw + 1;
  return 4 * kw + 2 * jw + iw + 1;
}

/* ---------------------------------------------------------------------- */

void spko_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  spko_philox4x32_10(ctr, key, out);
}

uint64_t spko_hash(const int32_t *spin, int64_t n) {
  uint64_t h = 1469598103934665603ULL;
  for (int64_t i = 0; i < n; i++) {
    uint32_t v = (uint32_t)spin[i];
    for (int b = 0; b < 4; b++) {
      h ^= (v >> (8 * b)) & 0xFFu;
      h *= 1099511628211ULL;
    }
  }
  return h;
}

void spko_init_spins(uint32_t seed, int64_t n, int lo, int hi, int32_t *spin) {
  for (int64_t i = 0; i < n; i++) spin[i] = spko_init_spin(seed, (uint64_t)i, lo, hi);
}

void spko_init_values(uint32_t seed, int64_t n, const int64_t *ids, int lo, int hi, int32_t *out) {
  for (int64_t k = 0; k < n; k++) out[k] = spko_init_spin(seed, (uint64_t)ids[k], lo, hi);
}

static int64_t nsites(const spko_cfg *c) { return (int64_t)c->nx * c->ny * c->nz; }

/* site_energy: count of unlike neighbours
   (src/app_ising.cpp:88-95, src/app_potts.cpp:97-104) */
static double site_energy(const int32_t *spin, int64_t i, const int64_t *nb, int nn) {
  int e = 0;
  for (int j = 0; j < nn; j++)
    if (spin[i] != spin[nb[j]]) e++;
  return (double)e;
}

/* ---------------------------------------------------------------------- */
/* RandomPark / RanMars restatements                                      */
/* ---------------------------------------------------------------------- */

/* RandomPark::uniform, Park-Miller with Schrage (src/random_park.cpp:79-86) */
double spko_park_uniform(int32_t *seed) {
  const int IA = 16807, IM = 2147483647, IQ = 127773, IR = 2836;
  int k = *seed / IQ;
  *seed = IA * (*seed - k * IQ) - IR * k;
  if (*seed < 0) *seed += IM;
  return (1.0 / IM) * (*seed);
}

/* RandomPark(double) (src/random_park.cpp:44-48) */
int32_t spko_park_seed_from_double(double rseed) {
  int s = (int)(rseed * 2147483647);
  if (s == 0) s = 1;
  return s;
}

/* RandomPark::reset / tagreset (src/random_park.cpp:57-75) */
int32_t spko_park_reset(double rseed, int64_t offset, int warmup) {
  int32_t s = (int32_t)fmod(rseed * 2147483647 + (double)offset, 2147483647);
  if (s < 0) s = -s;
  if (s == 0) s = 1;
  for (int i = 0; i < warmup; i++) spko_park_uniform(&s);
  return s;
}

static int park_irandom(int32_t *seed, int n) {
  int i = (int)(spko_park_uniform(seed) * n) + 1;
  if (i > n) i = n;
  return i;
}

/* RanMars::init (src/random_mars.cpp:43-83) */
void spko_ranmars_init(spko_ranmars *r, int seed) {
  int ij, kl, i, j, k, l, ii, jj, m;
  double s, t;
  while (seed > 900000000) seed -= 900000000;
  ij = (seed - 1) / 30082;
  kl = (seed - 1) - 30082 * ij;
  i = (ij / 177) % 177 + 2;
  j = ij % 177 + 2;
  k = (kl / 169) % 178 + 1;
  l = kl % 169;
  for (ii = 1; ii <= 97; ii++) {
    s = 0.0;
    t = 0.5;
    for (jj = 1; jj <= 24; jj++) {
      m = ((i * j) % 179) * k % 179;
      i = j;
      j = k;
      k = m;
      l = (53 * l + 1) % 169;
      if ((l * m) % 64 >= 32) s = s + t;
      t = 0.5 * t;
    }
    r->u[ii] = s;
  }
  r->c = 362436.0 / 16777216.0;
  r->cd = 7654321.0 / 16777216.0;
  r->cm = 16777213.0 / 16777216.0;
  r->i97 = 97;
  r->j97 = 33;
  spko_ranmars_uniform(r);
}

/* RanMars::uniform (src/random_mars.cpp:89-105) */
double spko_ranmars_uniform(spko_ranmars *r) {
  double uni = r->u[r->i97] - r->u[r->j97];
  if (uni < 0.0) uni += 1.0;
  r->u[r->i97] = uni;
  r->i97--;
  if (r->i97 == 0) r->i97 = 97;
  r->j97--;
  if (r->j97 == 0) r->j97 = 97;
  r->c -= r->cd;
  if (r->c < 0.0) r->c += r->cm;
  uni -= r->c;
  if (uni < 0.0) uni += 1.0;
  return uni;
}

/* Set::set_range, loop option on (the default), no region/condition:
   one irandom per site ID in ascending order (src/set.cpp:598-624) */
void spko_set_range(int32_t park_seed, int64_t n, int lo, int hi, int32_t *spin) {
  int range = hi - lo + 1;
  for (int64_t i = 0; i < n; i++) spin[i] = park_irandom(&park_seed, range) - 1 + lo;
}

/* ---------------------------------------------------------------------- */
/* per-site rejection event                                               */
/* ---------------------------------------------------------------------- */

typedef struct {
  int mode;          /* SPKO_RNG_PHILOX / SPKO_RNG_STRICT */
  uint32_t x[2];     /* Philox words of this site update */
  int ising;         /* x[0] is the ising site's one word (both draws) */
  int used;
  int32_t *park;     /* strict: the site's Park-Miller state */
} draw_src;

static double draw_uniform(draw_src *d) {
  if (d->mode == SPKO_RNG_STRICT) return spko_park_uniform(d->park);
  if (d->used >= 2) {
    fprintf(stderr, "oracle: more than two draws in one site update\n");
    abort();
  }
  if (d->ising) {
    double u = d->used == 0 ? spko_ising_u0(d->x[0]) : spko_ising_u1(d->x[0]);
    d->used++;
    return u;
  }
  return spko_u(d->x[d->used++]);
}

/* the Boltzmann test shared by all four apps
   (e.g. src/app_ising.cpp:117-124): returns 1 if the proposal stays */
static int boltzmann_accept(double einitial, double efinal, double temperature, draw_src *d) {
  if (efinal <= einitial) return 1;
  if (temperature == 0.0) return 0;
  double t_inverse = 1.0 / temperature;
  if (draw_uniform(d) > exp((einitial - efinal) * t_inverse)) return 0;
  return 1;
}

/* one site_event_rejection of the configured app:
   ising           src/app_ising.cpp:104-136
   potts           src/app_potts.cpp:112-146
   potts/neighonly src/app_potts_neighonly.cpp:71-117
   potts/neigh     src/app_potts_neigh.cpp:71-116
   nb holds the site's neighbours (AppLattice::neighbor[i]).
   returns 1 if the spin changed */
static int site_event_rejection_nb(const spko_cfg *c, int32_t *spin, int64_t i, const int64_t *nb, int nn,
                                   draw_src *d, uint8_t *mask) {
  int oldstate = spin[i];
  double einitial = site_energy(spin, i, nb, nn);
  int unique[27];
  int nevent = 0;

  if (c->app == SPKO_ISING) {
    if (draw_uniform(d) < 0.5) spin[i] = 1;
    else spin[i] = 2;
  } else if (c->app == SPKO_POTTS) {
    int iran = (int)(c->nspins * draw_uniform(d)) + 1;
    if (iran > c->nspins) iran = c->nspins;
    spin[i] = iran;
  } else {
    for (int j = 0; j < nn; j++) {
      int value = spin[nb[j]];
      if (value == spin[i]) continue;
      int m;
      for (m = 0; m < nevent; m++)
        if (value == unique[m]) break;
      if (m < nevent) continue;
      unique[nevent++] = value;
    }
    if (c->app == SPKO_NEIGHONLY) {
      if (nevent == 0) return 0;
      int iran = (int)(nevent * draw_uniform(d));
      if (iran >= nevent) iran = nevent - 1;
      spin[i] = unique[iran];
    } else {
      int iran = (int)(spko_maxneigh(c->lattice) * draw_uniform(d));
      if (iran >= nevent) return 0;
      spin[i] = unique[iran];
    }
  }
  double efinal = site_energy(spin, i, nb, nn);
  if (!boltzmann_accept(einitial, efinal, c->temperature, d)) spin[i] = oldstate;

  if (mask) {
    if (einitial < 0.5 * nn) mask[i] = 1;
    if (spin[i] != oldstate)
      for (int j = 0; j < nn; j++) mask[nb[j]] = 0;
  }
  return spin[i] != oldstate;
}

static int site_event_rejection(const spko_cfg *c, int32_t *spin, int64_t i, draw_src *d, uint8_t *mask) {
  int64_t nb[26];
  int nn = spko_neighbors(c, i, nb);
  return site_event_rejection_nb(c, spin, i, nb, nn, d, mask);
}

/* the per-site rule of one colour-sweep visit, applied to sites given with
   the values they see (site_event_rejection_nb on a local copy) */
int64_t spko_site_updates(const spko_cfg *c, int64_t n, const int64_t *ids, const int32_t *self,
                          const int32_t *nbv, uint32_t sweep, uint32_t pass, int32_t *out) {
  int nn = spko_maxneigh(c->lattice);
  int64_t nb[26];
  int32_t local[27];
  int64_t changed = 0;
  for (int j = 0; j < nn; j++) nb[j] = j + 1;
  for (int64_t k = 0; k < n; k++) {
    local[0] = self[k];
    for (int j = 0; j < nn; j++) local[j + 1] = nbv[k * nn + j];
    draw_src d;
    d.mode = SPKO_RNG_PHILOX;
    d.used = 0;
    d.ising = 0;
    d.park = NULL;
    if (c->app == SPKO_ISING) {
      d.x[0] = d.x[1] = spko_ising_word(c->seed, c->stream_base, (uint64_t)ids[k], sweep, pass);
      d.ising = 1;
    } else {
      spko_site_draws(c->seed, c->stream_base, (uint64_t)ids[k], sweep, pass, &d.x[0], &d.x[1]);
    }
    changed += site_event_rejection_nb(c, local, 0, nb, nn, &d, NULL);
    out[k] = local[0];
  }
  return changed;
}

void spko_neighbors_many(const spko_cfg *c, int64_t n, const int64_t *ids, int64_t *out) {
  int nn = spko_maxneigh(c->lattice);
  for (int64_t k = 0; k < n; k++) spko_neighbors(c, ids[k], out + k * nn);
}

/* ---------------------------------------------------------------------- */
/* colour sweeps: AppLattice::iterate_rejection (src/app_lattice.cpp:632-711)
   with sweep color / color/strict; sets are colours, or sectors x colours
   with sectors outer (src/app_lattice.cpp:684-690)                       */
/* ---------------------------------------------------------------------- */

/* border sites of a sector set: a site with a neighbour outside its sector
   (AppLattice::find_border_sites, src/app_lattice.cpp:1094-1149); with a
   processor grid a sector is per processor */
static int in_same_set(const spko_cfg *c, int64_t a, int64_t b) {
  return proc_index(c, a) == proc_index(c, b) && spko_sector(c, a) == spko_sector(c, b);
}

int spko_color_sweeps(const spko_cfg *c, int32_t *spin, int64_t sweep0, int nsweeps,
                      int64_t *naccept, int64_t *nattempt, uint64_t *hashes,
                      int32_t *siteseeds, uint8_t *mask) {
  int64_t n = nsites(c);
  int ncol = spko_ncolors(c->lattice);
  int nsec = c->nsector > 1 ? c->nsector : 1;
  int nloop = c->nloop > 0 ? c->nloop : 1;
  int nprocs = (c->px > 0 ? c->px : 1) * (c->py > 0 ? c->py : 1) * (c->pz > 0 ? c->pz : 1);
  int nn = spko_maxneigh(c->lattice);
  if (c->rng == SPKO_RNG_STRICT && !siteseeds) return -1;
  /* the reference's own layout: neighbor[i][j] and one ascending site list
     per (sector, colour, processor) set (AppLattice::create_set) */
  int64_t *nbt = (int64_t *)malloc(sizeof(int64_t) * n * nn);
  int nsets = nsec * ncol * nprocs;
  int64_t *count = (int64_t *)calloc((size_t)nsets + 1, sizeof(int64_t));
  int *setof = (int *)malloc(sizeof(int) * n);
  for (int64_t i = 0; i < n; i++) {
    spko_neighbors(c, i, nbt + i * nn);
    int k = ((spko_sector(c, i) - 1) * ncol + (spko_color(c, i) - 1)) * nprocs + proc_index(c, i);
    setof[i] = k;
    count[k + 1]++;
  }
  for (int k = 0; k < nsets; k++) count[k + 1] += count[k];
  int64_t *lists = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
  int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (nsets + 1));
  memcpy(fill, count, sizeof(int64_t) * (nsets + 1));
  for (int64_t i = 0; i < n; i++) lists[fill[setof[i]]++] = i;
  for (int s = 0; s < nsweeps; s++) {
    uint32_t sweep = (uint32_t)(sweep0 + s);
    for (int isec = 1; isec <= nsec; isec++) {
      /* with a mask, clear it on the border sites of the set about to be
         swept (AppLattice::boundary_clear_mask, src/app_lattice.cpp:1157) */
      if (mask && nsec > 1) {
        for (int64_t i = 0; i < n; i++) {
          if (spko_sector(c, i) != isec) continue;
          for (int j = 0; j < nn; j++)
            if (!in_same_set(c, i, nbt[i * nn + j])) {
              mask[i] = 0;
              break;
            }
        }
      }
      for (int icol = 1; icol <= ncol; icol++) {
        int64_t setsize = 0;
        for (int proc = 0; proc < nprocs; proc++) {
          int k = ((isec - 1) * ncol + (icol - 1)) * nprocs + proc;
          setsize += count[k + 1] - count[k];
          /* colour sets: every site borders another set */
          if (mask && nsec == 1)
            for (int64_t m = count[k]; m < count[k + 1]; m++) mask[lists[m]] = 0;
        }
        for (int p = 0; p < nloop; p++) {
          for (int proc = 0; proc < nprocs; proc++) {
            int k = ((isec - 1) * ncol + (icol - 1)) * nprocs + proc;
            for (int64_t m = count[k]; m < count[k + 1]; m++) {
              int64_t i = lists[m];
              if (mask && mask[i]) continue;
              draw_src d;
              d.mode = c->rng;
              d.used = 0;
              d.ising = 0;
              d.park = siteseeds ? &siteseeds[i] : NULL;
              if (c->rng == SPKO_RNG_PHILOX && c->app == SPKO_ISING) {
                d.x[0] = d.x[1] = spko_ising_word(c->seed, c->stream_base, (uint64_t)i, sweep, (uint32_t)p);
                d.ising = 1;
              } else if (c->rng == SPKO_RNG_PHILOX) {
                spko_site_draws(c->seed, c->stream_base, (uint64_t)i, sweep, (uint32_t)p, &d.x[0],
                                &d.x[1]);
              }
              *naccept += site_event_rejection_nb(c, spin, i, nbt + i * nn, nn, &d, mask);
            }
          }
        }
        /* nattempt counts every site of the set, masked or not
           (src/app_lattice.cpp:690) */
        *nattempt += setsize * nloop;
      }
    }
    if (hashes) hashes[s] = spko_hash(spin, n);
  }
  free(nbt);
  free(count);
  free(setof);
  free(lists);
  free(fill);
  return 0;
}

/* ---------------------------------------------------------------------- */
/* sweep random with sectors: iterate_rejection RANDOM branch
   (src/app_lattice.cpp:662-670); nselect = (int)(nstop*nlocal) per sector
   (src/app_lattice.cpp:389-394)                                          */
/* ---------------------------------------------------------------------- */

int spko_random_sector_sweeps(const spko_cfg *c, int32_t *spin, int32_t *ranapp, int nsweeps,
                              int64_t *naccept, int64_t *nattempt) {
  int64_t n = nsites(c);
  int nsec = c->nsector > 1 ? c->nsector : 1;
  int64_t *lists[8];
  int64_t counts[8];
  for (int s = 0; s < nsec; s++) {
    counts[s] = 0;
    lists[s] = (int64_t *)malloc(sizeof(int64_t) * n);
  }
  for (int64_t i = 0; i < n; i++) {
    int s = spko_sector(c, i) - 1;
    lists[s][counts[s]++] = i;
  }
  int64_t *sitelist = (int64_t *)malloc(sizeof(int64_t) * n);
  for (int sw = 0; sw < nsweeps; sw++) {
    for (int s = 0; s < nsec; s++) {
      int nrange = (int)counts[s];
      int nselect = (int)(1.0 * nrange);
      for (int k = 0; k < nselect; k++) sitelist[k] = lists[s][park_irandom(ranapp, nrange) - 1];
      for (int k = 0; k < nselect; k++) {
        draw_src d;
        d.mode = SPKO_RNG_STRICT;
        d.used = 0;
        d.ising = 0;
        d.park = ranapp;
        *naccept += site_event_rejection(c, spin, sitelist[k], &d, NULL);
      }
      *nattempt += nselect;
    }
  }
  for (int s = 0; s < nsec; s++) free(lists[s]);
  free(sitelist);
  return 0;
}

double spko_energy(const spko_cfg *c, const int32_t *spin) {
  int64_t n = nsites(c);
  double e = 0.0;
  int64_t nb[26];
  for (int64_t i = 0; i < n; i++) {
    int nn = spko_neighbors(c, i, nb);
    e += site_energy(spin, i, nb, nn);
  }
  return e;
}

/* Cluster analysis of `diag_style cluster` on one process: sites are taken
   in index order, each unvisited site starts a cluster that grows through
   equal-valued neighbours (DiagCluster::generate_clusters,
   src/diag_cluster.cpp:229-360; AppLattice::push_connected_neighbors,
   src/app_lattice.cpp:1187-1201); with periodic wrap the pieces the
   reference joins across the boundary (src/diag_cluster.cpp:480-597) are
   one component here.  Volumes and volume^(1/dim) are summed in cluster
   order, as the reference does (src/diag_cluster.cpp:597-605). */
int spko_clusters(const spko_cfg *c, const int32_t *spin, int64_t *ncluster, double *vav, double *rav) {
  int64_t n = nsites(c);
  int32_t *seen = (int32_t *)calloc((size_t)n, sizeof(int32_t));
  int64_t *stack = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  if (!seen || !stack) {
    free(seen);
    free(stack);
    return -1;
  }
  int dim = is2d(c) ? 2 : 3;
  double invdim = 1.0 / dim;
  double volsum = 0.0, rsum = 0.0;
  int64_t nc = 0;
  int64_t nb[26];
  for (int64_t i = 0; i < n; i++) {
    if (seen[i]) continue;
    nc++;
    int64_t top = 0;
    stack[top++] = i;
    seen[i] = 1;
    double vol = 0.0;
    while (top > 0) {
      int64_t ii = stack[--top];
      vol += 1.0;
      int nn = spko_neighbors(c, ii, nb);
      for (int j = 0; j < nn; j++) {
        int64_t m = nb[j];
        if (spin[m] == spin[ii] && !seen[m]) {
          seen[m] = 1;
          stack[top++] = m;
        }
      }
    }
    volsum += vol;
    rsum += pow(vol, invdim);
  }
  free(seen);
  free(stack);
  *ncluster = nc;
  *vav = nc ? volsum / (double)nc : 0.0;
  *rav = nc ? rsum / (double)nc : 0.0;
  return 0;
}

/* ---------------------------------------------------------------------- */
/* KMC with the tree solver over sectors                                  */
/* ---------------------------------------------------------------------- */

/* SolveTree state (src/solve_tree.cpp:70-224) */
typedef struct {
  int nevents;
  int offset;
  int ntotal;
  double *tree;
  double sum;
  int num_active;
  uint64_t nevent_drawn;
} tree_t;

static void tree_init(tree_t *t, int n, const double *prop) {
  t->nevents = n;
  int nround = 1;
  while (nround < n) nround *= 2;
  t->offset = nround - 1;
  t->ntotal = 2 * nround - 1;
  free(t->tree);
  t->tree = (double *)calloc((size_t)t->ntotal, sizeof(double));
  for (int i = 0; i < n; i++) t->tree[t->offset + i] = prop[i];
  for (int parent = t->offset - 1; parent >= 0; parent--)
    t->tree[parent] = t->tree[2 * parent + 1] + t->tree[2 * parent + 2];
  t->sum = t->tree[0];
  t->num_active = 0;
  for (int i = t->offset; i < t->ntotal; i++)
    if (t->tree[i] > 0.0) t->num_active++;
}

static void tree_set(tree_t *t, int i, double value) {
  if (t->tree[t->offset + i] > 0.0) t->num_active--;
  if (value > 0.0) t->num_active++;
  t->tree[t->offset + i] = value;
  i += t->offset;
  while (i > 0) {
    int sibling = (i % 2) ? i + 1 : i - 1;
    int parent = (i - 1) / 2;
    t->tree[parent] = t->tree[i] + t->tree[sibling];
    i = parent;
  }
  t->sum = t->tree[0];
}

static int tree_find(const tree_t *t, double value) {
  int i = 0;
  while (i < t->offset) {
    int left = 2 * i + 1;
    if (value <= t->tree[left]) i = left;
    else {
      value -= t->tree[left];
      i = left + 1;
    }
  }
  return i - t->offset;
}

typedef struct {
  int nlocal;
  int64_t *site2i;
  int64_t nborder;
  int64_t *border;
  double *propensity;
  tree_t tree;
} kset_t;

struct spko_kmc {
  spko_cfg cfg;
  int64_t n;
  int nsets;          /* nprocs * nsector chains */
  kset_t *sets;
  int *i2site;        /* per site: index within its own set */
  int *i2set;         /* per site: its set */
  int ladapt;
  double nstop, tstop;
  double dt_kmc;
  int first_run;
};

/* AppIsing::site_propensity (src/app_ising.cpp:143-163) and
   AppPotts::site_propensity (src/app_potts.cpp:153-189) */
static double site_propensity(const spko_cfg *c, int32_t *spin, int64_t i) {
  int64_t nb[26];
  int nn = spko_neighbors(c, i, nb);
  double t_inverse = c->temperature != 0.0 ? 1.0 / c->temperature : 0.0;
  if (c->app == SPKO_ISING) {
    int oldstate = spin[i];
    int newstate = (oldstate == 1) ? 2 : 1;
    double einitial = site_energy(spin, i, nb, nn);
    spin[i] = newstate;
    double efinal = site_energy(spin, i, nb, nn);
    spin[i] = oldstate;
    if (efinal <= einitial) return 1.0;
    if (c->temperature == 0.0) return 0.0;
    return exp((einitial - efinal) * t_inverse);
  }
  int unique[27];
  int nevent = 0;
  for (int j = 0; j < nn; j++) {
    int value = spin[nb[j]];
    if (value == spin[i]) continue;
    int m;
    for (m = 0; m < nevent; m++)
      if (value == unique[m]) break;
    if (m < nevent) continue;
    unique[nevent++] = value;
  }
  int oldstate = spin[i];
  double einitial = site_energy(spin, i, nb, nn);
  double prob = 0.0;
  for (int m = 0; m < nevent; m++) {
    spin[i] = unique[m];
    double efinal = site_energy(spin, i, nb, nn);
    if (efinal <= einitial) prob += 1.0;
    else if (c->temperature > 0.0) prob += exp((einitial - efinal) * t_inverse);
  }
  spin[i] = oldstate;
  return prob;
}

/* site_event + propensity refresh of self and in-set neighbours
   (src/app_ising.cpp:170-196, src/app_potts.cpp:196-244) */
static void site_event(spko_kmc *k, int32_t *spin, int64_t i, double uthresh) {
  const spko_cfg *c = &k->cfg;
  kset_t *set = &k->sets[k->i2set[i]];
  int64_t nb[26];
  int nn = spko_neighbors(c, i, nb);
  double t_inverse = c->temperature != 0.0 ? 1.0 / c->temperature : 0.0;
  if (c->app == SPKO_ISING) {
    spin[i] = (spin[i] == 1) ? 2 : 1;
  } else {
    double threshhold = uthresh * set->propensity[k->i2site[i]];
    int oldstate = spin[i];
    double einitial = site_energy(spin, i, nb, nn);
    double prob = 0.0;
    int unique[27];
    int nevent = 0;
    for (int j = 0; j < nn; j++) {
      int value = spin[nb[j]];
      if (value == oldstate) continue;
      int m;
      for (m = 0; m < nevent; m++)
        if (value == unique[m]) break;
      if (m < nevent) continue;
      unique[nevent++] = value;
      spin[i] = value;
      double efinal = site_energy(spin, i, nb, nn);
      if (efinal <= einitial) prob += 1.0;
      else if (c->temperature > 0.0) prob += exp((einitial - efinal) * t_inverse);
      if (prob >= threshhold) break;
    }
  }
  int myset = k->i2set[i];
  int isite = k->i2site[i];
  set->propensity[isite] = site_propensity(c, spin, i);
  tree_set(&set->tree, isite, set->propensity[isite]);
  for (int j = 0; j < nn; j++) {
    int64_t m = nb[j];
    if (k->i2set[m] != myset) continue;
    int is = k->i2site[m];
    set->propensity[is] = site_propensity(c, spin, m);
    tree_set(&set->tree, is, set->propensity[is]);
  }
}

spko_kmc *spko_kmc_create(const spko_cfg *c, int nstop_mode, double nstop, double tstop) {
  spko_kmc *k = (spko_kmc *)calloc(1, sizeof(spko_kmc));
  k->cfg = *c;
  k->n = nsites(c);
  int nprocs = (c->px > 0 ? c->px : 1) * (c->py > 0 ? c->py : 1) * (c->pz > 0 ? c->pz : 1);
  int nsec = c->nsector > 1 ? c->nsector : 1;
  k->nsets = nprocs * nsec;
  k->sets = (kset_t *)calloc((size_t)k->nsets, sizeof(kset_t));
  k->i2site = (int *)malloc(sizeof(int) * k->n);
  k->i2set = (int *)malloc(sizeof(int) * k->n);
  for (int64_t i = 0; i < k->n; i++) {
    int s = proc_index(c, i) * nsec + (spko_sector(c, i) - 1);
    k->i2set[i] = s;
    k->i2site[i] = k->sets[s].nlocal++;
  }
  for (int s = 0; s < k->nsets; s++) {
    k->sets[s].site2i = (int64_t *)malloc(sizeof(int64_t) * (k->sets[s].nlocal + 1));
    k->sets[s].propensity = (double *)calloc((size_t)k->sets[s].nlocal + 1, sizeof(double));
    k->sets[s].border = (int64_t *)malloc(sizeof(int64_t) * (k->sets[s].nlocal + 1));
  }
  for (int64_t i = 0; i < k->n; i++) {
    kset_t *st = &k->sets[k->i2set[i]];
    st->site2i[k->i2site[i]] = i;
  }
  for (int s = 0; s < k->nsets; s++) {
    kset_t *st = &k->sets[s];
    for (int m = 0; m < st->nlocal; m++) {
      int64_t i = st->site2i[m];
      int64_t nb[26];
      int nn = spko_neighbors(c, i, nb);
      for (int j = 0; j < nn; j++)
        if (k->i2set[nb[j]] != s) {
          st->border[st->nborder++] = i;
          break;
        }
    }
  }
  k->ladapt = (nstop_mode != 0);
  k->nstop = nstop;
  k->tstop = tstop;
  k->first_run = 1;
  return k;
}

void spko_kmc_destroy(spko_kmc *k) {
  if (!k) return;
  for (int s = 0; s < k->nsets; s++) {
    free(k->sets[s].site2i);
    free(k->sets[s].propensity);
    free(k->sets[s].border);
    free(k->sets[s].tree.tree);
  }
  free(k->sets);
  free(k->i2site);
  free(k->i2set);
  free(k);
}

/* AppLattice::setup KMC part (src/app_lattice.cpp:340-377) followed by
   iterate_kmc_sector (src/app_lattice.cpp:517-626).  With a processor
   grid, sector iset of every processor runs in the same phase; their
   chains touch disjoint sites, so running them one after another equals
   running them concurrently. */
int spko_kmc_run(spko_kmc *k, int32_t *spin, double *ptime, double stoptime, int64_t *naccept,
                 uint64_t *hashes, double *pass_times, int maxrec) {
  const spko_cfg *c = &k->cfg;
  int nsec = c->nsector > 1 ? c->nsector : 1;
  int nprocs = k->nsets / nsec;
  double time = *ptime;
  for (int s = 0; s < k->nsets; s++) {
    kset_t *st = &k->sets[s];
    for (int m = 0; m < st->nlocal; m++) st->propensity[m] = site_propensity(c, spin, st->site2i[m]);
    tree_init(&st->tree, st->nlocal, st->propensity);
  }
  if (k->tstop > 0.0) k->dt_kmc = k->tstop;
  if (k->ladapt) {
    double pmax = 0.0;
    for (int s = 0; s < k->nsets; s++) {
      int ntmp = k->sets[s].tree.num_active;
      if (ntmp > 0) {
        double ptmp = k->sets[s].tree.sum / ntmp;
        pmax = pmax > ptmp ? pmax : ptmp;
      }
    }
    if (pmax > 0.0) k->dt_kmc = k->nstop / pmax;
    else k->dt_kmc = stoptime - time;
  }
  if (k->dt_kmc > stoptime - time) k->dt_kmc = stoptime - time;

  int npass = 0;
  if (!(stoptime > time)) {
    *ptime = time;
    return 0;
  }
  int alldone = 0;
  while (!alldone) {
    double pmax = 0.0;
    for (int iset = 0; iset < nsec; iset++) {
      for (int proc = 0; proc < nprocs; proc++) {
        int s = proc * nsec + iset;
        kset_t *st = &k->sets[s];
        for (int64_t b = 0; b < st->nborder; b++) {
          int64_t i = st->border[b];
          int isite = k->i2site[i];
          st->propensity[isite] = site_propensity(c, spin, i);
          tree_set(&st->tree, isite, st->propensity[isite]);
        }
        if (k->ladapt) {
          int ntmp = st->tree.num_active;
          if (ntmp > 0) {
            double ptmp = st->tree.sum / ntmp;
            pmax = pmax > ptmp ? pmax : ptmp;
          }
        }
        int done = 0;
        double timesector = 0.0;
        while (!done) {
          if (st->tree.sum == 0.0) {
            done = 1;
            break;
          }
          uint32_t w[4];
          spko_kmc_draws(c->seed, (uint32_t)s, st->tree.nevent_drawn, w);
          st->tree.nevent_drawn++;
          double r2 = spko_u(w[0]);
          int m = tree_find(&st->tree, r2 * st->tree.sum);
          double dt = -1.0 / st->tree.sum * log(spko_u(w[1]));
          timesector += dt;
          if (timesector >= k->dt_kmc) done = 1;
          else {
            site_event(k, spin, st->site2i[m], spko_u(w[2]));
            (*naccept)++;
          }
        }
      }
    }
    if (hashes && npass < maxrec) hashes[npass] = spko_hash(spin, k->n);
    npass++;
    time += k->dt_kmc;
    if (pass_times && npass - 1 < maxrec) pass_times[npass - 1] = time;
    if (time >= stoptime) alldone = 1;
    if (k->ladapt) {
      if (pmax > 0.0) k->dt_kmc = k->nstop / pmax;
      else k->dt_kmc = stoptime - time;
      if (k->dt_kmc > stoptime - time) k->dt_kmc = stoptime - time;
    }
  }
  *ptime = time;
  return npass;
}

double spko_kmc_total_propensity(spko_kmc *k) {
  double s = 0.0;
  for (int i = 0; i < k->nsets; i++) s += k->sets[i].tree.sum;
  return s;
}

int spko_kmc_nchains(spko_kmc *k) { return k->nsets; }

uint64_t spko_kmc_chain_events(spko_kmc *k, int chain) {
  return k->sets[chain].tree.nevent_drawn;
}
