/* spkgpu: GB300-native (sm_103a) on-lattice Monte Carlo hot path of SPPARKS.

   A plain C ABI (pointers, sizes, status codes) over hand-written CUDA
   kernels.  It replaces, for one lattice on one GPU, the per-site virtual
   calls that AppLattice makes on the host:

     spkgpu_sweep        AppLattice::iterate_rejection with `sweep color` or
                         `sweep color/strict` (src/app_lattice.cpp:632-711)
                         calling AppIsing/AppPotts/AppPottsNeighOnly/
                         AppPottsNeigh::site_event_rejection
                         (src/app_ising.cpp:104-136, src/app_potts.cpp:112-146,
                         src/app_potts_neighonly.cpp:71-117,
                         src/app_potts_neigh.cpp:71-116)
     spkgpu_kmc_run      AppLattice::iterate_kmc_sector with `solve_style tree`
                         (src/app_lattice.cpp:517-626, src/solve_tree.cpp:109-224,
                         src/app_potts.cpp:153-244, src/app_ising.cpp:143-196)
     spkgpu_energy       spparks_energy / DiagEnergy (src/library.cpp:118-147,
                         src/diag_energy.cpp:53-68)
     spkgpu_upload_spins / spkgpu_download_spins
                         the host<->device sync of App::iarray[0] that a host
                         AppLattice subclass performs around iterate()
                         (src/app.cpp:179-182)

   Every entry point returns 0 on success or a negative SPKGPU_ERR_* code and
   never exits the process; spkgpu_last_error() returns the message of the
   last failure on a handle.  A handle owns one CUDA stream; calls on one
   handle must come from one host thread at a time.

   Random numbers: Philox4x32-10 keyed by (seed, stream) with counter
   (site quad for ising, site pair for the other apps; sweep, pass), as stated
   in spparks_gb300/csrc/spk_philox.cuh.  With
   SPKGPU_RNG_STRICT each site carries the reference's own Park-Miller state
   (sweep color/strict, src/app_lattice.cpp:287-295, 796-805) instead. */
#ifndef SPKGPU_H
#define SPKGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPKGPU_OK 0
#define SPKGPU_ERR_ARG (-1)         /* invalid argument or configuration */
#define SPKGPU_ERR_CUDA (-2)        /* a CUDA runtime call failed */
#define SPKGPU_ERR_STATE (-3)       /* call not valid in the handle's state */
#define SPKGPU_ERR_NOMEM (-4)       /* device allocation failed */
#define SPKGPU_ERR_UNSUPPORTED (-5) /* combination not implemented */
#define SPKGPU_ERR_INVALID_SPIN (-6) /* a site value is outside 1..nspins */
#define SPKGPU_ERR_DEVICE (-7)      /* a device-side wait gave up (error flag set) */
#define SPKGPU_ERR_TOO_LARGE (-8)   /* lattice exceeds SPKGPU_NOALLOC_MAX_BYTES */

/* lattice styles (src/lattice.cpp:43-57); periodic boxes only */
#define SPKGPU_SQ_4N 0
#define SPKGPU_SQ_8N 1
#define SPKGPU_SC_6N 2
#define SPKGPU_SC_26N 3

/* app styles (AppStyle names in src/app_*.h) */
#define SPKGPU_ISING 0
#define SPKGPU_POTTS 1
#define SPKGPU_POTTS_NEIGHONLY 2
#define SPKGPU_POTTS_NEIGH 3

#define SPKGPU_RNG_PHILOX 0
#define SPKGPU_RNG_STRICT 1

typedef struct spkgpu_lattice spkgpu_lattice;

typedef struct spkgpu_desc {
  int32_t lattice;      /* SPKGPU_SQ_4N ... */
  int32_t nx, ny, nz;   /* sites per axis; nz = 1 for 2d styles */
  int32_t app;          /* SPKGPU_ISING ... */
  int32_t nspins;       /* Q (2 for Ising); must be < 2^21 */
  int32_t spin_bytes;   /* device storage per site: 1, 2, 4, 0 = smallest
                           that holds nspins, or -1 = bit-packed, 64 sites per
                           uint64 (Ising on sc/6n, nx a multiple of 64, no
                           sectors, mask or strict RNG) */
  int32_t nsector;      /* 1 = no sectors, else 2, 4, 8 (`sector`) */
  int32_t nloop;        /* passes over each set per sweep (`sector nstop`) */
  int32_t procs[3];     /* processor grid (`processors`), 1 1 1 = serial */
  int32_t rng;          /* SPKGPU_RNG_PHILOX or SPKGPU_RNG_STRICT */
  int32_t mask;         /* 1 = `sweep ... mask yes` */
  uint32_t seed;        /* Philox key word */
  int32_t device;       /* CUDA device ordinal */
  int32_t variant;      /* 0 = fastest kernel for the configuration,
                           1 = always the per-colour phase kernel,
                           2 = the tile kernel (one launch per sweep) even
                               where the whole lattice fits one CTA */
} spkgpu_desc;

typedef struct spkgpu_stats {
  int64_t naccept;      /* site values changed (src/app_ising.cpp:124) */
  int64_t nattempt;     /* site updates attempted */
  int64_t nsweeps;      /* sweeps done on this handle */
} spkgpu_stats;

/* lifecycle ------------------------------------------------------------ */
int spkgpu_create(const spkgpu_desc *desc, spkgpu_lattice **out);
int spkgpu_destroy(spkgpu_lattice *h);
const char *spkgpu_last_error(const spkgpu_lattice *h);
int spkgpu_version(void);

/* `temperature T` (AppLattice::set_temperature, src/app_lattice.cpp:893-898) */
int spkgpu_set_temperature(spkgpu_lattice *h, double temperature);

/* site values in App::iarray[0] order (site index = id - 1) */
int spkgpu_upload_spins(spkgpu_lattice *h, const int32_t *spin, int64_t n);
int spkgpu_download_spins(spkgpu_lattice *h, int32_t *spin, int64_t n);
/* fill the lattice on the device with seeded values uniform in lo..hi:
   site s (= id-1) gets lo + ((hi-lo+1) * x) >> 32 for the Philox word x of
   stream 3, counter (s>>1, s>>33, 0, 0), word 2*(s&1) - the role of
   `set site range lo hi` (src/set.cpp:582-760) without a host array */
int spkgpu_init_spins(spkgpu_lattice *h, int32_t lo, int32_t hi);
/* per-site Park-Miller states for SPKGPU_RNG_STRICT (AppLattice::siteseeds) */
int spkgpu_upload_siteseeds(spkgpu_lattice *h, const int32_t *seeds, int64_t n);
int spkgpu_download_siteseeds(spkgpu_lattice *h, int32_t *seeds, int64_t n);
/* mask bytes for `sweep ... mask yes` (AppLattice::mask) */
int spkgpu_upload_mask(spkgpu_lattice *h, const uint8_t *mask, int64_t n);
int spkgpu_download_mask(spkgpu_lattice *h, uint8_t *mask, int64_t n);

/* rejection sweeps --------------------------------------------------------
   Enqueues nsweeps sweeps on the handle's stream and returns; the sweep
   index (Philox counter word) continues from the previous call. */
int spkgpu_sweep(spkgpu_lattice *h, int32_t nsweeps);
int spkgpu_set_sweep_index(spkgpu_lattice *h, int64_t sweep);
/* waits for the stream, then reports the counters */
int spkgpu_get_stats(spkgpu_lattice *h, spkgpu_stats *out);
/* total energy = sum of site energies (waits for the stream) */
int spkgpu_energy(spkgpu_lattice *h, double *energy);
/* sum, minimum and maximum of the site values (vmin, vmax may be NULL):
   `diag_style array i1 mean|sum|min|max` (src/diag_array.cpp:107-200; mean
   = sum / nsites); the Ising magnetisation is 2 * mean - 3 */
int spkgpu_site_stats(spkgpu_lattice *h, int64_t *sum, int32_t *vmin, int32_t *vmax);
/* `diag_style cluster` (src/diag_cluster.cpp:229-609): connected components
   of equal site values over the lattice neighbours with periodic wrap;
   ncluster = Nclust, mean_volume = <N>, mean_radius = <R> (mean of
   volume^(1/dimension)).  At most 2^31-1 sites; allocates 8 bytes per site
   of scratch on first use, kept until spkgpu_destroy. */
int spkgpu_clusters(spkgpu_lattice *h, int64_t *ncluster, double *mean_volume, double *mean_radius);
int spkgpu_synchronize(spkgpu_lattice *h);
/* enqueue nsweeps sweeps bracketed by CUDA events on the handle's stream,
   wait, and report the elapsed device time in milliseconds */
int spkgpu_timed_sweeps(spkgpu_lattice *h, int32_t nsweeps, float *ms);
/* the handle's stream (cudaStream_t) and device spin buffer, for callers
   that keep their own data resident on the device */
int spkgpu_stream(spkgpu_lattice *h, void **stream);
int spkgpu_device_spins(spkgpu_lattice *h, void **dptr, int64_t *bytes);
/* number of kernel launches this handle has issued */
int spkgpu_launch_count(const spkgpu_lattice *h, int64_t *count);

/* rejection-free KMC with the tree solver over sectors --------------------
   adapt = 1: `sector ... nstop N` (dt_kmc = N / max per-site propensity),
   adapt = 0: `sector ... tstop dt`.  fp64 = 1 computes propensities in FP64
   (bit-exact mode); 0 and 2 in FP32, with tree sums, roots and the clock in
   FP64 always.  fp64 = 0 also keeps an all-FP64 shadow of every pass's
   per-chain propensity sums (one extra propensity evaluation per site and
   pass) and reports its errors in the run's stats; fp64 = 2 runs without it.
   spkgpu_kmc_run performs one `run` from *time to stoptime. */
typedef struct spkgpu_kmc_stats {
  double time;          /* simulated time reached */
  int64_t naccept;      /* events executed (cumulative) */
  int64_t npass;        /* passes over all sectors (cumulative) */
  double dt_kmc;        /* current sector time increment */
  double total_propensity; /* sum of all tree roots after the run */
  double prop_rel_err;  /* fp64 = 0: relative error of the final lattice's total propensity
                           from FP32 site propensities against all-FP64 (else 0) */
  double dt_rel_err;    /* fp64 = 0: max relative error of the run's adaptive time steps
                           nstop/pmax against all-FP64 propensities (else 0) */
} spkgpu_kmc_stats;
int spkgpu_kmc_setup(spkgpu_lattice *h, int32_t adapt, double nstop, double tstop, int32_t fp64);
int spkgpu_kmc_run(spkgpu_lattice *h, double *time, double stoptime, spkgpu_kmc_stats *out);
/* the same run in pieces, for output during it: first = 1 starts a run (the
   setup spkgpu_kmc_run does), first = 0 continues the current one; passes
   stop once *time reaches stoptime (which alone bounds the time steps, as
   the run's end does in the reference) or, earlier, once a pass ends at or
   after `until` (the next output time).  Runs equal spkgpu_kmc_run's for
   any sequence of `until` values. */
int spkgpu_kmc_run_until(spkgpu_lattice *h, double *time, double stoptime, double until, int32_t first,
                         spkgpu_kmc_stats *out);

/* integer-issue ceiling ------------------------------------------------------
   No counterpart in the reference.  Philox4x32-10 blocks per second that
   device computes with the sweep kernels' own Philox code and nothing else
   (iters blocks x 4 per thread, 8 CTAs of 128 threads per SM); an ising
   sweep spends one block per four sites and the other apps one per x-pair,
   so 4 x (ising) or 2 x (the others) this rate bounds every sweep of the
   Philox draw contract. */
int spkgpu_philox_rate(int32_t device, int32_t iters, double *blocks_per_s);

/* sweeping without allocating ----------------------------------------------
   No counterpart in the reference.  For callers that cannot allocate device
   memory themselves or through this library: those that own all of it via
   their own pool (e.g. a framework's caching allocator), or that must not
   incur the device-wide synchronisation cudaMalloc/cudaFree can cause while
   their other streams run.  Runs nsweeps fused sq/4n colour sweeps (the same
   update and draws as spkgpu_sweep on an sq/4n lattice without sectors) on a
   lattice the caller keeps in device memory: `spin` holds nx*ny values of
   spin_bytes each (1, 2 or 4; row-major, site index = id-1) and is updated in
   place; nx and ny must be multiples of 32 and `spin` 8-byte aligned (as
   every cudaMalloc pointer is).  Sweep k uses Philox sweep index
   sweep0+k.  The second sweep buffer and the change counter come from one
   static device array of SPKGPU_NOALLOC_MAX_BYTES (+2048) bytes that every
   GPU loading the library holds until exit; larger lattices return
   SPKGPU_ERR_TOO_LARGE.  The array is shared by all calls and keeps the last
   call's contents, so calls whose GPU work overlaps race: serialise them.
   The first call on a device looks up the array's device address
   (cudaGetSymbolAddress) and should precede any stream capture; it is
   looked up again when the device's context changes (cudaDeviceReset).  Work
   goes on `stream` (a cudaStream_t, NULL = default stream); if naccept is not
   NULL the call waits for the stream and stores the number of changed site
   values there, otherwise it returns without waiting.  Inside a stream
   capture naccept must be NULL (SPKGPU_ERR_ARG otherwise, with nothing
   enqueued).  It allocates nothing. */
#define SPKGPU_NOALLOC_MAX_BYTES (4u << 20)
int spkgpu_sweep_sq4_noalloc(void *spin, int32_t nx, int32_t ny, int32_t spin_bytes, int32_t app,
                             int32_t nspins, double temperature, uint32_t seed, int64_t sweep0,
                             int32_t nsweeps, void *stream, int64_t *naccept);

/* batched ensemble of independent sq/4n lattices ---------------------------
   Many replicas of uneven size L x L (L a multiple of 32) and their own
   temperatures swept together, with parallel-tempering replica exchange
   between neighbouring temperatures of equal-L replicas every exchange_every
   sweeps, on the device.  Two execution forms give identical results: one
   persistent cooperative kernel per step (sweeps separated by a bounded grid
   barrier), or one launch per sweep over every tile of every replica with
   the exchange as separate launches; create times one captured step of each
   on the replica set and keeps the fastest (SPKGPU_ENSEMBLE_MODE=persistent,
   launches, launches2, launches4, warps, warps2 or warps4 in the environment forces one).  Each replica
   follows the same per-site rule as a single `sweep color` lattice (same as
   spkgpu_sweep with sq/4n); replica r draws from Philox stream (r+1) << 8.
   The reference has no ensemble; it corresponds to running one reference
   instance per replica (src/app_lattice.cpp:632-711).  Site values of
   replica r occupy L_r*L_r consecutive int32 entries, replicas in order. */
typedef struct spkgpu_ensemble spkgpu_ensemble;
typedef struct spkgpu_ensemble_desc {
  int32_t nreplica;
  const int32_t *L;           /* per-replica edge, multiple of 32 */
  const double *temperature;  /* per-replica initial temperature (> 0) */
  int32_t app;                /* SPKGPU_ISING or SPKGPU_POTTS (nspins <= 127) */
  int32_t nspins;
  uint32_t seed;
  int32_t exchange_every;     /* sweeps between exchange rounds, 0 = never */
  int32_t device;
} spkgpu_ensemble_desc;
typedef struct spkgpu_ensemble_stats {
  int64_t naccept;            /* site values changed, all replicas */
  int64_t nattempt;
  int64_t nsweeps;
  int64_t exchange_tries;
  int64_t exchange_accepts;
} spkgpu_ensemble_stats;
int spkgpu_ensemble_create(const spkgpu_ensemble_desc *desc, spkgpu_ensemble **out);
int spkgpu_ensemble_destroy(spkgpu_ensemble *e);
const char *spkgpu_ensemble_last_error(const spkgpu_ensemble *e);
int spkgpu_ensemble_upload(spkgpu_ensemble *e, const int32_t *spin, int64_t n);
int spkgpu_ensemble_download(spkgpu_ensemble *e, int32_t *spin, int64_t n);
/* enqueue nsweeps sweeps; whole exchange periods run as replays of a
   captured CUDA graph of one step */
int spkgpu_ensemble_run(spkgpu_ensemble *e, int32_t nsweeps);
int spkgpu_ensemble_timed_run(spkgpu_ensemble *e, int32_t nsweeps, float *ms);
/* Pipelined host I/O: enqueue one step that loads every site value from
   `in` (host, int32, replicas in order), runs nsweeps sweeps and stores the
   result into `out` (host, int32), and return at once.  With page-locked
   buffers (cudaHostAlloc or cudaHostRegister) the copy engines move a call's
   input while the previous call's sweeps run and its result while the next
   call's sweeps run (four int32 device staging buffers of every site, two
   per direction used by alternate calls, are allocated on the first call).  Both buffers must stay untouched until
   spkgpu_ensemble_synchronize returns; that call reports invalid input values
   (SPKGPU_ERR_INVALID_SPIN), found after the sweeps have run on them.
   Pageable buffers take upload, run and download in turn (synchronous). */
int spkgpu_ensemble_run_io(spkgpu_ensemble *e, const int32_t *in, int32_t *out, int32_t nsweeps);
int spkgpu_ensemble_synchronize(spkgpu_ensemble *e);
int spkgpu_ensemble_get_stats(spkgpu_ensemble *e, spkgpu_ensemble_stats *out);
/* current temperature of each replica and energy (unlike-neighbour bonds,
   each counted once) measured at the last exchange round */
int spkgpu_ensemble_temperatures(spkgpu_ensemble *e, double *temperature);
int spkgpu_ensemble_energies(spkgpu_ensemble *e, int64_t *bonds);
int spkgpu_ensemble_launch_count(const spkgpu_ensemble *e, int64_t *count);
/* execution form in use and the autotuner's time of one step in each form
   (tune_ms[SPKGPU_ENSEMBLE_NMODES], ms; -1 where not timed); tune_ms may be
   NULL.  The per-sweep forms sweep 1, 2 or 4 consecutive tiles per CTA of
   64 threads, or (warps, warps2, warps4; Ising only) one warp per tile, the
   two warps of a CTA on two tiles of one replica, each warp sweeping 1, 2 or
   4 tiles per launch one after another. */
#define SPKGPU_ENSEMBLE_PERSISTENT 0
#define SPKGPU_ENSEMBLE_LAUNCHES 1
#define SPKGPU_ENSEMBLE_LAUNCHES2 2
#define SPKGPU_ENSEMBLE_LAUNCHES4 3
#define SPKGPU_ENSEMBLE_WARPS 4
#define SPKGPU_ENSEMBLE_WARPS2 5
#define SPKGPU_ENSEMBLE_WARPS4 6
#define SPKGPU_ENSEMBLE_NMODES 7
int spkgpu_ensemble_mode(const spkgpu_ensemble *e, int32_t *mode, float *tune_ms);
/* device time (ms) of the sweep kernels in the most recent replay of the
   captured step and how many launches that covers (1 persistent kernel, or
   one launch per sweep); waits for that replay */
int spkgpu_ensemble_sweep_kernel_ms(spkgpu_ensemble *e, float *ms, int32_t *nlaunch);

#ifdef __cplusplus
}
#endif
#endif
