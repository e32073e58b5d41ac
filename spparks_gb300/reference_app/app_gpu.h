/* The GB300 path as SPPARKS app styles: the reference-side binding of
   include/spkgpu.h.

   SPPARKS runs a lattice app through the virtual AppLattice::iterate()
   (src/app.h:62, src/app_lattice.cpp:444-464), which calls the virtual
   iterate_rejection() for `sweep color` / `sweep color/strict`
   (src/app_lattice.h:159, src/app_lattice.cpp:632-711) and the non-virtual
   iterate_kmc_sector() for `solve_style tree` with sectors
   (src/app_lattice.cpp:517-626).  AppGPU<Base> derives from a stock app
   (AppIsing, AppPotts, AppPottsNeighOnly) and replaces both loops with the
   device: the stock app still reads the input, creates the sites and sets,
   seeds its generators and computes the diagnostics; between runs the host
   arrays are authoritative, during a run the device copy is.

   Per run the site values (and, for color/strict, the per-site Park-Miller
   seeds; with `mask yes`, the mask) go to the device, the passes run there,
   and at each output time the counters and site values come back before
   Output::compute, exactly where the stock loops call it.  With
   color/strict the device consumes the same per-site seeds in the same
   order as the stock app, so a run equals the stock run site for site;
   `sweep color` and tree KMC take Philox draws keyed by one value drawn
   from the master generator (RanMars) when the device handle is made.

   Limits: one process (the serial build), a simple square or cubic
   lattice filling the box (sq/4n, sq/8n, sc/6n, sc/26n), site ids in
   lattice order, sweep color or color/strict, or tree KMC with sectors;
   anything else ends with error->all.  Add this directory and the
   repository's include/ to the include path, link
   spparks_gb300/_lib/libspkgpu.so, compile app_gpu.cpp with the reference's
   sources, and list the style headers in style_app.h (app_ising_gpu.h,
   app_potts_gpu.h, app_potts_neighonly_gpu.h). */

#ifndef SPK_APP_GPU_H
#define SPK_APP_GPU_H

#include <math.h>
#include <stdint.h>
#include <string.h>

#include "app_lattice.h"
#include "domain.h"
#include "error.h"
#include "lattice.h"
#include "random_mars.h"
#include "random_park.h"
#include "solve.h"
#include "spkgpu.h"
#include "spparks.h"
#include "timer.h"

namespace SPPARKS_NS {

// Output::compute of the instance (app_gpu.cpp: output.h has no include
// guard, so only that file includes it)
double spk_gpu_output_compute(class SPPARKS *spk, double time, int done);

template <class Base>
class AppGPU : public Base {
 public:
  AppGPU(class SPPARKS *spk, int narg, char **arg) : Base(spk, narg, arg) {}
  ~AppGPU() override {
    if (h) spkgpu_destroy(h);
  }

  void iterate() override {
    // tree KMC over sectors on the device; every other loop as the stock
    // AppLattice::iterate dispatches it (iterate_rejection is overridden)
    if (this->solve && this->sectorflag && !(this->allow_app_update && this->app_update_only)) {
      this->timer->barrier_start(TIME_LOOP);
      iterate_kmc_gpu(this->stoptime);
      this->timer->barrier_stop(TIME_LOOP);
      return;
    }
    Base::iterate();
  }

 protected:
  spkgpu_lattice *h = nullptr;
  bool kmc_ready = false;

  // the stock app's enums (src/lattice.cpp:32, src/app_lattice.cpp:40)
  enum { LAT_SQ_4N = 2, LAT_SQ_8N = 3, LAT_SC_6N = 5, LAT_SC_26N = 6 };
  enum { SWEEP_COLOR = 3, SWEEP_COLOR_STRICT = 4 };

  void check(int rc) {
    if (rc) this->error->all(FLERR, h ? spkgpu_last_error(h) : "spkgpu call failed");
  }

  int *site_values() { return this->spin; }

  int gpu_app() const {
    if (!strcmp(this->style, "ising/gpu")) return SPKGPU_ISING;
    if (!strcmp(this->style, "potts/neighonly/gpu")) return SPKGPU_POTTS_NEIGHONLY;
    return SPKGPU_POTTS;
  }

  int nvalues() const { return gpu_app() == SPKGPU_ISING ? 2 : this->nspins_of(); }
  virtual int nspins_of() const { return 2; }

  // the device handle, made on the first run from the app's own settings
  void make_handle() {
    if (h) return;
    if (this->nprocs != 1) this->error->all(FLERR, "GPU app styles run in one process");
    if (!this->simple) this->error->all(FLERR, "GPU app styles need a simple lattice filling the box");
    spkgpu_desc d;
    memset(&d, 0, sizeof(d));
    switch (this->domain->lattice->style) {
      case LAT_SQ_4N: d.lattice = SPKGPU_SQ_4N; break;
      case LAT_SQ_8N: d.lattice = SPKGPU_SQ_8N; break;
      case LAT_SC_6N: d.lattice = SPKGPU_SC_6N; break;
      case LAT_SC_26N: d.lattice = SPKGPU_SC_26N; break;
      default: this->error->all(FLERR, "GPU app styles need lattice sq/4n, sq/8n, sc/6n or sc/26n");
    }
    d.nx = this->xhi_simple - this->xlo_simple + 1;
    d.ny = this->yhi_simple - this->ylo_simple + 1;
    d.nz = this->zhi_simple - this->zlo_simple + 1;
    if ((int64_t)d.nx * d.ny * d.nz != this->nlocal) this->error->all(FLERR, "GPU app styles need every site local");
    for (int i = 0; i < this->nlocal; i++)
      if (this->id[i] != (tagint)(i + 1)) this->error->all(FLERR, "GPU app styles need site ids in lattice order");
    d.app = gpu_app();
    d.nspins = nvalues();
    d.spin_bytes = 0;
    d.nsector = this->sectorflag ? this->nsector : 1;
    const int first = this->bothflag ? this->nsector : 0;
    d.nloop = this->solve ? 1 : this->set[first].nloop;
    d.procs[0] = d.procs[1] = d.procs[2] = 1;
    d.rng = this->sweepflag == SWEEP_COLOR_STRICT ? SPKGPU_RNG_STRICT : SPKGPU_RNG_PHILOX;
    d.mask = this->Lmask ? 1 : 0;
    // the Philox key: one draw of the master generator
    d.seed = (uint32_t)fmod(this->ranmaster->uniform() * 4294967296.0, 4294967296.0);
    d.device = 0;
    d.variant = 0;
    if (spkgpu_create(&d, &h)) this->error->all(FLERR, "spkgpu_create refused the lattice or the settings");
  }

  void to_device() {
    make_handle();
    check(spkgpu_set_temperature(h, this->temperature));
    check(spkgpu_upload_spins(h, site_values(), this->nlocal));
    if (this->siteseeds) check(spkgpu_upload_siteseeds(h, this->siteseeds, this->nlocal));
    if (this->Lmask) check(spkgpu_upload_mask(h, (const uint8_t *)this->mask, this->nlocal));
  }

  void from_device() {
    check(spkgpu_download_spins(h, site_values(), this->nlocal));
    if (this->siteseeds) check(spkgpu_download_siteseeds(h, this->siteseeds, this->nlocal));
    if (this->Lmask) check(spkgpu_download_mask(h, (uint8_t *)this->mask, this->nlocal));
  }

  // AppLattice::iterate_rejection (src/app_lattice.cpp:632-711) with every
  // pass over the sets on the device
  void iterate_rejection(double stoptime) override {
    if (this->sweepflag != SWEEP_COLOR && this->sweepflag != SWEEP_COLOR_STRICT)
      this->error->all(FLERR, "GPU app styles sweep with sweep color or color/strict");
    to_device();
    int done = 0;
    while (!done) {
      check(spkgpu_sweep(h, 1));
      this->nsweeps++;
      this->time += this->dt_rkmc;
      if (this->time >= stoptime) done = 1;
      if (done || this->time >= this->nextoutput) {
        spkgpu_stats st;
        check(spkgpu_get_stats(h, &st));
        this->naccept = st.naccept;
        this->nattempt = st.nattempt;
        from_device();
        this->nextoutput = spk_gpu_output_compute(this->spk, this->time, done);
      }
    }
  }

  // AppLattice::iterate_kmc_sector (src/app_lattice.cpp:517-626): passes up
  // to each output time on the device (the first call of a run recomputes
  // every propensity and the adaptive step, as AppLattice::setup does)
  void iterate_kmc_gpu(double stoptime) {
    to_device();
    if (!kmc_ready) {
      check(spkgpu_kmc_setup(h, this->Ladapt ? 1 : 0, this->nstop, this->tstop, 1));
      kmc_ready = true;
    }
    int done = 0, first = 1;
    while (!done) {
      spkgpu_kmc_stats ks;
      check(spkgpu_kmc_run_until(h, &this->time, stoptime, this->nextoutput, first, &ks));
      first = 0;
      this->naccept = ks.naccept;
      this->nsweeps = (int)ks.npass;
      done = this->time >= stoptime;
      from_device();
      this->nextoutput = spk_gpu_output_compute(this->spk, this->time, done);
    }
  }
};

}  // namespace SPPARKS_NS

#endif
