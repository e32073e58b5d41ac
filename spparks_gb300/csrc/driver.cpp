// Input-script driver behind the reference's library interface
// (src/library.h: spparks_open_no_mpi, spparks_close, spparks_file,
// spparks_command, spparks_extract, spparks_energy; bound by python/spparks.py),
// running the GB300 kernels through the spkgpu C ABI.
//
// It accepts the commands of the hot path with the reference's meaning:
//   seed N                          Input::seed (src/input.cpp:942-951)
//   app_style ising | potts Q | potts/neighonly Q | potts/neigh Q
//   dimension 2|3, lattice sq/4n|sq/8n|sc/6n|sc/26n 1.0
//   region NAME block 0 NX 0 NY (-0.5 0.5 | 0 NZ), create_box, create_sites
//   processors PX PY PZ              Domain::set_processors
//   set site range LO HI | set site value V   (Set::command, src/set.cpp)
//   sweep color | color/strict [mask yes|no]   (AppLattice::set_sweep)
//   sector yes|no|2|4|8 [nstop N | tstop T]     (AppLattice::set_sector)
//   temperature T, solve_style tree | none, stats DT
//   diag_style energy | array i1 mean|sum|min|max ... | cluster
//                                   stats columns of DiagEnergy, DiagArray,
//                                   DiagCluster (src/diag_*.cpp), computed on
//                                   the device (spkgpu_energy/site_stats/
//                                   clusters)
//   dump ID text|sites DT FILE [id site x y z energy i1]   (src/dump_text.cpp,
//                                   src/dump_sites.cpp), dump_modify ID
//                                   delay|delta|flush|tol, undump ID, dump_one ID
//   read_sites FILE                 Values section (src/read_sites.cpp)
//   log FILE | none                 Input::log
//   run DT [upto] [pre yes|no] [post yes|no]    (App::run, src/app.cpp:86-148)
// Stats, diagnostics and dumps follow Output::setup/compute
// (src/output.cpp:82-201), also between the passes of tree KMC.  Other
// output-only commands (the cluster diagnostic's files, ...) are accepted
// and ignored with a warning.  `sweep random|raster` (serial by definition) is
// refused.  Errors are printed as "ERROR: ..." like Error::all, but the
// process is not terminated: the command returns NULL and the message stays
// readable through spkgpu_driver_error().
//
// Random numbers: the master stream is the reference's Marsaglia generator
// (RanMars, src/random_mars.cpp) and per-use streams its Park-Miller
// RandomPark (src/random_park.cpp), consumed in the reference's order
// (`set site range`: one master draw; first run: two draws for ranapp, two
// more for color/strict per-site seeds), so initial values and color/strict
// runs equal the unmodified reference's.  `sweep color` draws Philox words
// keyed by the `seed` value.

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/spkgpu.h"

namespace {

std::vector<std::string> split_words(const char *line);

// Marsaglia RNG of RanMars (src/random_mars.cpp:43-105): the published
// universal generator of Marsaglia, Zaman and Tsang
struct MasterRng {
  double u[98];
  double c, cd, cm;
  int i97, j97;
  bool ready = false;
  void init(int seed) {
    int ij, kl, i, j, k, l, ii, jj, m;
    while (seed > 900000000) seed -= 900000000;
    ij = (seed - 1) / 30082;
    kl = (seed - 1) - 30082 * ij;
    i = (ij / 177) % 177 + 2;
    j = ij % 177 + 2;
    k = (kl / 169) % 178 + 1;
    l = kl % 169;
    for (ii = 1; ii <= 97; ii++) {
      double s = 0.0, t = 0.5;
      for (jj = 1; jj <= 24; jj++) {
        m = ((i * j) % 179) * k % 179;
        i = j;
        j = k;
        k = m;
        l = (53 * l + 1) % 169;
        if ((l * m) % 64 >= 32) s = s + t;
        t = 0.5 * t;
      }
      u[ii] = s;
    }
    c = 362436.0 / 16777216.0;
    cd = 7654321.0 / 16777216.0;
    cm = 16777213.0 / 16777216.0;
    i97 = 97;
    j97 = 33;
    ready = true;
    uniform();
  }
  double uniform() {
    double uni = u[i97] - u[j97];
    if (uni < 0.0) uni += 1.0;
    u[i97] = uni;
    if (--i97 == 0) i97 = 97;
    if (--j97 == 0) j97 = 97;
    c -= cd;
    if (c < 0.0) c += cm;
    uni -= c;
    if (uni < 0.0) uni += 1.0;
    return uni;
  }
};

// Park-Miller minimal standard (Park & Miller 1988) with Schrage's
// factorisation, the RandomPark recurrence (src/random_park.cpp:79-86)
struct Park {
  int seed = 1;
  static int from_double(double r) {
    int s = (int)(r * 2147483647);
    return s == 0 ? 1 : s;
  }
  static int reset(double r, long long offset, int warmup) {
    Park p;
    p.seed = (int)fmod(r * 2147483647 + (double)offset, 2147483647);
    if (p.seed < 0) p.seed = -p.seed;
    if (p.seed == 0) p.seed = 1;
    for (int i = 0; i < warmup; i++) p.uniform();
    return p.seed;
  }
  double uniform() {
    int k = seed / 127773;
    seed = 16807 * (seed - k * 127773) - 2836 * k;
    if (seed < 0) seed += 2147483647;
    return (1.0 / 2147483647) * seed;
  }
  int irandom(int n) {
    int i = (int)(uniform() * n) + 1;
    return i > n ? n : i;
  }
};

enum { SWEEP_NONE = 0, SWEEP_COLOR = 1, SWEEP_STRICT = 2 };

struct Driver {
  FILE *screen = stdout;
  FILE *logfile = nullptr;
  std::string error;
  MasterRng master;
  int seed = 0;
  // app
  std::string app;
  int app_id = -1, nspins = 0;
  int dimension = 3;
  int lattice = -1;
  double latconst = 1.0;
  int nx = 0, ny = 0, nz = 0;
  bool have_region = false, box = false, sites = false;
  int procs[3] = {1, 1, 1};
  std::vector<int32_t> site;       // host copy of iarray[0]
  bool host_valid = false;         // host copy is current (or authoritative)
  bool device_valid = false;       // device copy is current
  int sweepflag = SWEEP_NONE;
  bool mask = false;
  int nsector_user = 0, sectorflag = 0;
  double nstop = 1.0, tstop = 0.0;
  double temperature = 0.0;
  bool tree = false;
  double stats_delta = 0.0;
  // diagnostics in declaration order (Output::stats_header prints them so)
  enum { DIAG_ENERGY, DIAG_ARRAY, DIAG_CLUSTER };
  enum { AMEAN, ASUM, AMIN, AMAX };
  struct DiagSpec {
    int kind;
    bool stats = true;
    std::vector<int> methods;  // array: one column per (i1, method) pair
  };
  std::vector<DiagSpec> diags;
  // dumps in declaration order
  enum { F_ID, F_SITE, F_X, F_Y, F_Z, F_ENERGY };
  struct DumpSpec {
    std::string id, style, filename, columns, columns_orig;
    double delta = 0.0, delay = 0.0, tolerance = 0.0, next_time = 0.0;
    std::vector<int> fields;
    bool multifile = false, flush = true, first = true;
    int idump = 0, pad = 0;
    FILE *fp = nullptr;  // the single file, open from the first run on
  };
  std::vector<DumpSpec> dumps;
  double stats_time = 0.0;
  // run state
  double time = 0.0;
  int64_t nsweeps = 0, naccept = 0, nattempt = 0;
  bool first_run = true;
  spkgpu_lattice *h = nullptr;
  int h_key[13] = {0};
  bool kmc_ready = false;
  std::vector<int32_t> siteseeds;
  bool seeds_on_device = false;
  std::string extract_name;
  int64_t nglobal_store = 0;
  int nlocal_store = 0;
  double box_store[6] = {0, 0, 0, 0, 0, 0};

  ~Driver() {
    if (h) spkgpu_destroy(h);
    for (DumpSpec &d : dumps)
      if (d.fp) fclose(d.fp);
    if (logfile) fclose(logfile);
  }

  void print(const char *fmt, ...) {
    char buf[4096];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (screen) fputs(buf, screen);
    if (logfile) fputs(buf, logfile);
  }

  bool fail(const std::string &m) {
    error = m;
    print("ERROR: %s\n", m.c_str());
    return false;
  }

  int64_t n() const { return (int64_t)nx * ny * nz; }
  int maxneigh() const {
    static const int mn[4] = {4, 8, 6, 26};
    return lattice >= 0 ? mn[lattice] : 0;
  }
  double dt_sweep() const {
    if (app_id == SPKGPU_ISING) return 1.0 / 2.0;
    if (app_id == SPKGPU_POTTS) return 1.0 / nspins;
    return 1.0 / maxneigh();
  }
  int nsector() const {
    if (!sectorflag) return 1;
    if (nsector_user) return nsector_user;
    return dimension == 2 ? 4 : 8;
  }
  // passes over each set per sweep (src/app_lattice.cpp:398-407)
  int nloop() const {
    if (sweepflag == SWEEP_NONE) return 1;
    if (tstop > 0.0) return (int)(tstop / dt_sweep());
    return (int)nstop;
  }

  bool command(std::vector<std::string> &w);
  bool run(std::vector<std::string> &w);
  bool diag_style(std::vector<std::string> &w);
  std::string diag_header() const;
  std::string diag_values();
  bool ensure_handle();
  bool sync_to_host();
  void stats_line(double cpu);
  // output (src/output.cpp)
  static double next_time(double t, double delta, double delay);
  bool output_setup(double stoptime, double *tnext);
  bool output_compute(double stoptime, bool done, double cpu, double *tnext);
  bool dump_command(std::vector<std::string> &w);
  bool dump_modify(std::vector<std::string> &w);
  bool dump_write(DumpSpec &d);
  bool read_sites(const std::string &file);
  bool current_sites(std::vector<int32_t> &out);
};

double wall() {
  struct timeval tv;
  gettimeofday(&tv, nullptr);
  return tv.tv_sec + 1e-6 * tv.tv_usec;
}

bool parse_int(const std::string &s, int *out) {
  char *e = nullptr;
  long v = strtol(s.c_str(), &e, 10);
  if (!e || *e) return false;
  *out = (int)v;
  return true;
}

bool parse_double(const std::string &s, double *out) {
  char *e = nullptr;
  double v = strtod(s.c_str(), &e);
  if (!e || *e) return false;
  *out = v;
  return true;
}

bool Driver::sync_to_host() {
  if (host_valid) return true;
  if (!h || !device_valid) return true;
  site.resize(n());
  if (spkgpu_download_spins(h, site.data(), n()) != 0) return fail(spkgpu_last_error(h));
  host_valid = true;
  return true;
}

bool Driver::ensure_handle() {
  int key[13] = {lattice, nx, ny, nz, app_id, nspins, nsector(), procs[0], procs[1], procs[2],
                 sweepflag == SWEEP_STRICT ? 1 : 0, mask ? 1 : 0, nloop()};
  if (h && memcmp(key, h_key, sizeof(key)) == 0) return true;
  if (h) {
    if (!sync_to_host()) return false;
    spkgpu_destroy(h);
    h = nullptr;
    device_valid = false;
    seeds_on_device = false;
    kmc_ready = false;
  }
  spkgpu_desc d;
  memset(&d, 0, sizeof(d));
  d.lattice = lattice;
  d.nx = nx;
  d.ny = ny;
  d.nz = nz;
  d.app = app_id;
  d.nspins = nspins;
  d.spin_bytes = 0;
  d.nsector = nsector();
  d.nloop = nloop() < 1 ? 1 : nloop();
  d.procs[0] = procs[0];
  d.procs[1] = procs[1];
  d.procs[2] = procs[2];
  d.rng = sweepflag == SWEEP_STRICT ? SPKGPU_RNG_STRICT : SPKGPU_RNG_PHILOX;
  d.mask = mask ? 1 : 0;
  d.seed = (uint32_t)seed;
  d.device = 0;
  d.variant = 0;
  int rc = spkgpu_create(&d, &h);
  if (rc != 0) return fail("the GPU path cannot run this configuration (spkgpu_create returned " +
                           std::to_string(rc) + ")");
  memcpy(h_key, key, sizeof(key));
  return true;
}

void Driver::stats_line(double cpu) {
  char line[256];
  int off = snprintf(line, sizeof(line), "%10g %10lld %10lld %10lld %10.3g", time, (long long)naccept,
                     (long long)(tree ? 0 : nattempt - naccept), (long long)nsweeps, cpu);
  std::string out = line;
  if (h) out += diag_values();
  print("%s\n", out.c_str());
}

// Diag::Diag (src/diag.cpp:40-98) keywords, then the style's own:
// DiagArray takes (iN|dN, mean|sum|min|max) pairs only
// (src/diag_array.cpp:36-90), DiagCluster filename/dump/site/size
// (src/diag_cluster.cpp:60-110; their files are not written here)
bool Driver::diag_style(std::vector<std::string> &w) {
  if (app_id < 0) return fail("Diag_style command before app_style set");
  if (w.size() < 2) return fail("Illegal diag_style command");
  DiagSpec d;
  size_t k = 2;
  auto base_keywords = [&]() -> bool {
    while (k < w.size()) {
      if (w[k] == "stats") {
        if (k + 1 >= w.size() || (w[k + 1] != "yes" && w[k + 1] != "no")) return fail("Illegal diag_style command");
        d.stats = w[k + 1] == "yes";
        k += 2;
      } else if (w[k] == "delt" || w[k] == "delay") {
        if (k + 1 >= w.size()) return fail("Illegal diag_style command");
        print("WARNING: diag_style %s is ignored by the GPU driver\n", w[k].c_str());
        k += 2;
      } else if (w[k] == "logfreq" || w[k] == "loglinfreq") {
        if (k + 2 >= w.size()) return fail("Illegal diag_style command");
        print("WARNING: diag_style %s is ignored by the GPU driver\n", w[k].c_str());
        k += 3;
      } else {
        break;
      }
    }
    return true;
  };
  if (w[1] == "energy") {
    d.kind = DIAG_ENERGY;
    if (!base_keywords()) return false;
    if (k < w.size()) return fail("Illegal diag_style command");
  } else if (w[1] == "array") {
    d.kind = DIAG_ARRAY;
    if ((w.size() - 2) % 2 != 0 || w.size() < 4) return fail("Invalid diag_style command");
    for (k = 2; k < w.size(); k += 2) {
      // the on-lattice apps of this path have one integer array (the site
      // values) and no double arrays
      if (w[k] != "i1") return fail("Invalid diag_style command");
      const std::string &m = w[k + 1];
      if (m == "mean") d.methods.push_back(AMEAN);
      else if (m == "sum") d.methods.push_back(ASUM);
      else if (m == "min") d.methods.push_back(AMIN);
      else if (m == "max") d.methods.push_back(AMAX);
      else return fail("Invalid diag_style command");
    }
  } else if (w[1] == "cluster") {
    d.kind = DIAG_CLUSTER;
    if (!base_keywords()) return false;
    while (k < w.size()) {
      if (w[k] == "filename" && k + 1 < w.size()) k += 2;
      else if (w[k] == "dump" && k + 1 < w.size()) k += (w[k + 1] == "none") ? 2 : 3;
      else if (w[k] == "site/size") k += 1;
      else return fail("Illegal diag_style cluster command");
      print("WARNING: diag_style cluster output files are not written by the GPU driver\n");
    }
  } else {
    print("WARNING: diag_style %s is ignored by the GPU driver\n", w[1].c_str());
    return true;
  }
  diags.push_back(d);
  return true;
}

std::string Driver::diag_header() const {
  static const char *names[] = {"mean", "sum", "min", "max"};
  std::string out;
  char buf[64];
  for (const DiagSpec &d : diags) {
    if (!d.stats) continue;
    if (d.kind == DIAG_ENERGY) {
      snprintf(buf, sizeof(buf), " %10s", "Energy");
      out += buf;
    } else if (d.kind == DIAG_ARRAY) {
      for (int m : d.methods) {
        std::string col = std::string(names[m]) + "(i1)";
        snprintf(buf, sizeof(buf), " %10s", col.c_str());
        out += buf;
      }
    } else {
      snprintf(buf, sizeof(buf), " %10s %10s %10s", "Nclust", "<N>", "<R>");
      out += buf;
    }
  }
  return out;
}

// the diag columns of one stats line, from the device lattice
std::string Driver::diag_values() {
  std::string out;
  char buf[96];
  for (const DiagSpec &d : diags) {
    if (!d.stats) continue;
    if (d.kind == DIAG_ENERGY) {
      double e = 0.0;
      if (spkgpu_energy(h, &e) != 0) continue;
      snprintf(buf, sizeof(buf), " %10g", e);
      out += buf;
    } else if (d.kind == DIAG_ARRAY) {
      int64_t sum = 0;
      int32_t lo = 0, hi = 0;
      if (spkgpu_site_stats(h, &sum, &lo, &hi) != 0) continue;
      for (int m : d.methods) {
        double v = m == AMEAN ? (double)sum / (double)n()
                              : m == ASUM ? (double)sum : m == AMIN ? (double)lo : (double)hi;
        snprintf(buf, sizeof(buf), " %10g", v);
        out += buf;
      }
    } else {
      int64_t nc = 0;
      double vav = 0.0, rav = 0.0;
      if (spkgpu_clusters(h, &nc, &vav, &rav) != 0) continue;
      snprintf(buf, sizeof(buf), " %10d %10g %10g", (int)nc, vav, rav);
      out += buf;
    }
  }
  return out;
}

// Output::next_time without log spacing (src/output.cpp:414-437)
double Driver::next_time(double t, double delta, double delay) {
  double tnew = ceil(t / delta) * delta;
  if (tnew == t) tnew = t + delta;
  return tnew > delay ? tnew : delay;
}

// the site values as they are now: the host copy, or the device's during a run
bool Driver::current_sites(std::vector<int32_t> &out) {
  if (host_valid || !h || !device_valid) {
    out = site;
    return true;
  }
  out.resize(n());
  if (spkgpu_download_spins(h, out.data(), n()) != 0) return fail(spkgpu_last_error(h));
  return true;
}

// neighbour offsets of the lattice style (CreateSites::offsets_2d/3d,
// src/create_sites.cpp:1303-1371)
static void lattice_offsets(int lattice, std::vector<int> &dx, std::vector<int> &dy, std::vector<int> &dz) {
  const bool is3d = lattice >= 2;
  for (int a = -1; a <= 1; a++)
    for (int b = -1; b <= 1; b++)
      for (int c = is3d ? -1 : 0; c <= (is3d ? 1 : 0); c++) {
        const int r2 = a * a + b * b + c * c;
        const bool keep = (lattice == 0 || lattice == 2) ? r2 == 1 : r2 >= 1;
        if (!keep) continue;
        dx.push_back(a);
        dy.push_back(b);
        dz.push_back(c);
      }
}

// Dump::write with the DumpText (src/dump_text.cpp:347-421) and DumpSites
// (src/dump_sites.cpp:51-67) headers; one process, so rows in id order
bool Driver::dump_write(DumpSpec &d) {
  std::vector<int32_t> v;
  if (!current_sites(v)) return false;
  FILE *fp = d.fp;
  if (d.multifile) {
    const size_t star = d.filename.find('*');
    char num[32];
    snprintf(num, sizeof(num), "%0*d", d.pad, d.idump);
    const std::string name = d.filename.substr(0, star) + num + d.filename.substr(star + 1);
    fp = fopen(name.c_str(), "w");
    if (!fp) return fail("Cannot open dump file " + name);
  } else if (!fp) {
    d.fp = fp = fopen(d.filename.c_str(), "w");
    if (!fp) return fail("Cannot open dump file " + d.filename);
  }
  const long long nd = (long long)n();
  const double zlo = dimension == 2 ? -0.5 : 0.0, zhi = dimension == 2 ? 0.5 : (double)nz;
  if (d.style == "sites") {
    fprintf(fp, "Site file written by dump sites %s command at time: %d %g\n\n", d.id.c_str(), d.idump, time);
    fprintf(fp, "%d dimension\n", dimension);
    fprintf(fp, "%lld sites\n", nd);
    fprintf(fp, "%s values\n", d.columns_orig.c_str());
    fprintf(fp, "%g %g xlo xhi\n", 0.0, (double)nx);
    fprintf(fp, "%g %g ylo yhi\n", 0.0, (double)ny);
    fprintf(fp, "%g %g zlo zhi\n", zlo, zhi);
    fprintf(fp, "\nValues\n\n");
  } else {
    fprintf(fp, "ITEM: TIMESTEP\n");
    fprintf(fp, "%d %10g\n", d.idump, time);
    fprintf(fp, "ITEM: NUMBER OF ATOMS\n");
    fprintf(fp, "%lld\n", nd);
    fprintf(fp, "ITEM: BOX BOUNDS\n");
    fprintf(fp, "%g %g\n", 0.0, (double)nx);
    fprintf(fp, "%g %g\n", 0.0, (double)ny);
    fprintf(fp, "%g %g\n", zlo, zhi);
    fprintf(fp, "ITEM: ATOMS %s\n", d.columns.c_str());
  }
  std::vector<int> ox, oy, oz;
  lattice_offsets(lattice, ox, oy, oz);
  for (int64_t i = 0; i < (int64_t)nd; i++) {
    const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((int64_t)nx * ny));
    for (int f : d.fields) {
      switch (f) {
        case F_ID: fprintf(fp, "%d ", (int)(i + 1)); break;
        case F_SITE: fprintf(fp, "%d ", v[i]); break;
        case F_X: fprintf(fp, "%g ", (double)x); break;
        case F_Y: fprintf(fp, "%g ", (double)y); break;
        case F_Z: fprintf(fp, "%g ", (double)z); break;
        default: {
          // site_energy: unlike neighbours (src/app_potts.cpp:97-104)
          int e = 0;
          for (size_t j = 0; j < ox.size(); j++) {
            const int xn = (x + ox[j] + nx) % nx, yn = (y + oy[j] + ny) % ny, zn = (z + oz[j] + nz) % nz;
            e += v[xn + (int64_t)nx * (yn + (int64_t)ny * zn)] != v[i];
          }
          fprintf(fp, "%g ", (double)e);
        }
      }
    }
    fputc('\n', fp);
  }
  if (d.flush) fflush(fp);
  if (d.multifile) fclose(fp);
  d.first = false;
  d.idump++;
  return true;
}

// Output::setup (src/output.cpp:82-141): first dumps, stats header and row
bool Driver::output_setup(double stoptime, double *tnext) {
  double dump_time = stoptime;
  for (DumpSpec &d : dumps) {
    if (d.first && time >= d.delay)
      if (!dump_write(d)) return false;
    d.next_time = next_time(time + d.tolerance, d.delta, d.delay) - d.tolerance;
    dump_time = std::min(dump_time, d.next_time);
  }
  print("%10s %10s %10s %10s %10s%s\n", "Time", "Naccept", "Nreject", "Nsweeps", "CPU", diag_header().c_str());
  stats_line(0.0);
  stats_time = stats_delta > 0.0 ? next_time(time, stats_delta, 0.0) : stoptime;
  *tnext = std::min(stoptime, std::min(dump_time, stats_time));
  return true;
}

// Output::compute (src/output.cpp:148-201): stats row when due or done, then
// the dumps that are due
bool Driver::output_compute(double stoptime, bool done, double cpu, double *tnext) {
  if (time >= stats_time || done) {
    stats_line(cpu);
    stats_time = stats_delta > 0.0 ? next_time(time, stats_delta, 0.0) : stoptime;
  }
  double dump_time = stoptime;
  for (DumpSpec &d : dumps) {
    if (time >= d.next_time - d.tolerance) {
      if (!dump_write(d)) return false;
      d.next_time = next_time(time + d.tolerance, d.delta, d.delay) - d.tolerance;
    }
    dump_time = std::min(dump_time, d.next_time);
  }
  *tnext = std::min(stoptime, std::min(dump_time, stats_time));
  return true;
}

// dump ID style DELTA FILE fields (Dump::Dump, src/dump.cpp:40-140;
// DumpText::parse_fields, src/dump_text.cpp:426-490; DumpSites checks,
// src/dump_sites.cpp:29-48)
bool Driver::dump_command(std::vector<std::string> &w) {
  if (app_id < 0) return fail("Dump command before app_style set");
  if (w.size() < 5) return fail("Illegal dump command");
  for (const DumpSpec &o : dumps)
    if (o.id == w[1]) return fail("Reuse of dump ID");
  DumpSpec d;
  d.id = w[1];
  d.style = w[2];
  if (d.style != "text" && d.style != "sites") {
    print("WARNING: dump style %s is not written by the GPU driver\n", d.style.c_str());
    return true;
  }
  if (!parse_double(w[3], &d.delta) || d.delta <= 0.0) return fail("Illegal dump command");
  d.filename = w[4];
  auto ends = [&](const char *suf) {
    size_t k = strlen(suf);
    return d.filename.size() > k && d.filename.compare(d.filename.size() - k, k, suf) == 0;
  };
  if (ends(".bin") || ends(".gz")) return fail("the GPU driver writes text dumps only");
  size_t pct = d.filename.find('%');
  if (pct != std::string::npos) {
    if (d.style == "sites") return fail("Dump sites cannot write multiple files per snapshot");
    d.filename.replace(pct, 1, "0");  // one process
  }
  d.multifile = d.filename.find('*') != std::string::npos;
  std::vector<std::string> f(w.begin() + 5, w.end());
  if (f.empty() && d.style == "text") f = {"id", "site", "x", "y", "z"};
  for (const std::string &a : f) {
    if (a == "id") d.fields.push_back(F_ID);
    else if (a == "site" || a == "i1") d.fields.push_back(F_SITE);
    else if (a == "x") d.fields.push_back(F_X);
    else if (a == "y") d.fields.push_back(F_Y);
    else if (a == "z") d.fields.push_back(F_Z);
    else if (a == "energy") d.fields.push_back(F_ENERGY);
    else if (a == "propensity") return fail("dump propensity is not written by the GPU driver");
    else return fail("Invalid keyword in dump command");
    if (!d.columns.empty()) d.columns += " ";
    d.columns += a.find("site") != std::string::npos ? "type" : a;
    if (!d.columns_orig.empty()) d.columns_orig += " ";
    d.columns_orig += a;
  }
  if (d.style == "sites") {
    if (!d.multifile) return fail("Dump sites must write one file per snapshot");
    if (d.fields.empty() || d.fields[0] != F_ID) return fail("Dump sites requires ID as first field");
    if (d.fields.size() < 2) return fail("Dump sites requires two or more fields");
  }
  dumps.push_back(d);
  return true;
}

// dump_modify ID keyword value ... (Dump::modify_params, src/dump.cpp:640-800)
bool Driver::dump_modify(std::vector<std::string> &w) {
  if (w.size() < 2) return fail("Illegal dump_modify command");
  DumpSpec *d = nullptr;
  for (DumpSpec &o : dumps)
    if (o.id == w[1]) d = &o;
  if (!d) return fail("Could not find dump ID in dump_modify command");
  for (size_t k = 2; k < w.size(); k += 2) {
    if (k + 1 >= w.size()) return fail("Illegal dump_modify command");
    const std::string &key = w[k], &val = w[k + 1];
    double v = 0.0;
    if (key == "delay" && parse_double(val, &v)) d->delay = v;
    else if (key == "delta" && parse_double(val, &v) && v > 0.0) d->delta = v;
    else if (key == "tol" && parse_double(val, &v) && v >= 0.0) d->tolerance = v;
    else if (key == "flush" && (val == "yes" || val == "no")) d->flush = val == "yes";
    else if (key == "pad" && parse_int(val, &d->pad) && d->pad >= 0) {}
    else return fail("dump_modify " + key + " is not supported by the GPU driver");
  }
  return true;
}

// read_sites FILE: the Values section onto existing sites (ReadSites::command,
// header, values: src/read_sites.cpp:69-640); Sites/Neighbors sections
// describe explicit lattices, which the GPU path creates with create_sites
bool Driver::read_sites(const std::string &file) {
  if (app_id < 0) return fail("Read_sites command before app_style set");
  FILE *fp = fopen(file.c_str(), "r");
  if (!fp) return fail("Cannot open file " + file);
  print("Reading site file ...\n");
  char line[4096];
  std::string columns;
  bool have_columns = false;
  auto done_with = [&](bool ok) {
    fclose(fp);
    return ok;
  };
  if (!fgets(line, sizeof(line), fp)) return done_with(fail("Unexpected end of data file"));
  std::string keyword;
  while (fgets(line, sizeof(line), fp)) {
    if (char *c = strchr(line, '#')) *c = '\0';
    if (strspn(line, " \t\n\r") == strlen(line)) continue;
    std::string l = line;
    double a = 0.0, b = 0.0;
    if (l.find("dimension") != std::string::npos) {
      int dim = atoi(line);
      if (box && dim != dimension) return done_with(fail("Data file dimension does not match existing box"));
    } else if (l.find("max neighbors") != std::string::npos) {
      return done_with(fail("read_sites Sites/Neighbors describe explicit lattices; the GPU path uses create_sites"));
    } else if (l.find("sites") != std::string::npos) {
      long long ng = atoll(line);
      if (sites && ng != (long long)n())
        return done_with(fail("Data file number of sites does not match existing sites"));
    } else if (l.find("values") != std::string::npos) {
      columns = l.substr(0, l.find("values"));
      have_columns = true;
    } else if (l.find("xlo xhi") != std::string::npos || l.find("ylo yhi") != std::string::npos ||
               l.find("zlo zhi") != std::string::npos) {
      sscanf(line, "%lg %lg", &a, &b);
    } else {
      size_t s0 = l.find_first_not_of(" \t\n\r"), s1 = l.find_last_not_of(" \t\n\r");
      keyword = l.substr(s0, s1 - s0 + 1);
      break;
    }
  }
  bool any = false;
  while (!keyword.empty()) {
    if (keyword != "Values")
      return done_with(fail(keyword == "Sites" || keyword == "Neighbors"
                                ? "read_sites " + keyword + " sections are not on the GPU path (use create_sites)"
                                : "Unknown identifier in data file: " + keyword));
    if (!sites) return done_with(fail("Cannot read Values before sites exist or are read"));
    if (!fgets(line, sizeof(line), fp)) return done_with(fail("Unexpected end of data file"));  // blank line
    // columns: "id" then site|i1 (the apps here have one integer per site)
    std::vector<int> cols;
    if (!have_columns) {
      cols.push_back(1);
    } else {
      std::vector<std::string> words = split_words(columns.c_str());
      if (words.size() < 2) return done_with(fail("Read sites Values section has no values per site"));
      if (words[0] != "id") return done_with(fail("Read sites values header keyword must start with id"));
      for (size_t k = 1; k < words.size(); k++) {
        if (words[k] == "site" || words[k] == "i1") cols.push_back(1);
        else return done_with(fail("Invalid keyword in read sites values header"));
      }
    }
    if (!sync_to_host()) return done_with(false);
    for (int64_t r = 0; r < n(); r++) {
      if (!fgets(line, sizeof(line), fp)) return done_with(fail("Unexpected end of data file"));
      std::vector<std::string> words = split_words(line);
      if (words.size() != cols.size() + 1) return done_with(fail("Incorrect value format in data file"));
      long long id = atoll(words[0].c_str());
      if (id < 1 || id > (long long)n()) continue;  // not a site of this lattice
      for (size_t k = 0; k < cols.size(); k++) site[id - 1] = atoi(words[k + 1].c_str());
    }
    host_valid = true;
    device_valid = false;
    any = true;
    print("  %lld values\n", (long long)n() * (long long)cols.size());
    // next keyword: skip blank lines, then read the keyword line
    keyword.clear();
    while (fgets(line, sizeof(line), fp)) {
      if (strspn(line, " \t\n\r") == strlen(line)) continue;
      std::string l = line;
      size_t s0 = l.find_first_not_of(" \t\n\r"), s1 = l.find_last_not_of(" \t\n\r");
      keyword = l.substr(s0, s1 - s0 + 1);
      break;
    }
  }
  if (!any) return done_with(fail("Site file has no Sites, Neighbors, or Values"));
  return done_with(true);
}

bool Driver::run(std::vector<std::string> &w) {
  if (app_id < 0) return fail("Run command before app_style set");
  if (!box) return fail("Cannot run application until simulation box is defined");
  if (!sites) return fail("Cannot run application until sites exist");
  if (w.size() < 2) return fail("Illegal run command");
  double delta;
  if (!parse_double(w[1], &delta)) return fail("Illegal run command");
  double stoptime = time + delta;
  if (stoptime < time) return fail("Illegal run command");
  bool upto = false;
  for (size_t k = 2; k < w.size(); k++) {
    if (w[k] == "upto") upto = true;
    else if ((w[k] == "pre" || w[k] == "post") && k + 1 < w.size()) k++;
    else return fail("Illegal run command");
  }
  if (upto) stoptime -= time;
  if (!tree && sweepflag == SWEEP_NONE) return fail("App needs a KMC or rejection KMC solver");
  if (tree && sweepflag != SWEEP_NONE) return fail("App cannot use both a KMC and rejection KMC solver");
  if (sectorflag && sweepflag == SWEEP_STRICT) return fail("Cannot use color/strict rejection KMC with sectors");
  if (tree && !sectorflag) return fail("the GPU path runs tree KMC with sectors (sector yes)");
  if (host_valid)
    for (int32_t v : site)
      if (v < 1 || v > nspins) return fail("One or more sites have invalid values");
  if (!ensure_handle()) return false;
  // first run: ranapp (two master draws), then the color/strict seeds
  // (src/app_lattice.cpp:274-295)
  if (first_run) {
    if (!master.ready) return fail("Seed command has not been used");
    master.uniform();
    master.uniform();
    if (sweepflag == SWEEP_STRICT) {
      master.uniform();
      double rs = master.uniform();
      siteseeds.resize(n());
      for (int64_t i = 0; i < n(); i++) siteseeds[i] = Park::reset(rs, i + 1, 100);
    }
  }
  if (spkgpu_set_temperature(h, temperature) != 0) return fail(spkgpu_last_error(h));
  if (!device_valid) {
    if (spkgpu_upload_spins(h, site.data(), n()) != 0) return fail(spkgpu_last_error(h));
    device_valid = true;
  }
  if (sweepflag == SWEEP_STRICT && !seeds_on_device) {
    if (spkgpu_upload_siteseeds(h, siteseeds.data(), n()) != 0) return fail(spkgpu_last_error(h));
    seeds_on_device = true;
  }
  host_valid = false;
  first_run = false;
  print("Setting up run ...\n");
  double t0 = wall();
  double nextoutput = stoptime;
  if (!output_setup(stoptime, &nextoutput)) return false;
  if (tree) {
    spkgpu_kmc_stats ks;
    // one solver state per handle: consecutive runs continue its event
    // counters, as the reference reuses its solvers (src/app_lattice.cpp:205-211)
    if (!kmc_ready) {
      if (spkgpu_kmc_setup(h, tstop > 0.0 ? 0 : 1, nstop, tstop, 1) != 0) return fail(spkgpu_last_error(h));
      kmc_ready = true;
    }
    if (stoptime > time) {
      // passes up to each output time (src/app_lattice.cpp:517-626)
      bool done = false, first = true;
      while (!done) {
        if (spkgpu_kmc_run_until(h, &time, stoptime, nextoutput, first ? 1 : 0, &ks) != 0)
          return fail(spkgpu_last_error(h));
        first = false;
        naccept = ks.naccept;
        nsweeps = ks.npass;
        done = time >= stoptime;
        if (!output_compute(stoptime, done, wall() - t0, &nextoutput)) return false;
      }
    } else if (!output_compute(stoptime, true, wall() - t0, &nextoutput)) {
      return false;
    }
  } else {
    // rejection KMC: dt_rkmc = nloop * dt_sweep per pass over all sets
    // (src/app_lattice.cpp:398-420)
    if (nloop() < 1) return fail("Choice of sector stop led to no rKMC events");
    double dt_rkmc = nloop() * dt_sweep();
    dt_rkmc = fmin(dt_rkmc, stoptime - time);
    bool done = !(stoptime > time);
    while (!done) {
      if (spkgpu_sweep(h, 1) != 0) return fail(spkgpu_last_error(h));
      nsweeps++;
      time += dt_rkmc;
      if (time >= stoptime) done = true;
      if (done || time >= nextoutput) {
        spkgpu_stats st;
        if (spkgpu_get_stats(h, &st) != 0) return fail(spkgpu_last_error(h));
        naccept = st.naccept;
        nattempt = st.nattempt;
        if (!output_compute(stoptime, done, wall() - t0, &nextoutput)) return false;
      }
    }
  }
  print("Loop time of %g on 1 procs\n\n", wall() - t0);
  return true;
}

bool Driver::command(std::vector<std::string> &w) {
  const std::string &c = w[0];
  auto need = [&](size_t k) { return w.size() >= k; };
  if (c == "seed") {
    int s;
    if (w.size() != 2 || !parse_int(w[1], &s) || s <= 0) return fail("Illegal seed command");
    seed = s;
    master.init(s);
  } else if (c == "app_style") {
    if (box) return fail("App_style command after simulation box is defined");
    if (!need(2)) return fail("Illegal app_style command");
    app = w[1];
    if (app == "ising") {
      if (w.size() != 2) return fail("Illegal app_style command");
      app_id = SPKGPU_ISING;
      nspins = 2;
    } else if (app == "potts" || app == "potts/neighonly" || app == "potts/neigh") {
      if (w.size() != 3 || !parse_int(w[2], &nspins) || nspins <= 0) return fail("Illegal app_style command");
      app_id = app == "potts" ? SPKGPU_POTTS : (app == "potts/neighonly" ? SPKGPU_POTTS_NEIGHONLY : SPKGPU_POTTS_NEIGH);
    } else {
      return fail("app_style " + app + " is not on the GPU path (ising, potts, potts/neighonly, potts/neigh)");
    }
  } else if (c == "dimension") {
    if (w.size() != 2 || !parse_int(w[1], &dimension) || (dimension != 2 && dimension != 3))
      return fail("Illegal dimension command");
  } else if (c == "lattice") {
    if (w.size() != 3 || !parse_double(w[2], &latconst)) return fail("Illegal lattice command");
    static const char *names[4] = {"sq/4n", "sq/8n", "sc/6n", "sc/26n"};
    lattice = -1;
    for (int k = 0; k < 4; k++)
      if (w[1] == names[k]) lattice = k;
    if (lattice < 0) return fail("lattice " + w[1] + " is not on the GPU path (sq/4n, sq/8n, sc/6n, sc/26n)");
    if (latconst != 1.0) return fail("the GPU path takes lattice constant 1.0");
    if ((lattice <= 1) != (dimension == 2)) return fail("Lattice style does not match dimension");
  } else if (c == "region") {
    if (w.size() != 9 || w[2] != "block") return fail("the GPU path takes one region: NAME block 0 NX 0 NY ZLO ZHI");
    double b[6];
    for (int k = 0; k < 6; k++)
      if (!parse_double(w[3 + k], &b[k])) return fail("Illegal region command");
    if (b[0] != 0.0 || b[2] != 0.0 || b[1] != floor(b[1]) || b[3] != floor(b[3]))
      return fail("region bounds must be 0 .. N in lattice units");
    nx = (int)b[1];
    ny = (int)b[3];
    if (dimension == 2) {
      if (b[4] != -0.5 || b[5] != 0.5) return fail("2d regions span z -0.5 0.5");
      nz = 1;
    } else {
      if (b[4] != 0.0 || b[5] != floor(b[5])) return fail("region bounds must be 0 .. N in lattice units");
      nz = (int)b[5];
    }
    for (int k = 0; k < 6; k++) box_store[k] = b[k];
    have_region = true;
  } else if (c == "create_box") {
    if (!have_region || app_id < 0 || lattice < 0) return fail("Create_box command before region/app/lattice");
    box = true;
  } else if (c == "create_sites") {
    if (!box) return fail("Create_sites command before simulation box is defined");
    sites = true;
    site.assign(n(), 0);
    host_valid = true;
    device_valid = false;
    print("Creating sites ...\n  %lld sites\n", (long long)n());
  } else if (c == "processors") {
    if (w.size() != 4) return fail("Illegal processors command");
    for (int k = 0; k < 3; k++)
      if (!parse_int(w[1 + k], &procs[k]) || procs[k] < 1) return fail("Illegal processors command");
  } else if (c == "set") {
    if (!sites) return fail("Set command before sites exist");
    if (w.size() < 3 || w[1] != "site") return fail("the GPU driver supports `set site range|value`");
    if (!sync_to_host()) return false;
    if (w[2] == "value" && w.size() == 4) {
      int v;
      if (!parse_int(w[3], &v)) return fail("Illegal set command");
      for (auto &x : site) x = v;
    } else if (w[2] == "range" && w.size() == 5) {
      int lo, hi;
      if (!parse_int(w[3], &lo) || !parse_int(w[4], &hi)) return fail("Illegal set command");
      if (!master.ready) return fail("Seed command has not been used");
      // loop option (the default): one stream over all site IDs in order
      Park p;
      p.seed = Park::from_double(master.uniform());
      for (auto &x : site) x = p.irandom(hi - lo + 1) - 1 + lo;
    } else {
      return fail("the GPU driver supports `set site range LO HI` and `set site value V`");
    }
    host_valid = true;
    device_valid = false;
    print("  %lld settings made for site\n", (long long)n());
  } else if (c == "sweep") {
    if (!need(2)) return fail("Illegal sweep command");
    if (w[1] == "color") sweepflag = SWEEP_COLOR;
    else if (w[1] == "color/strict") sweepflag = SWEEP_STRICT;
    else if (w[1] == "none") sweepflag = SWEEP_NONE;
    else if (w[1] == "random" || w[1] == "raster")
      return fail("sweep " + w[1] + " is a serial site order; the GPU path runs sweep color and color/strict");
    else return fail("Illegal sweep command");
    mask = false;
    for (size_t k = 2; k < w.size(); k += 2) {
      if (w[k] != "mask" || k + 1 >= w.size()) return fail("Illegal sweep command");
      if (w[k + 1] == "yes") mask = true;
      else if (w[k + 1] == "no") mask = false;
      else return fail("Illegal sweep command");
    }
  } else if (c == "sector") {
    if (!need(2)) return fail("Illegal sector command");
    nsector_user = 0;
    if (w[1] == "yes") sectorflag = 1;
    else if (w[1] == "no") sectorflag = 0;
    else {
      sectorflag = 1;
      if (!parse_int(w[1], &nsector_user) || (nsector_user != 2 && nsector_user != 4 && nsector_user != 8))
        return fail("Illegal sector command");
    }
    nstop = 1.0;
    tstop = 0.0;
    for (size_t k = 2; k < w.size(); k += 2) {
      double v;
      if (k + 1 >= w.size() || !parse_double(w[k + 1], &v) || v <= 0.0) return fail("Illegal sector command");
      if (w[k] == "nstop") {
        nstop = v;
        tstop = 0.0;
      } else if (w[k] == "tstop") {
        tstop = v;
        nstop = 0.0;
      } else {
        return fail("Illegal sector command");
      }
    }
  } else if (c == "temperature") {
    if (w.size() != 2 || !parse_double(w[1], &temperature)) return fail("Illegal temperature command");
  } else if (c == "solve_style") {
    if (app_id < 0) return fail("Solve_style command before app_style set");
    if (!need(2)) return fail("Illegal solve_style command");
    if (w[1] == "tree") {
      tree = true;
      // SolveTree's own RandomPark (src/solve_tree.cpp:25-27): two master draws
      if (master.ready) {
        master.uniform();
        master.uniform();
      }
    } else if (w[1] == "none") {
      tree = false;
    } else {
      return fail("solve_style " + w[1] + " is not on the GPU path (tree)");
    }
  } else if (c == "stats") {
    if (!need(2) || !parse_double(w[1], &stats_delta)) return fail("Illegal stats command");
  } else if (c == "diag_style") {
    return diag_style(w);
  } else if (c == "run") {
    return run(w);
  } else if (c == "dump") {
    return dump_command(w);
  } else if (c == "dump_modify") {
    return dump_modify(w);
  } else if (c == "undump" || c == "dump_one") {
    if (w.size() != 2) return fail("Illegal " + c + " command");
    for (size_t k = 0; k < dumps.size(); k++) {
      if (dumps[k].id != w[1]) continue;
      if (c == "dump_one") return dump_write(dumps[k]);
      if (dumps[k].fp) fclose(dumps[k].fp);
      dumps.erase(dumps.begin() + k);
      return true;
    }
    return fail("Could not find dump ID in " + c + " command");
  } else if (c == "read_sites") {
    if (w.size() != 2) return fail("Illegal read_sites command");
    return read_sites(w[1]);
  } else if (c == "log") {
    // Input::log (src/input.cpp:663-690): a new log file, or none
    if (w.size() != 2) return fail("Illegal log command");
    if (logfile) fclose(logfile);
    logfile = nullptr;
    if (w[1] != "none") {
      logfile = fopen(w[1].c_str(), "w");
      if (!logfile) return fail("Cannot open logfile " + w[1]);
      fprintf(logfile, "SPPARKS (GB300 driver) -- continued logfile from same input script\n");
    }
  } else if (c == "echo" || c == "reset_time" || c == "shell") {
    print("WARNING: %s is ignored by the GPU driver\n", c.c_str());
  } else {
    return fail("Unknown command: " + c);
  }
  return true;
}

std::vector<std::string> split_words(const char *line) {
  std::vector<std::string> w;
  std::string cur;
  for (const char *p = line; *p; p++) {
    if (*p == '#') break;
    if (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r') {
      if (!cur.empty()) w.push_back(cur), cur.clear();
    } else {
      cur += *p;
    }
  }
  if (!cur.empty()) w.push_back(cur);
  return w;
}

}  // namespace

extern "C" {

void spparks_open_no_mpi(int argc, char **argv, void **ptr) {
  Driver *d = new Driver();
  for (int k = 1; k < argc; k++) {
    if (!strcmp(argv[k], "-screen") && k + 1 < argc) {
      k++;
      if (!strcmp(argv[k], "none")) d->screen = nullptr;
      else d->screen = fopen(argv[k], "w");
    } else if (!strcmp(argv[k], "-log") && k + 1 < argc) {
      k++;
      if (strcmp(argv[k], "none")) d->logfile = fopen(argv[k], "w");
    }
  }
  d->print("SPPARKS (GB300 spkgpu driver)\n");
  *ptr = d;
}

void spparks_close(void *ptr) { delete (Driver *)ptr; }

char *spparks_command(void *ptr, char *str) {
  Driver *d = (Driver *)ptr;
  if (!d || !str) return nullptr;
  std::vector<std::string> w = split_words(str);
  if (w.empty()) return str;
  d->error.clear();
  if (!d->command(w)) return nullptr;
  return str;
}

void spparks_file(void *ptr, char *path) {
  Driver *d = (Driver *)ptr;
  FILE *fp = fopen(path, "r");
  if (!fp) {
    d->fail(std::string("Cannot open input script ") + path);
    return;
  }
  char line[4096];
  while (fgets(line, sizeof(line), fp)) {
    d->print("%s", line);
    std::vector<std::string> w = split_words(line);
    if (w.empty()) continue;
    if (!d->command(w)) break;
  }
  fclose(fp);
}

// names of src/app.cpp:163-196 that the GPU driver keeps
void *spparks_extract(void *ptr, char *name) {
  Driver *d = (Driver *)ptr;
  if (!d || !name) return nullptr;
  std::string n = name;
  if (n == "site" || n == "iarray1") {
    if (!d->sites || !d->sync_to_host()) return nullptr;
    // the caller may write into it: it becomes the authoritative copy
    d->device_valid = false;
    return d->site.data();
  }
  if (n == "dimension") return &d->dimension;
  if (n == "nglobal") {
    d->nglobal_store = d->n();
    return &d->nglobal_store;
  }
  if (n == "nlocal") {
    d->nlocal_store = (int)d->n();
    return &d->nlocal_store;
  }
  if (n == "boxxlo") return &d->box_store[0];
  if (n == "boxxhi") return &d->box_store[1];
  if (n == "boxylo") return &d->box_store[2];
  if (n == "boxyhi") return &d->box_store[3];
  if (n == "boxzlo") return &d->box_store[4];
  if (n == "boxzhi") return &d->box_store[5];
  return nullptr;
}

double spparks_energy(void *ptr) {
  Driver *d = (Driver *)ptr;
  if (!d || !d->sites) return 0.0;
  if (d->h && d->device_valid) {
    double e = 0.0;
    if (spkgpu_energy(d->h, &e) == 0) return e;
  }
  if (!d->ensure_handle()) return 0.0;
  if (spkgpu_upload_spins(d->h, d->site.data(), d->n()) != 0) return 0.0;
  d->device_valid = true;
  double e = 0.0;
  spkgpu_energy(d->h, &e);
  return e;
}

const char *spkgpu_driver_error(void *ptr) {
  Driver *d = (Driver *)ptr;
  return d ? d->error.c_str() : "null handle";
}

double spkgpu_driver_time(void *ptr) {
  Driver *d = (Driver *)ptr;
  return d ? d->time : 0.0;
}

}  // extern "C"
