/* Oracle (test infrastructure only): drives the reference build through its
   own library interface (src/library.h: spparks_open_no_mpi, spparks_command,
   spparks_extract, spparks_energy, spparks_close) and prints what the parity
   fixtures need.

   usage: ref_runner SCRIPT
   SCRIPT holds reference input commands, one per line, plus directives:
     #! seed S          Philox key for the shim build and for init_spins
     #! stream B        stream word base of the sweep draws (shim build;
                        replica r of an ensemble uses (r+1) << 8)
     #! init_spins LO HI  overwrite site values with Philox initial spins
     #! record on|off   per-sweep records (shim build only)
     #! snap TAG        print the hash and all site values
     #! energy          print spparks_energy (only after a run)
     #! timed TAG CMD   run the input command CMD and print its wall time
     #! appstats        print the app's stats line (App::stats: time,
                        Naccept, Nreject, Nsweeps)
   Output lines:
     sweep N NACCEPT NATTEMPT HASH TIME
     snap TAG HASH NLOCAL v1 v2 ...
     energy E
     timed TAG SECONDS
     appstats TIME NACCEPT NREJECT NSWEEPS
*/

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <stdint.h>
#include <time.h>

#include "app.h"
#include "library.h"
#include "spparks.h"
#include "../philox_oracle.h"

#ifdef SPK_SHIM
#include "oracle_apps.h"
#include "shim_ctx.h"
#endif

static uint64_t fnv_spins(const int *spin, int n) {
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

#ifdef SPK_SHIM
static void flush_records() {
  for (size_t k = 0; k < spk_oracle::records.size(); k++) {
    const spk_oracle::SweepRecord &r = spk_oracle::records[k];
    printf("sweep %d %lld %lld %016llx %.17g\n", r.sweep, r.naccept, r.nattempt,
           (unsigned long long)r.hash, r.time);
  }
  spk_oracle::records.clear();
}
#else
static void flush_records() {}
#endif

int main(int argc, char **argv) {
  if (argc != 2) {
    fprintf(stderr, "usage: ref_runner SCRIPT\n");
    return 2;
  }
  FILE *fp = fopen(argv[1], "r");
  if (!fp) {
    fprintf(stderr, "cannot open %s\n", argv[1]);
    return 2;
  }
  char *spk_argv[] = {(char *)"ref_runner", (char *)"-screen", (char *)"none",
                      (char *)"-log", (char *)"none"};
  void *spk = NULL;
  spparks_open_no_mpi(5, spk_argv, &spk);

  uint32_t seed = 12345;
  char line[4096];
  while (fgets(line, sizeof(line), fp)) {
    size_t len = strlen(line);
    while (len && (line[len - 1] == '\n' || line[len - 1] == '\r')) line[--len] = 0;
    if (strncmp(line, "#!", 2) == 0) {
      char cmd[64] = {0}, a1[256] = {0}, a2[256] = {0};
      int n = sscanf(line + 2, "%63s %255s %255s", cmd, a1, a2);
      if (n < 1) continue;
      if (!strcmp(cmd, "seed")) {
        seed = (uint32_t)strtoul(a1, NULL, 10);
#ifdef SPK_SHIM
        spk_shim::philox_seed = seed;
#endif
      } else if (!strcmp(cmd, "stream")) {
#ifdef SPK_SHIM
        spk_shim::stream_base = (uint32_t)strtoul(a1, NULL, 10);
#endif
      } else if (!strcmp(cmd, "init_spins")) {
        int lo = atoi(a1), hi = atoi(a2);
        int nlocal = *(int *)spparks_extract(spk, (char *)"nlocal");
        int *site = (int *)spparks_extract(spk, (char *)"site");
        int *id32 = (int *)spparks_extract(spk, (char *)"id");
        for (int i = 0; i < nlocal; i++)
          site[i] = spko_init_spin(seed, (uint64_t)(id32[i] - 1), lo, hi);
      } else if (!strcmp(cmd, "energy")) {
        // valid only after a run: spparks_energy needs the app's comm set up
        printf("energy %.17g\n", spparks_energy(spk));
      } else if (!strcmp(cmd, "timed")) {
        // the command is the rest of the line after the tag
        const char *rest = strstr(line + 2, a1) + strlen(a1);
        while (*rest == ' ') rest++;
        char buf[4096];
        snprintf(buf, sizeof(buf), "%s", rest);
        timespec t0, t1;
        clock_gettime(CLOCK_MONOTONIC, &t0);
        spparks_command(spk, buf);
        clock_gettime(CLOCK_MONOTONIC, &t1);
        flush_records();
        printf("timed %s %.9f\n", a1, (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec));
        fflush(stdout);
      } else if (!strcmp(cmd, "appstats")) {
        char buf[512];
        ((SPPARKS_NS::SPPARKS *)spk)->app->stats(buf);
        printf("appstats %s\n", buf);
        fflush(stdout);
      } else if (!strcmp(cmd, "record")) {
#ifdef SPK_SHIM
        spk_oracle::record_on = !strcmp(a1, "on");
#endif
      } else if (!strcmp(cmd, "snap")) {
        flush_records();
        int nlocal = *(int *)spparks_extract(spk, (char *)"nlocal");
        int *site = (int *)spparks_extract(spk, (char *)"site");
        printf("snap %s %016llx %d", a1, (unsigned long long)fnv_spins(site, nlocal), nlocal);
        for (int i = 0; i < nlocal; i++) printf(" %d", site[i]);
        printf("\n");
      } else {
        fprintf(stderr, "unknown directive %s\n", cmd);
        return 2;
      }
      continue;
    }
    if (len == 0 || line[0] == '#') continue;
    spparks_command(spk, line);
    flush_records();
  }
  fclose(fp);
  flush_records();
  spparks_close(spk);
  return 0;
}
