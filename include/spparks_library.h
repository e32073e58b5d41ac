/* The reference's library interface (src/library.h:27-36, bound by
   python/spparks.py:20-95), exported by libspkgpu.so over the GB300 input
   script driver (spparks_gb300/csrc/driver.cpp).  Same names, arguments and
   meaning as the reference, except that an error prints "ERROR: ..." and
   returns (spparks_command returns NULL) instead of terminating the process;
   spkgpu_driver_error returns the message.  spparks_open (with an MPI
   communicator) is not provided: the GPU path is one process on one GPU. */
#ifndef SPKGPU_SPPARKS_LIBRARY_H
#define SPKGPU_SPPARKS_LIBRARY_H

#ifdef __cplusplus
extern "C" {
#endif

/* src/library.h:31 spparks_open_no_mpi: -screen FILE|none, -log FILE|none */
void spparks_open_no_mpi(int argc, char **argv, void **ptr);
/* src/library.h:32 */
void spparks_close(void *ptr);
/* src/library.h:33: run every command of an input script */
void spparks_file(void *ptr, char *path);
/* src/library.h:34: one command; returns str, or NULL on error */
char *spparks_command(void *ptr, char *str);
/* src/library.h:36 / src/app.cpp:163-196: "site" (int*, writable, taken as
   the current values by the next run), "nlocal", "dimension" (int*),
   "nglobal" (int64*), "boxxlo".."boxzhi" (double*) */
void *spparks_extract(void *ptr, char *name);
/* src/library.h:37 / src/library.cpp:118-147: sum of site energies */
double spparks_energy(void *ptr);

/* GB300 driver additions (no counterpart in the reference) */
const char *spkgpu_driver_error(void *ptr);  /* message of the last error */
double spkgpu_driver_time(void *ptr);        /* simulated time */

#ifdef __cplusplus
}
#endif
#endif
