"""spparks_gb300: GB300-native (sm_103a) on-lattice Monte Carlo hot path of SPPARKS.

Python binding (ctypes) over the C ABI in ``include/spkgpu.h``.  Two levels:

* :class:`Lattice` - one lattice on the GPU: the calls a host ``AppLattice``
  subclass makes (upload site values, set the temperature, sweep, KMC run,
  download, energy).
* :class:`SPPARKS` - the reference's library interface (``spparks_open_no_mpi``,
  ``spparks_command``, ``spparks_file``, ``spparks_extract``, ``spparks_energy``,
  ``spparks_close``; src/library.h, python/spparks.py) over the repo's own
  input-script driver, so a script written for the reference's ``sweep color``
  or ``solve_style tree`` path runs unchanged on the GPU.

There is no CPU fallback: if ``_lib/libspkgpu.so`` is missing or no GPU is
present the calls raise.
"""

from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_lib" / "libspkgpu.so"

SQ_4N, SQ_8N, SC_6N, SC_26N = 0, 1, 2, 3
ISING, POTTS, POTTS_NEIGHONLY, POTTS_NEIGH = 0, 1, 2, 3
RNG_PHILOX, RNG_STRICT = 0, 1
LATTICE_STYLES = {"sq/4n": SQ_4N, "sq/8n": SQ_8N, "sc/6n": SC_6N, "sc/26n": SC_26N}
APP_STYLES = {"ising": ISING, "potts": POTTS, "potts/neighonly": POTTS_NEIGHONLY, "potts/neigh": POTTS_NEIGH}

ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "invalid state", -4: "out of device memory",
          -5: "unsupported", -6: "invalid site value", -7: "device wait gave up", -8: "too large"}


class SpkGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"spkgpu error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


class Desc(ctypes.Structure):
    _fields_ = [
        ("lattice", ctypes.c_int32),
        ("nx", ctypes.c_int32),
        ("ny", ctypes.c_int32),
        ("nz", ctypes.c_int32),
        ("app", ctypes.c_int32),
        ("nspins", ctypes.c_int32),
        ("spin_bytes", ctypes.c_int32),
        ("nsector", ctypes.c_int32),
        ("nloop", ctypes.c_int32),
        ("procs", ctypes.c_int32 * 3),
        ("rng", ctypes.c_int32),
        ("mask", ctypes.c_int32),
        ("seed", ctypes.c_uint32),
        ("device", ctypes.c_int32),
        ("variant", ctypes.c_int32),
    ]


class Stats(ctypes.Structure):
    _fields_ = [("naccept", ctypes.c_int64), ("nattempt", ctypes.c_int64), ("nsweeps", ctypes.c_int64)]


class KmcStats(ctypes.Structure):
    _fields_ = [("time", ctypes.c_double), ("naccept", ctypes.c_int64), ("npass", ctypes.c_int64),
                ("dt_kmc", ctypes.c_double), ("total_propensity", ctypes.c_double),
                ("prop_rel_err", ctypes.c_double), ("dt_rel_err", ctypes.c_double)]


# execution forms of an ensemble, in the order of SPKGPU_ENSEMBLE_* (spkgpu.h);
# "warps" (one tile per warp) exists for Ising only
ENSEMBLE_MODES = ("persistent", "launches", "launches2", "launches4", "warps", "warps2", "warps4")


class EnsembleDesc(ctypes.Structure):
    _fields_ = [
        ("nreplica", ctypes.c_int32),
        ("L", ctypes.POINTER(ctypes.c_int32)),
        ("temperature", ctypes.POINTER(ctypes.c_double)),
        ("app", ctypes.c_int32),
        ("nspins", ctypes.c_int32),
        ("seed", ctypes.c_uint32),
        ("exchange_every", ctypes.c_int32),
        ("device", ctypes.c_int32),
    ]


class EnsembleStats(ctypes.Structure):
    _fields_ = [("naccept", ctypes.c_int64), ("nattempt", ctypes.c_int64), ("nsweeps", ctypes.c_int64),
                ("exchange_tries", ctypes.c_int64), ("exchange_accepts", ctypes.c_int64)]


# every symbol include/spkgpu.h (and the other include/*.h) declares
EXPORTS = [
    "spkgpu_create", "spkgpu_destroy", "spkgpu_last_error", "spkgpu_version", "spkgpu_set_temperature",
    "spkgpu_upload_spins", "spkgpu_download_spins", "spkgpu_init_spins", "spkgpu_upload_siteseeds", "spkgpu_download_siteseeds",
    "spkgpu_upload_mask", "spkgpu_download_mask", "spkgpu_sweep", "spkgpu_set_sweep_index",
    "spkgpu_get_stats", "spkgpu_energy", "spkgpu_site_stats", "spkgpu_clusters", "spkgpu_synchronize", "spkgpu_timed_sweeps", "spkgpu_stream",
    "spkgpu_device_spins", "spkgpu_launch_count", "spkgpu_kmc_setup", "spkgpu_kmc_run", "spkgpu_kmc_run_until",
    "spkgpu_ensemble_create", "spkgpu_ensemble_destroy", "spkgpu_ensemble_last_error", "spkgpu_ensemble_upload",
    "spkgpu_ensemble_download", "spkgpu_ensemble_run", "spkgpu_ensemble_timed_run", "spkgpu_ensemble_synchronize",
    "spkgpu_ensemble_run_io",
    "spkgpu_ensemble_get_stats", "spkgpu_ensemble_temperatures", "spkgpu_ensemble_energies",
    "spkgpu_ensemble_launch_count", "spkgpu_ensemble_mode", "spkgpu_ensemble_sweep_kernel_ms",
    "spkgpu_sweep_sq4_noalloc", "spkgpu_philox_rate",
    "spparks_open_no_mpi", "spparks_close", "spparks_file", "spparks_command", "spparks_extract", "spparks_energy",
    "spkgpu_driver_error", "spkgpu_driver_time",
]

_lib = None


def load_library(path: Path | None = None):
    """Load libspkgpu.so; raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise SpkGpuError(-3, f"{p} is missing: build it with `python -m spparks_gb300.build`")
    L = ctypes.CDLL(str(p))
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    L.spkgpu_create.argtypes = [P(Desc), P(vp)]
    L.spkgpu_destroy.argtypes = [vp]
    L.spkgpu_last_error.argtypes = [vp]
    L.spkgpu_last_error.restype = ctypes.c_char_p
    L.spkgpu_set_temperature.argtypes = [vp, ctypes.c_double]
    L.spkgpu_init_spins.argtypes = [vp, ctypes.c_int32, ctypes.c_int32]
    for name in ("spkgpu_upload_spins", "spkgpu_download_spins", "spkgpu_upload_siteseeds",
                 "spkgpu_download_siteseeds"):
        getattr(L, name).argtypes = [vp, P(ctypes.c_int32), ctypes.c_int64]
    for name in ("spkgpu_upload_mask", "spkgpu_download_mask"):
        getattr(L, name).argtypes = [vp, P(ctypes.c_uint8), ctypes.c_int64]
    L.spkgpu_sweep.argtypes = [vp, ctypes.c_int32]
    L.spkgpu_set_sweep_index.argtypes = [vp, ctypes.c_int64]
    L.spkgpu_get_stats.argtypes = [vp, P(Stats)]
    L.spkgpu_energy.argtypes = [vp, P(ctypes.c_double)]
    L.spkgpu_site_stats.argtypes = [vp, P(ctypes.c_int64), P(ctypes.c_int32), P(ctypes.c_int32)]
    L.spkgpu_clusters.argtypes = [vp, P(ctypes.c_int64), P(ctypes.c_double), P(ctypes.c_double)]
    L.spkgpu_synchronize.argtypes = [vp]
    L.spkgpu_timed_sweeps.argtypes = [vp, ctypes.c_int32, P(ctypes.c_float)]
    L.spkgpu_stream.argtypes = [vp, P(vp)]
    L.spkgpu_device_spins.argtypes = [vp, P(vp), P(ctypes.c_int64)]
    L.spkgpu_launch_count.argtypes = [vp, P(ctypes.c_int64)]
    L.spkgpu_kmc_setup.argtypes = [vp, ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_int32]
    L.spkgpu_kmc_run.argtypes = [vp, P(ctypes.c_double), ctypes.c_double, P(KmcStats)]
    L.spkgpu_kmc_run_until.argtypes = [vp, P(ctypes.c_double), ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                       P(KmcStats)]
    L.spkgpu_ensemble_create.argtypes = [P(EnsembleDesc), P(vp)]
    L.spkgpu_ensemble_destroy.argtypes = [vp]
    L.spkgpu_ensemble_last_error.argtypes = [vp]
    L.spkgpu_ensemble_last_error.restype = ctypes.c_char_p
    L.spkgpu_ensemble_upload.argtypes = [vp, P(ctypes.c_int32), ctypes.c_int64]
    L.spkgpu_ensemble_download.argtypes = [vp, P(ctypes.c_int32), ctypes.c_int64]
    L.spkgpu_ensemble_run.argtypes = [vp, ctypes.c_int32]
    L.spkgpu_ensemble_run_io.argtypes = [vp, P(ctypes.c_int32), P(ctypes.c_int32), ctypes.c_int32]
    L.spkgpu_ensemble_timed_run.argtypes = [vp, ctypes.c_int32, P(ctypes.c_float)]
    L.spkgpu_ensemble_synchronize.argtypes = [vp]
    L.spkgpu_ensemble_get_stats.argtypes = [vp, P(EnsembleStats)]
    L.spkgpu_ensemble_temperatures.argtypes = [vp, P(ctypes.c_double)]
    L.spkgpu_ensemble_energies.argtypes = [vp, P(ctypes.c_int64)]
    L.spkgpu_ensemble_launch_count.argtypes = [vp, P(ctypes.c_int64)]
    L.spkgpu_ensemble_mode.argtypes = [vp, P(ctypes.c_int32), P(ctypes.c_float)]
    L.spkgpu_ensemble_sweep_kernel_ms.argtypes = [vp, P(ctypes.c_float), P(ctypes.c_int32)]
    L.spkgpu_sweep_sq4_noalloc.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                           ctypes.c_int32, ctypes.c_double, ctypes.c_uint32, ctypes.c_int64,
                                           ctypes.c_int32, vp, P(ctypes.c_int64)]
    L.spkgpu_philox_rate.argtypes = [ctypes.c_int32, ctypes.c_int32, P(ctypes.c_double)]
    if path is None:
        _lib = L
    return L


def philox_rate(device: int = 0, iters: int = 4096) -> float:
    """Philox4x32-10 blocks/s of the device with the sweeps' own code
    (spkgpu_philox_rate): a quarter of the draw-side ceiling of an Ising
    sweep (four sites per block), half that of the other apps."""
    lib = load_library()
    v = ctypes.c_double()
    rc = lib.spkgpu_philox_rate(int(device), int(iters), ctypes.byref(v))
    if rc != 0:
        raise SpkGpuError(rc, "spkgpu_philox_rate failed")
    return v.value


def _i32p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


class Lattice:
    """One lattice on the GPU behind the C ABI."""

    def __init__(self, lattice="sq/4n", nx=16, ny=16, nz=1, app="ising", nspins=2, spin_bytes=0, nsector=1,
                 nloop=1, procs=(1, 1, 1), rng=RNG_PHILOX, mask=False, seed=12345, device=0, variant=0):
        self.lib = load_library()
        d = Desc()
        d.lattice = LATTICE_STYLES[lattice] if isinstance(lattice, str) else int(lattice)
        d.nx, d.ny, d.nz = nx, ny, nz
        d.app = APP_STYLES[app] if isinstance(app, str) else int(app)
        d.nspins = nspins
        d.spin_bytes = spin_bytes
        d.nsector = nsector
        d.nloop = nloop
        d.procs[0], d.procs[1], d.procs[2] = procs
        d.rng = rng
        d.mask = int(bool(mask))
        d.seed = seed & 0xFFFFFFFF
        d.device = device
        d.variant = variant
        self.desc = d
        self.n = nx * ny * nz
        self.h = ctypes.c_void_p()
        rc = self.lib.spkgpu_create(ctypes.byref(d), ctypes.byref(self.h))
        if rc != 0:
            self.h = None
            raise SpkGpuError(rc, "spkgpu_create rejected the lattice description")

    def _check(self, rc):
        if rc != 0:
            raise SpkGpuError(rc, self.lib.spkgpu_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.lib.spkgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_temperature(self, t: float):
        self._check(self.lib.spkgpu_set_temperature(self.h, float(t)))

    def upload(self, spin: np.ndarray):
        s = np.ascontiguousarray(spin, dtype=np.int32)
        self._check(self.lib.spkgpu_upload_spins(self.h, _i32p(s), s.size))

    def init_spins(self, lo: int = 1, hi: int | None = None):
        """Seeded values lo..hi generated on the device (Philox init stream)."""
        self._check(self.lib.spkgpu_init_spins(self.h, int(lo), int(self.desc.nspins if hi is None else hi)))

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        out = np.empty(self.n, dtype=np.int32) if out is None else out
        self._check(self.lib.spkgpu_download_spins(self.h, _i32p(out), out.size))
        return out

    def upload_siteseeds(self, seeds: np.ndarray):
        s = np.ascontiguousarray(seeds, dtype=np.int32)
        self._check(self.lib.spkgpu_upload_siteseeds(self.h, _i32p(s), s.size))

    def download_siteseeds(self) -> np.ndarray:
        out = np.empty(self.n, dtype=np.int32)
        self._check(self.lib.spkgpu_download_siteseeds(self.h, _i32p(out), out.size))
        return out

    def upload_mask(self, mask: np.ndarray):
        m = np.ascontiguousarray(mask, dtype=np.uint8)
        self._check(self.lib.spkgpu_upload_mask(self.h, m.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), m.size))

    def download_mask(self) -> np.ndarray:
        out = np.empty(self.n, dtype=np.uint8)
        self._check(self.lib.spkgpu_download_mask(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                                  out.size))
        return out

    def sweep(self, nsweeps: int = 1):
        self._check(self.lib.spkgpu_sweep(self.h, int(nsweeps)))

    def set_sweep_index(self, sweep: int):
        self._check(self.lib.spkgpu_set_sweep_index(self.h, int(sweep)))

    def timed_sweeps(self, nsweeps: int) -> float:
        ms = ctypes.c_float()
        self._check(self.lib.spkgpu_timed_sweeps(self.h, int(nsweeps), ctypes.byref(ms)))
        return ms.value

    def stats(self) -> dict:
        s = Stats()
        self._check(self.lib.spkgpu_get_stats(self.h, ctypes.byref(s)))
        return {"naccept": s.naccept, "nattempt": s.nattempt, "nsweeps": s.nsweeps}

    def energy(self) -> float:
        e = ctypes.c_double()
        self._check(self.lib.spkgpu_energy(self.h, ctypes.byref(e)))
        return e.value

    def site_stats(self) -> dict:
        """sum, min, max and mean of the site values (diag_style array i1)."""
        s, lo, hi = ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32()
        self._check(self.lib.spkgpu_site_stats(self.h, ctypes.byref(s), ctypes.byref(lo), ctypes.byref(hi)))
        return {"sum": s.value, "min": lo.value, "max": hi.value, "mean": s.value / self.n}

    def clusters(self) -> dict:
        """diag_style cluster: number of clusters, <N> and <R>."""
        nc, vav, rav = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.spkgpu_clusters(self.h, ctypes.byref(nc), ctypes.byref(vav), ctypes.byref(rav)))
        return {"ncluster": nc.value, "mean_volume": vav.value, "mean_radius": rav.value}

    def synchronize(self):
        self._check(self.lib.spkgpu_synchronize(self.h))

    def launch_count(self) -> int:
        c = ctypes.c_int64()
        self._check(self.lib.spkgpu_launch_count(self.h, ctypes.byref(c)))
        return c.value

    def kmc_setup(self, adapt=True, nstop=1.0, tstop=0.0, fp64=True, shadow=True):
        """fp64: FP64 propensities (bit-exact); else FP32 propensities, with the
        all-FP64 shadow of the per-chain sums when `shadow`."""
        mode = 1 if fp64 else (0 if shadow else 2)
        self._check(self.lib.spkgpu_kmc_setup(self.h, int(bool(adapt)), float(nstop), float(tstop), mode))

    def kmc_run(self, time: float, stoptime: float, until: float | None = None, first: bool = True) -> dict:
        """one KMC run from `time` to `stoptime`; with `until`, only the passes
        up to that output time (continue with first=False)."""
        t = ctypes.c_double(time)
        s = KmcStats()
        if until is None:
            self._check(self.lib.spkgpu_kmc_run(self.h, ctypes.byref(t), float(stoptime), ctypes.byref(s)))
        else:
            self._check(self.lib.spkgpu_kmc_run_until(self.h, ctypes.byref(t), float(stoptime), float(until),
                                                      int(bool(first)), ctypes.byref(s)))
        return {"time": s.time, "naccept": s.naccept, "npass": s.npass, "dt_kmc": s.dt_kmc,
                "total_propensity": s.total_propensity, "prop_rel_err": s.prop_rel_err,
                "dt_rel_err": s.dt_rel_err}


class Ensemble:
    """Batched sq/4n replicas of uneven size and temperature with on-device
    replica exchange (spkgpu_ensemble_* in include/spkgpu.h)."""

    def __init__(self, L, temperature, app="ising", nspins=2, seed=12345, exchange_every=10, device=0):
        self.lib = load_library()
        self.L = np.ascontiguousarray(L, dtype=np.int32)
        self.T = np.ascontiguousarray(temperature, dtype=np.float64)
        d = EnsembleDesc()
        d.nreplica = len(self.L)
        d.L = self.L.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        d.temperature = self.T.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.app = APP_STYLES[app] if isinstance(app, str) else int(app)
        d.nspins = nspins
        d.seed = seed & 0xFFFFFFFF
        d.exchange_every = exchange_every
        d.device = device
        self.nsites = int(np.sum(self.L.astype(np.int64) ** 2))
        self.offsets = np.concatenate([[0], np.cumsum(self.L.astype(np.int64) ** 2)])
        self.h = ctypes.c_void_p()
        rc = self.lib.spkgpu_ensemble_create(ctypes.byref(d), ctypes.byref(self.h))
        if rc != 0:
            self.h = None
            raise SpkGpuError(rc, "spkgpu_ensemble_create rejected the ensemble description")

    def _check(self, rc):
        if rc != 0:
            raise SpkGpuError(rc, self.lib.spkgpu_ensemble_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.lib.spkgpu_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, spin):
        s = np.ascontiguousarray(spin, dtype=np.int32)
        self._check(self.lib.spkgpu_ensemble_upload(self.h, _i32p(s), s.size))

    def download(self, out=None):
        out = np.empty(self.nsites, dtype=np.int32) if out is None else out
        self._check(self.lib.spkgpu_ensemble_download(self.h, _i32p(out), out.size))
        return out

    def replica(self, spin, r):
        return spin[self.offsets[r]:self.offsets[r + 1]]

    def run(self, nsweeps):
        self._check(self.lib.spkgpu_ensemble_run(self.h, int(nsweeps)))

    def run_io(self, spin_in: np.ndarray, spin_out: np.ndarray, nsweeps):
        """Enqueue one step: load spin_in, run nsweeps sweeps, store into
        spin_out (both int32, every site; page-locked memory makes
        successive steps overlap).  Neither array may change until
        synchronize() returns, which also reports invalid input values."""
        for a in (spin_in, spin_out):
            if a.dtype != np.int32 or not a.flags["C_CONTIGUOUS"] or a.size != self.nsites:
                raise ValueError("run_io wants contiguous int32 arrays of every site")
        self._check(self.lib.spkgpu_ensemble_run_io(self.h, _i32p(spin_in), _i32p(spin_out), int(nsweeps)))

    def timed_run(self, nsweeps) -> float:
        ms = ctypes.c_float()
        self._check(self.lib.spkgpu_ensemble_timed_run(self.h, int(nsweeps), ctypes.byref(ms)))
        return ms.value

    def synchronize(self):
        self._check(self.lib.spkgpu_ensemble_synchronize(self.h))

    def stats(self) -> dict:
        s = EnsembleStats()
        self._check(self.lib.spkgpu_ensemble_get_stats(self.h, ctypes.byref(s)))
        return {"naccept": s.naccept, "nattempt": s.nattempt, "nsweeps": s.nsweeps,
                "exchange_tries": s.exchange_tries, "exchange_accepts": s.exchange_accepts}

    def mode(self) -> dict:
        """Execution form the autotuner kept (one of ENSEMBLE_MODES) and its
        time of one step in each form (ms, None where not timed)."""
        m = ctypes.c_int32()
        names = ENSEMBLE_MODES
        ms = (ctypes.c_float * len(names))()
        self._check(self.lib.spkgpu_ensemble_mode(self.h, ctypes.byref(m), ms))
        return {"mode": names[m.value],
                "tune_ms": {names[k]: (float(ms[k]) if ms[k] >= 0 else None) for k in range(len(names))}}

    def sweep_kernel_ms(self):
        """(ms, launches): device time of the sweep kernels in the last replay
        of the captured step, and how many launches that time covers."""
        ms, n = ctypes.c_float(), ctypes.c_int32()
        self._check(self.lib.spkgpu_ensemble_sweep_kernel_ms(self.h, ctypes.byref(ms), ctypes.byref(n)))
        return float(ms.value), int(n.value)

    def temperatures(self) -> np.ndarray:
        out = np.empty(len(self.L), dtype=np.float64)
        self._check(self.lib.spkgpu_ensemble_temperatures(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out

    def energies(self) -> np.ndarray:
        out = np.empty(len(self.L), dtype=np.int64)
        self._check(self.lib.spkgpu_ensemble_energies(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        return out

    def launch_count(self) -> int:
        c = ctypes.c_int64()
        self._check(self.lib.spkgpu_ensemble_launch_count(self.h, ctypes.byref(c)))
        return c.value


class SPPARKS:
    """The reference's Python wrapper interface (python/spparks.py: command,
    file, extract, energy, close) over libspkgpu.so's input-script driver.

    ``extract(name, type)`` follows the reference's type codes: 0 = int
    scalar, 1 = int vector, 3 = double scalar (``extract("site", 1)`` returns a
    writable ctypes int pointer to the site values; writes are taken as the
    current values by the next ``run``)."""

    def __init__(self, name="", cmdargs=None):
        self.lib = load_library()
        self.lib.spparks_open_no_mpi.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                                 ctypes.POINTER(ctypes.c_void_p)]
        self.lib.spparks_close.argtypes = [ctypes.c_void_p]
        self.lib.spparks_file.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        self.lib.spparks_command.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        self.lib.spparks_command.restype = ctypes.c_char_p
        self.lib.spparks_extract.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        self.lib.spparks_extract.restype = ctypes.c_void_p
        self.lib.spparks_energy.argtypes = [ctypes.c_void_p]
        self.lib.spparks_energy.restype = ctypes.c_double
        self.lib.spkgpu_driver_error.argtypes = [ctypes.c_void_p]
        self.lib.spkgpu_driver_error.restype = ctypes.c_char_p
        self.lib.spkgpu_driver_time.argtypes = [ctypes.c_void_p]
        self.lib.spkgpu_driver_time.restype = ctypes.c_double
        args = ["spparks.py"] + list(cmdargs or [])
        cargs = (ctypes.c_char_p * len(args))(*[a.encode() for a in args])
        self.spk = ctypes.c_void_p()
        self.lib.spparks_open_no_mpi(len(args), cargs, ctypes.byref(self.spk))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def close(self):
        if getattr(self, "spk", None):
            self.lib.spparks_close(self.spk)
            self.spk = None

    def file(self, path):
        self.lib.spparks_file(self.spk, str(path).encode())

    def command(self, cmd):
        r = self.lib.spparks_command(self.spk, cmd.encode())
        if r is None:
            raise SpkGpuError(-1, self.lib.spkgpu_driver_error(self.spk).decode())
        return r.decode()

    def extract(self, name, type):
        p = self.lib.spparks_extract(self.spk, name.encode())
        if not p:
            return None
        if type == 0:
            return ctypes.cast(p, ctypes.POINTER(ctypes.c_int))[0]
        if type == 1:
            return ctypes.cast(p, ctypes.POINTER(ctypes.c_int))
        if type == 3:
            return ctypes.cast(p, ctypes.POINTER(ctypes.c_double))[0]
        if type == 4:
            return ctypes.cast(p, ctypes.POINTER(ctypes.c_double))
        return None

    def sites(self) -> np.ndarray:
        """Copy of the site values (iarray[0])."""
        n = self.extract("nlocal", 0)
        ptr = self.extract("site", 1)
        return np.ctypeslib.as_array(ptr, shape=(n,)).copy()

    def set_sites(self, values):
        n = self.extract("nlocal", 0)
        ptr = self.extract("site", 1)
        np.ctypeslib.as_array(ptr, shape=(n,))[:] = np.asarray(values, dtype=np.int32)

    def energy(self):
        return self.lib.spparks_energy(self.spk)

    def time(self):
        return self.lib.spkgpu_driver_time(self.spk)
