"""Oracle (test infrastructure only).

ctypes binding of the plain-C restatement in ``oracle/spk_oracle.c`` and the
recipe that builds it.  Only the tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this package; the product path
(``spparks_gb300``) never does.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libspkoracle.so"

LATTICES = {"sq/4n": 0, "sq/8n": 1, "sc/6n": 2, "sc/26n": 3}
APPS = {"ising": 0, "potts": 1, "potts/neighonly": 2, "potts/neigh": 3}
RNG_PHILOX, RNG_STRICT = 0, 1


def build(force: bool = False) -> Path:
    """Compile the oracle restatement into ``oracle/_build``."""
    src = HERE / "spk_oracle.c"
    deps = [src, HERE / "spk_oracle.h", HERE / "philox_oracle.h"]
    if not force and LIB.exists() and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB
    BUILD.mkdir(exist_ok=True)
    tmp = BUILD / f"libspkoracle.{os.getpid()}.so"
    subprocess.check_call(["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-o", str(tmp), str(src), "-lm"])
    os.replace(tmp, LIB)
    return LIB


REF_OUT = HERE / "_ref"
REF_STAGE = REF_OUT / "src"


def build_reference(jobs: int = 0) -> bool:
    """Build the reference (and its Philox-shim variant) into ``oracle/_ref``.

    Where the reference tree exists, its sources are also staged into
    ``oracle/_ref/src`` (git-ignored); where it does not (the GPU host), the
    same recipe builds from that staged copy, natively for the host CPU.
    Returns False when neither is present."""
    jobs = jobs or max(2, os.cpu_count() or 2)
    ref = os.environ.get("SPK_REFERENCE_SRC", "/root/reference/src")
    make = ["make", "-s", "-C", str(HERE / "ref"), f"-j{jobs}"]
    if Path(ref, "app_lattice.cpp").exists():
        subprocess.check_call(make + ["stage", f"REF={ref}"])
    elif Path(REF_STAGE, "app_lattice.cpp").exists():
        ref = str(REF_STAGE)
    else:
        return False
    subprocess.check_call(make + [f"REF={ref}"])
    return True


def build_reference_gpu(jobs: int = 0) -> bool:
    """Build oracle/_ref/spk_serial_gpu: the reference with the GPU app
    styles of spparks_gb300/reference_app linked to libspkgpu.so (the
    library must be built).  Returns False where no reference sources are."""
    jobs = jobs or max(2, os.cpu_count() or 2)
    ref = os.environ.get("SPK_REFERENCE_SRC", "/root/reference/src")
    if not Path(ref, "app_lattice.cpp").exists():
        if not Path(REF_STAGE, "app_lattice.cpp").exists():
            return False
        ref = str(REF_STAGE)
    subprocess.check_call(["make", "-s", "-C", str(HERE / "ref"), f"-j{jobs}", f"REF={ref}", "gpu"])
    return True


def reference_binary(name: str = "runner_plain"):
    """Path of a reference binary built by build_reference, or None."""
    p = REF_OUT / name
    return p if p.exists() and os.access(p, os.X_OK) else None


class Cfg(ctypes.Structure):
    _fields_ = [
        ("lattice", ctypes.c_int),
        ("nx", ctypes.c_int),
        ("ny", ctypes.c_int),
        ("nz", ctypes.c_int),
        ("app", ctypes.c_int),
        ("nspins", ctypes.c_int),
        ("temperature", ctypes.c_double),
        ("nsector", ctypes.c_int),
        ("nloop", ctypes.c_int),
        ("rng", ctypes.c_int),
        ("seed", ctypes.c_uint32),
        ("mask", ctypes.c_int),
        ("px", ctypes.c_int),
        ("py", ctypes.c_int),
        ("pz", ctypes.c_int),
        ("stream_base", ctypes.c_uint32),
    ]


class RanMars(ctypes.Structure):
    _fields_ = [
        ("u", ctypes.c_double * 98),
        ("c", ctypes.c_double),
        ("cd", ctypes.c_double),
        ("cm", ctypes.c_double),
        ("i97", ctypes.c_int),
        ("j97", ctypes.c_int),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB))
        P = ctypes.POINTER
        i32p, i64p, u64p, u8p, dblp = (P(ctypes.c_int32), P(ctypes.c_int64), P(ctypes.c_uint64),
                                       P(ctypes.c_uint8), P(ctypes.c_double))
        L.spko_philox.argtypes = [P(ctypes.c_uint32), P(ctypes.c_uint32), P(ctypes.c_uint32)]
        L.spko_neighbors.argtypes = [P(Cfg), ctypes.c_int64, i64p]
        L.spko_neighbors.restype = ctypes.c_int
        L.spko_maxneigh.argtypes = [ctypes.c_int]
        L.spko_maxneigh.restype = ctypes.c_int
        L.spko_color.argtypes = [P(Cfg), ctypes.c_int64]
        L.spko_sector.argtypes = [P(Cfg), ctypes.c_int64]
        L.spko_energy.argtypes = [P(Cfg), i32p]
        L.spko_energy.restype = ctypes.c_double
        L.spko_clusters.argtypes = [P(Cfg), i32p, P(ctypes.c_int64), P(ctypes.c_double), P(ctypes.c_double)]
        L.spko_clusters.restype = ctypes.c_int
        L.spko_hash.argtypes = [i32p, ctypes.c_int64]
        L.spko_hash.restype = ctypes.c_uint64
        L.spko_init_spins.argtypes = [ctypes.c_uint32, ctypes.c_int64, ctypes.c_int, ctypes.c_int, i32p]
        L.spko_color_sweeps.argtypes = [P(Cfg), i32p, ctypes.c_int64, ctypes.c_int, i64p, i64p, u64p,
                                        i32p, u8p]
        L.spko_color_sweeps.restype = ctypes.c_int
        L.spko_init_values.argtypes = [ctypes.c_uint32, ctypes.c_int64, i64p, ctypes.c_int, ctypes.c_int, i32p]
        L.spko_site_updates.argtypes = [P(Cfg), ctypes.c_int64, i64p, i32p, i32p, ctypes.c_uint32,
                                        ctypes.c_uint32, i32p]
        L.spko_site_updates.restype = ctypes.c_int64
        L.spko_neighbors_many.argtypes = [P(Cfg), ctypes.c_int64, i64p, i64p]
        L.spko_ranmars_init.argtypes = [P(RanMars), ctypes.c_int]
        L.spko_ranmars_uniform.argtypes = [P(RanMars)]
        L.spko_ranmars_uniform.restype = ctypes.c_double
        L.spko_park_uniform.argtypes = [i32p]
        L.spko_park_uniform.restype = ctypes.c_double
        L.spko_park_seed_from_double.argtypes = [ctypes.c_double]
        L.spko_park_seed_from_double.restype = ctypes.c_int32
        L.spko_park_reset.argtypes = [ctypes.c_double, ctypes.c_int64, ctypes.c_int]
        L.spko_park_reset.restype = ctypes.c_int32
        L.spko_set_range.argtypes = [ctypes.c_int32, ctypes.c_int64, ctypes.c_int, ctypes.c_int, i32p]
        L.spko_random_sector_sweeps.argtypes = [P(Cfg), i32p, i32p, ctypes.c_int, i64p, i64p]
        L.spko_kmc_create.argtypes = [P(Cfg), ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.spko_kmc_create.restype = ctypes.c_void_p
        L.spko_kmc_destroy.argtypes = [ctypes.c_void_p]
        L.spko_kmc_run.argtypes = [ctypes.c_void_p, i32p, dblp, ctypes.c_double, i64p, u64p, dblp,
                                   ctypes.c_int]
        L.spko_kmc_run.restype = ctypes.c_int
        L.spko_kmc_total_propensity.argtypes = [ctypes.c_void_p]
        L.spko_kmc_total_propensity.restype = ctypes.c_double
        L.spko_kmc_nchains.argtypes = [ctypes.c_void_p]
        L.spko_kmc_chain_events.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.spko_kmc_chain_events.restype = ctypes.c_uint64
        _lib = L
    return _lib


def _ptr(a, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def make_cfg(lattice="sq/4n", nx=8, ny=8, nz=1, app="ising", nspins=2, temperature=0.0, nsector=1,
             nloop=1, rng=RNG_PHILOX, seed=1, mask=0, procs=(1, 1, 1), stream_base=0) -> Cfg:
    return Cfg(LATTICES[lattice], nx, ny, nz, APPS[app], nspins, float(temperature), nsector, nloop, rng,
               seed & 0xFFFFFFFF, int(mask), procs[0], procs[1], procs[2], stream_base)


def philox(ctr, key):
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    lib().spko_philox(c, k, o)
    return list(o)


def nsites(cfg: Cfg) -> int:
    return cfg.nx * cfg.ny * cfg.nz


def init_spins(seed: int, n: int, lo: int, hi: int) -> np.ndarray:
    s = np.empty(n, dtype=np.int32)
    lib().spko_init_spins(seed & 0xFFFFFFFF, n, lo, hi, _ptr(s, ctypes.c_int32))
    return s


def init_values(seed: int, ids: np.ndarray, lo: int, hi: int) -> np.ndarray:
    """The initial values init_spins gives the sites `ids` alone."""
    ids = np.ascontiguousarray(ids, dtype=np.int64)
    out = np.empty(ids.size, dtype=np.int32)
    lib().spko_init_values(seed & 0xFFFFFFFF, ids.size, _ptr(ids, ctypes.c_int64), lo, hi, _ptr(out, ctypes.c_int32))
    return out


def neighbors(cfg: Cfg, i: int) -> list[int]:
    out = (ctypes.c_int64 * 26)()
    n = lib().spko_neighbors(ctypes.byref(cfg), i, out)
    return list(out[:n])


def color_sweeps(cfg: Cfg, spin: np.ndarray, sweep0: int, nsweeps: int, siteseeds=None, mask=None):
    """Runs nsweeps colour sweeps in place; returns (naccept, nattempt, hashes)."""
    assert spin.dtype == np.int32 and spin.flags.c_contiguous
    na = ctypes.c_int64(0)
    nt = ctypes.c_int64(0)
    hashes = np.zeros(max(nsweeps, 1), dtype=np.uint64)
    ss = _ptr(siteseeds, ctypes.c_int32) if siteseeds is not None else None
    mk = _ptr(mask, ctypes.c_uint8) if mask is not None else None
    rc = lib().spko_color_sweeps(ctypes.byref(cfg), _ptr(spin, ctypes.c_int32), sweep0, nsweeps,
                                 ctypes.byref(na), ctypes.byref(nt), _ptr(hashes, ctypes.c_uint64), ss, mk)
    if rc != 0:
        raise RuntimeError(f"oracle colour sweep failed: {rc}")
    return na.value, nt.value, hashes[:nsweeps]


def neighbors_many(cfg: Cfg, ids: np.ndarray) -> np.ndarray:
    """Neighbour ids of many sites, shape (n, maxneigh), reference order."""
    ids = np.ascontiguousarray(ids, dtype=np.int64)
    nn = lib().spko_maxneigh(cfg.lattice)
    out = np.empty((ids.size, nn), dtype=np.int64)
    lib().spko_neighbors_many(ctypes.byref(cfg), ids.size, _ptr(ids, ctypes.c_int64), _ptr(out, ctypes.c_int64))
    return out


def site_updates(cfg: Cfg, ids: np.ndarray, self_vals: np.ndarray, nbr_vals: np.ndarray, sweep: int,
                 npass: int = 0) -> np.ndarray:
    """New values of sites `ids` after their visit in colour sweep `sweep`,
    given their own values and their neighbours' values (n, maxneigh) as
    they see them at their turn."""
    ids = np.ascontiguousarray(ids, dtype=np.int64)
    sv = np.ascontiguousarray(self_vals, dtype=np.int32)
    nv = np.ascontiguousarray(nbr_vals, dtype=np.int32)
    out = np.empty(ids.size, dtype=np.int32)
    lib().spko_site_updates(ctypes.byref(cfg), ids.size, _ptr(ids, ctypes.c_int64), _ptr(sv, ctypes.c_int32),
                            _ptr(nv, ctypes.c_int32), sweep, npass, _ptr(out, ctypes.c_int32))
    return out


def energy(cfg: Cfg, spin: np.ndarray) -> float:
    return lib().spko_energy(ctypes.byref(cfg), _ptr(spin, ctypes.c_int32))


def clusters(cfg: Cfg, spin: np.ndarray) -> dict:
    """diag_style cluster of one lattice: Nclust, <N>, <R>."""
    s = np.ascontiguousarray(spin, dtype=np.int32)
    nc, vav, rav = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double()
    rc = lib().spko_clusters(ctypes.byref(cfg), _ptr(s, ctypes.c_int32), ctypes.byref(nc), ctypes.byref(vav),
                             ctypes.byref(rav))
    if rc != 0:
        raise MemoryError("spko_clusters")
    return {"ncluster": nc.value, "mean_volume": vav.value, "mean_radius": rav.value}


def spin_hash(spin: np.ndarray) -> int:
    s = np.ascontiguousarray(spin, dtype=np.int32)
    return int(lib().spko_hash(_ptr(s, ctypes.c_int32), s.size))


class Kmc:
    """Tree-solver KMC over sectors (and an optional processor grid)."""

    def __init__(self, cfg: Cfg, nstop: float = 1.0, tstop: float = 0.0):
        self.cfg = cfg
        self.h = lib().spko_kmc_create(ctypes.byref(cfg), 1 if tstop <= 0 else 0, nstop, tstop)
        self.time = 0.0
        self.naccept = 0

    def run(self, spin: np.ndarray, dt: float, maxrec: int = 100000):
        t = ctypes.c_double(self.time)
        na = ctypes.c_int64(self.naccept)
        hashes = np.zeros(maxrec, dtype=np.uint64)
        times = np.zeros(maxrec, dtype=np.float64)
        npass = lib().spko_kmc_run(self.h, _ptr(spin, ctypes.c_int32), ctypes.byref(t), self.time + dt,
                                   ctypes.byref(na), _ptr(hashes, ctypes.c_uint64), _ptr(times, ctypes.c_double),
                                   maxrec)
        self.time = t.value
        self.naccept = na.value
        k = min(npass, maxrec)
        return npass, hashes[:k], times[:k]

    def total_propensity(self) -> float:
        return lib().spko_kmc_total_propensity(self.h)

    def chain_events(self) -> list[int]:
        n = lib().spko_kmc_nchains(self.h)
        return [int(lib().spko_kmc_chain_events(self.h, c)) for c in range(n)]

    def __del__(self):
        if getattr(self, "h", None):
            lib().spko_kmc_destroy(self.h)
            self.h = None


def ranmars_draws(seed: int, n: int) -> list[float]:
    """The first n RanMars::uniform() values after `seed` (src/random_mars.cpp)."""
    r = RanMars()
    lib().spko_ranmars_init(ctypes.byref(r), seed)
    return [lib().spko_ranmars_uniform(ctypes.byref(r)) for _ in range(n)]


def park_seed(rseed: float) -> int:
    """RandomPark(double) seed (src/random_park.cpp:44-48)."""
    return lib().spko_park_seed_from_double(rseed)


def set_range(park: int, n: int, lo: int, hi: int) -> np.ndarray:
    """`set site range lo hi` values from a Park-Miller seed (src/set.cpp:598-624)."""
    s = np.empty(n, dtype=np.int32)
    lib().spko_set_range(park, n, lo, hi, _ptr(s, ctypes.c_int32))
    return s


def strict_siteseeds(rseed: float, n: int) -> np.ndarray:
    """Per-site seeds of sweep color/strict: tagreset(rseed, id, 100) (src/app_lattice.cpp:287-295)."""
    return np.array([lib().spko_park_reset(rseed, i + 1, 100) for i in range(n)], dtype=np.int32)


def bonds_sq4(spin2d: np.ndarray) -> int:
    """Unlike nearest-neighbour bonds of a periodic square lattice, each once."""
    s = spin2d
    return int(np.sum(s != np.roll(s, -1, axis=1)) + np.sum(s != np.roll(s, -1, axis=0)))


def _ensemble_block(job):
    """n colour sweeps of one ensemble replica from sweep index sweep0 (one
    process-pool task of EnsembleOracle.run); returns (sites, naccept)."""
    L, app, nspins, T, seed, stream_base, sp, sweep0, n = job
    cfg = make_cfg("sq/4n", L, L, 1, app, nspins, T, seed=seed, stream_base=stream_base)
    na, _, _ = color_sweeps(cfg, sp, sweep0, n)
    return sp, na


class EnsembleOracle:
    """Restatement of the batched ensemble: every replica follows the oracle's
    sq/4n colour sweep with Philox stream (r+1) << 8; every `every` sweeps the
    replicas of equal L exchange temperatures between neighbouring slots
    (sorted by T), slot pairs (j, j+1) with j = round mod 2, accepted when the
    Philox word x of counter (round, group, j) satisfies
    x < floor(exp((1/T_j - 1/T_j+1) (H_j - H_j+1)) 2^32) or the exponent is
    >= 0; H = unlike bonds."""

    def __init__(self, L, T, app="ising", nspins=2, seed=1, every=10):
        import math

        self.math = math
        self.L = [int(v) for v in L]
        self.T0 = [float(v) for v in T]
        self.app, self.nspins, self.seed, self.every = app, nspins, seed, every
        n = len(self.L)
        order = sorted(range(n), key=lambda r: (self.L[r], self.T0[r], r))
        self.groups = []
        for r in order:
            if not self.groups or self.L[self.groups[-1][0]] != self.L[r]:
                self.groups.append([])
            self.groups[-1].append(r)
        self.slot_t = [list(g) for g in self.groups]
        self.who = [list(g) for g in self.groups]
        self.tidx = list(range(n))
        self.sweep = 0
        self.xround = 0
        self.naccept = 0
        self.tries = 0
        self.accepts = 0
        self.last_bonds = [0] * n

    def run(self, spins: list, nsweeps: int, pool=None):
        """Runs nsweeps sweeps of every replica in place, with the exchange
        rounds that fall inside them.  Between two rounds the replicas are
        independent and keep their temperatures, so each replica's sweeps up
        to the next round are one oracle call; `pool` (a multiprocessing pool
        started with spawn) spreads those calls over processes."""
        done = 0
        while done < nsweeps:
            n = nsweeps - done
            if self.every:
                n = min(n, self.every - self.sweep % self.every)
            jobs = [(self.L[r], self.app, self.nspins, self.T0[self.tidx[r]], self.seed, (r + 1) << 8, sp,
                     self.sweep, n) for r, sp in enumerate(spins)]
            if pool is None:
                res = [_ensemble_block(j) for j in jobs]
            else:
                res = pool.map(_ensemble_block, jobs, chunksize=1)
            for r, (sp, na) in enumerate(res):
                if pool is not None:
                    spins[r][...] = sp
                self.naccept += na
            self.sweep += n
            done += n
            if self.every and self.sweep % self.every == 0:
                self._exchange(spins)

    def _exchange(self, spins):
        bonds = [bonds_sq4(sp.reshape(self.L[r], self.L[r])) for r, sp in enumerate(spins)]
        for g, (slots_t, who) in enumerate(zip(self.slot_t, self.who)):
            for j in range(self.xround & 1, len(who) - 1, 2):
                ra, rb = who[j], who[j + 1]
                ta, tb = slots_t[j], slots_t[j + 1]
                delta = (1.0 / self.T0[ta] - 1.0 / self.T0[tb]) * (float(bonds[ra]) - float(bonds[rb]))
                x = philox([self.xround, g, j, 0], [self.seed & 0xFFFFFFFF, 2])[0]
                ok = delta >= 0.0 or float(x) < self.math.floor(self.math.exp(delta) * 4294967296.0)
                self.tries += 1
                if ok:
                    who[j], who[j + 1] = rb, ra
                    self.tidx[ra], self.tidx[rb] = tb, ta
                    self.accepts += 1
        self.last_bonds = bonds
        self.xround += 1

    def temperatures(self):
        return [self.T0[t] for t in self.tidx]
