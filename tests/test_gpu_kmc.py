"""GPU parity of rejection-free KMC with the tree solver over sectors
(spkgpu_kmc_setup / spkgpu_kmc_run): FP64 propensities must reproduce the
reference (fixtures from the reference with the Philox shim) and the oracle
restatement exactly - lattice, event count, passes and clock; FP32
propensities must keep the total propensity within 1e-6 relative of FP64."""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    import spparks_gb300

    spparks_gb300.load_library()
    return spparks_gb300


@pytest.mark.parametrize("k", range(5))
def test_kmc_matches_reference_fixtures(sg, ref_fixtures, k):
    fx = ref_fixtures["kmc"][k]
    c = fx["case"]
    nsec = 4 if c["lattice"].startswith("sq") else 8
    lat = sg.Lattice(c["lattice"], c["nx"], c["ny"], c["nz"], c["app"], c["nspins"], nsector=nsec, seed=c["seed"])
    lat.set_temperature(c["temperature"])
    lat.upload(np.array(fx["snaps"]["init"]["spins"], dtype=np.int32))
    lat.kmc_setup(adapt=True, nstop=1.0, fp64=True)
    t = 0.0
    npass = 0
    for r, dt in enumerate(c["runs"]):
        st = lat.kmc_run(t, t + dt)
        t = st["time"]
        assert lat.download().tolist() == fx["snaps"][f"run{r}"]["spins"]
    ref = fx["sweeps"]
    assert st["npass"] == len(ref)
    assert st["naccept"] == ref[-1][1]
    assert t == pytest.approx(ref[-1][4], rel=1e-12)


KMC_CASES = [
    dict(lattice="sq/8n", nx=32, ny=32, nz=1, app="potts", nspins=10, T=1.0, procs=(2, 2, 1), nsector=4, run=2.0),
    dict(lattice="sq/4n", nx=24, ny=16, nz=1, app="ising", nspins=2, T=2.0, procs=(3, 2, 1), nsector=4, run=1.5),
    dict(lattice="sc/26n", nx=12, ny=12, nz=8, app="potts", nspins=20, T=0.8, procs=(2, 1, 1), nsector=8, run=0.4),
    dict(lattice="sc/6n", nx=12, ny=8, nz=8, app="potts/neighonly", nspins=6, T=0.7, procs=(1, 1, 1), nsector=2,
         run=1.0),
]


@pytest.mark.parametrize("c", KMC_CASES, ids=lambda c: f"{c['app']}-{c['lattice']}-{c['procs']}")
def test_kmc_processor_grid_matches_oracle(sg, c):
    seed = 1357
    n = c["nx"] * c["ny"] * c["nz"]
    spin = oracle.init_spins(seed, n, 1, c["nspins"])
    cfg = oracle.make_cfg(c["lattice"], c["nx"], c["ny"], c["nz"], c["app"], c["nspins"], c["T"], c["nsector"],
                          seed=seed, procs=c["procs"])
    km = oracle.Kmc(cfg)
    ref = spin.copy()
    npass, _, times = km.run(ref, c["run"])
    lat = sg.Lattice(c["lattice"], c["nx"], c["ny"], c["nz"], c["app"], c["nspins"], nsector=c["nsector"],
                     procs=c["procs"], seed=seed)
    lat.set_temperature(c["T"])
    lat.upload(spin)
    lat.kmc_setup(fp64=True)
    st = lat.kmc_run(0.0, c["run"])
    assert lat.download().tolist() == ref.tolist()
    assert st["naccept"] == km.naccept
    assert st["npass"] == npass
    assert st["time"] == pytest.approx(km.time, rel=1e-12)
    assert st["total_propensity"] == pytest.approx(km.total_propensity(), rel=1e-12)


def test_kmc_fp32_propensity_error(sg):
    """FP32 propensities, FP64 tree: relative error of the total propensity
    against the FP64 path on the same lattice state."""
    seed = 24
    nx = ny = 64
    spin = oracle.init_spins(seed, nx * ny, 1, 50)
    tot = {}
    for fp64 in (True, False):
        lat = sg.Lattice("sq/8n", nx, ny, 1, "potts", 50, nsector=4, procs=(4, 4, 1), seed=seed)
        lat.set_temperature(1.0)
        lat.upload(spin)
        lat.kmc_setup(fp64=fp64)
        st = lat.kmc_run(0.0, 0.0)
        tot[fp64] = st["total_propensity"]
    assert abs(tot[False] - tot[True]) / tot[True] < 1e-6


def test_kmc_fp32_run_states_its_error_against_fp64(sg):
    """An FP32-propensity run (FP64 tree sums, roots and clock) states its
    precision against all-FP64 propensities: the largest relative error of
    its adaptive time steps nstop/pmax (pmax sampled where the reference
    samples it) and of the final lattice's total propensity, both < 1e-6;
    an FP64 run reports zero for both."""
    seed = 31
    nx = ny = 64
    spin = oracle.init_spins(seed, nx * ny, 1, 20)
    for fp64 in (False, True):
        lat = sg.Lattice("sq/8n", nx, ny, 1, "potts", 20, nsector=4, procs=(4, 4, 1), seed=seed)
        lat.set_temperature(0.8)
        lat.upload(spin)
        lat.kmc_setup(fp64=fp64)
        st = lat.kmc_run(0.0, 2.0)
        assert st["naccept"] > 1000 and st["npass"] > 2
        if fp64:
            assert (st["dt_rel_err"], st["prop_rel_err"]) == (0.0, 0.0)
        else:
            assert 0.0 < st["dt_rel_err"] < 1e-6
            assert 0.0 < st["prop_rel_err"] < 1e-6
        lat.close()


def test_kmc_run_in_pieces_equals_one_run(sg):
    """a run paused at arbitrary output times and continued ends in the same
    state as one uninterrupted run"""
    seed, nx = 51, 32
    spin = oracle.init_spins(seed, nx * nx, 1, 12)
    finals = []
    for pieces in ([], [0.1, 0.35, 0.36, 0.9]):
        lat = sg.Lattice("sq/8n", nx, nx, 1, "potts", 12, nsector=4, procs=(2, 2, 1), seed=seed)
        lat.set_temperature(0.9)
        lat.upload(spin)
        lat.kmc_setup(fp64=True, nstop=0.25)
        t, first, npieces = 0.0, True, 0
        for until in pieces + [1.5]:
            if t >= 1.5:
                break  # the run is over: nothing to continue
            st = lat.kmc_run(t, 1.5, until=max(until, t), first=first)
            first = False
            npieces += 1
            assert st["time"] >= until or st["time"] >= 1.5
            t = st["time"]
        assert npieces > 1 or not pieces
        finals.append((st["naccept"], st["npass"], st["time"], lat.download().tolist()))
        lat.close()
    assert finals[0] == finals[1]


SERIAL_TREE_CASES = [
    # one processor: chains large enough that only the top 14 tree levels stay in shared memory and the
    # rest is fetched per event (3d site blocks of 125 values, box sides that are not powers of two)
    dict(lattice="sc/26n", nx=96, ny=96, nz=96, app="potts", nspins=20, T=0.8, nsector=8, run=0.004),
    dict(lattice="sc/6n", nx=64, ny=64, nz=64, app="ising", nspins=2, T=3.0, nsector=2, run=0.02),
    dict(lattice="sq/4n", nx=768, ny=512, nz=1, app="potts/neighonly", nspins=12, T=0.6, nsector=4, run=0.01),
]


@pytest.mark.parametrize("c", SERIAL_TREE_CASES, ids=lambda c: f"{c['app']}-{c['lattice']}-{c['nx']}")
def test_kmc_large_chains_match_oracle(sg, c):
    """serial chains whose trees exceed the shared-memory levels: the event
    loop fetches subtrees and paths from the global tree; lattice, events,
    passes and clock equal the oracle's"""
    seed = 97
    n = c["nx"] * c["ny"] * c["nz"]
    spin = oracle.init_spins(seed, n, 1, c["nspins"])
    cfg = oracle.make_cfg(c["lattice"], c["nx"], c["ny"], c["nz"], c["app"], c["nspins"], c["T"], c["nsector"],
                          seed=seed)
    km = oracle.Kmc(cfg)
    ref = spin.copy()
    npass, _, _ = km.run(ref, c["run"])
    assert km.naccept > 1000
    lat = sg.Lattice(c["lattice"], c["nx"], c["ny"], c["nz"], c["app"], c["nspins"], nsector=c["nsector"], seed=seed)
    lat.set_temperature(c["T"])
    lat.upload(spin)
    lat.kmc_setup(fp64=True)
    st = lat.kmc_run(0.0, c["run"])
    assert oracle.spin_hash(lat.download()) == oracle.spin_hash(ref)
    assert (st["naccept"], st["npass"]) == (km.naccept, npass)
    assert st["time"] == pytest.approx(km.time, rel=1e-12)
    lat.close()
