"""GPU parity of the colour-sweep path (spkgpu_sweep through the C ABI).

Lattices must be bit-identical to the reference (fixtures produced by the
reference built with the Philox RandomPark shim, and by the unmodified
reference for sweep color/strict) and to the oracle restatement after every
sweep; Naccept/Nattempt must match exactly."""

import numpy as np
import pytest

import oracle
from conftest import fixture_count

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    import spparks_gb300

    spparks_gb300.load_library()
    return spparks_gb300


def make_lattice(sg, case, spin_bytes=0, rng=0, seed=None, procs=(1, 1, 1)):
    return sg.Lattice(case["lattice"], case["nx"], case["ny"], case["nz"], case["app"], case["nspins"],
                      spin_bytes=spin_bytes, nsector=case.get("nsector", 1), nloop=case.get("nloop", 1),
                      procs=procs, rng=rng, mask=case.get("mask", False),
                      seed=case.get("seed", 0) if seed is None else seed)


@pytest.mark.parametrize("k", range(fixture_count("sweeps")))
def test_sweeps_match_reference_fixtures(sg, ref_fixtures, k):
    fx = ref_fixtures["sweeps"][k]
    case = fx["case"]
    init = np.array(fx["snaps"]["init"]["spins"], dtype=np.int32)
    for sb in (1, 2, 4):
        if sb == 1 and case["nspins"] > 127:
            continue
        lat = make_lattice(sg, case, spin_bytes=sb)
        lat.set_temperature(case["temperature"])
        lat.upload(init)
        hashes = []
        for s in range(case["nsweeps"]):
            lat.sweep(1)
            hashes.append(format(oracle.spin_hash(lat.download()), "016x"))
        assert hashes == [r[3] for r in fx["sweeps"]], (case["name"], sb)
        st = lat.stats()
        assert (st["naccept"], st["nattempt"]) == (fx["sweeps"][-1][1], fx["sweeps"][-1][2])
        assert lat.download().tolist() == fx["snaps"]["final"]["spins"]
        lat.close()


@pytest.mark.parametrize("k", range(3))
def test_strict_matches_unmodified_reference(sg, ref_fixtures, k):
    fx = ref_fixtures["strict"][k]
    case = fx["case"]
    n = case["nx"] * case["ny"] * case["nz"]
    u = oracle.ranmars_draws(case["master_seed"], 5)
    spin = oracle.set_range(oracle.park_seed(u[0]), n, 1, case["nspins"])
    seeds = oracle.strict_siteseeds(u[4], n)
    lat = make_lattice(sg, case, rng=1, seed=0)
    lat.set_temperature(case["temperature"])
    lat.upload(spin)
    lat.upload_siteseeds(seeds)
    for r in range(case["nruns"]):
        lat.sweep(case["sweeps_per_run"])
        assert lat.download().tolist() == fx["snaps"][f"run{r}"]["spins"]
        assert lat.energy() == fx["energies"][r]
    lat.close()


RANDOM_CASES = [
    dict(lattice="sc/26n", nx=16, ny=10, nz=6, app="potts", nspins=300, temperature=0.6),
    dict(lattice="sq/8n", nx=34, ny=12, nz=1, app="ising", nspins=2, temperature=1.7),
    dict(lattice="sq/4n", nx=64, ny=48, nz=1, app="potts", nspins=50, temperature=0.9),
    dict(lattice="sq/8n", nx=40, ny=40, nz=1, app="potts/neighonly", nspins=30, temperature=0.4),
    dict(lattice="sc/6n", nx=16, ny=12, nz=10, app="ising", nspins=2, temperature=4.5115),
    dict(lattice="sc/26n", nx=12, ny=12, nz=12, app="potts/neighonly", nspins=100, temperature=0.5),
    dict(lattice="sc/26n", nx=10, ny=8, nz=6, app="potts/neigh", nspins=7, temperature=1.3),
    dict(lattice="sq/4n", nx=32, ny=32, nz=1, app="ising", nspins=2, temperature=1.1345, nsector=4),
    dict(lattice="sc/6n", nx=12, ny=12, nz=12, app="potts", nspins=5, temperature=0.7, nsector=8),
    # zero temperature: every uphill move rejected (src/app_potts.cpp:128)
    dict(lattice="sq/8n", nx=40, ny=24, nz=1, app="potts", nspins=12, temperature=0.0),
    dict(lattice="sc/26n", nx=12, ny=10, nz=8, app="potts/neighonly", nspins=40, temperature=0.0),
    dict(lattice="sq/4n", nx=64, ny=32, nz=1, app="potts/neigh", nspins=6, temperature=0.0),
]


@pytest.mark.parametrize("variant", [0, 1])
@pytest.mark.parametrize("case", RANDOM_CASES,
                         ids=lambda c: f"{c['app']}-{c['lattice']}-{c.get('nsector', 1)}-T{c['temperature']}")
def test_random_cases_match_oracle(sg, case, variant):
    """variant 0 takes the fastest kernel (fused tile, row-pair or packed),
    variant 1 always the per-colour phase kernel."""
    seed = 97531
    n = case["nx"] * case["ny"] * case["nz"]
    spin = oracle.init_spins(seed, n, 1, case["nspins"])
    cfg = oracle.make_cfg(case["lattice"], case["nx"], case["ny"], case["nz"], case["app"], case["nspins"],
                          case["temperature"], case.get("nsector", 1), 1, 0, seed)
    ref = spin.copy()
    na, nt, hashes = oracle.color_sweeps(cfg, ref, 0, 5)
    lat = sg.Lattice(case["lattice"], case["nx"], case["ny"], case["nz"], case["app"], case["nspins"],
                     nsector=case.get("nsector", 1), seed=seed, variant=variant)
    lat.set_temperature(case["temperature"])
    lat.upload(spin)
    got = []
    for s in range(5):
        lat.sweep(1)
        got.append(oracle.spin_hash(lat.download()))
    assert got == [int(h) for h in hashes]
    st = lat.stats()
    assert (st["naccept"], st["nattempt"]) == (na, nt)


# the row-pair kernel (sq/8n and sc/26n without sectors): stamp table and
# packed counts for potts/neighonly and potts/neigh with values below 128,
# the pairwise scan above; 16-byte staged copies where a row's bytes are a
# multiple of 16, element copies elsewhere; one to sixteen warps per row
ROW_CASES = [
    dict(lattice="sc/26n", nx=16, ny=6, nz=4, app="potts/neighonly", nspins=20, temperature=0.5, sb=1),
    dict(lattice="sc/26n", nx=24, ny=4, nz=6, app="potts/neighonly", nspins=100, temperature=0.5, sb=2),
    dict(lattice="sc/26n", nx=20, ny=4, nz=4, app="potts/neigh", nspins=9, temperature=0.9, sb=1),
    dict(lattice="sc/26n", nx=10, ny=6, nz=4, app="potts/neighonly", nspins=300, temperature=0.7, sb=2),
    dict(lattice="sc/26n", nx=12, ny=4, nz=4, app="potts/neighonly", nspins=127, temperature=0.0, sb=4),
    dict(lattice="sq/8n", nx=300, ny=6, nz=1, app="potts/neighonly", nspins=127, temperature=0.6, sb=4),
    dict(lattice="sq/8n", nx=1024, ny=4, nz=1, app="potts/neighonly", nspins=50, temperature=0.8, sb=2),
    dict(lattice="sq/8n", nx=18, ny=8, nz=1, app="potts", nspins=5, temperature=0.8, sb=1),
    dict(lattice="sq/8n", nx=32, ny=8, nz=1, app="ising", nspins=2, temperature=1.5, sb=2),
    dict(lattice="sq/8n", nx=64, ny=4, nz=1, app="potts/neigh", nspins=30, temperature=0.4, sb=1),
    # the largest stamp table (128 value rows of 512 threads) beside 9 int32 rows: opt-in shared memory
    dict(lattice="sc/26n", nx=1024, ny=4, nz=4, app="potts/neighonly", nspins=127, temperature=0.6, sb=4),
    dict(lattice="sc/26n", nx=512, ny=6, nz=4, app="potts/neigh", nspins=127, temperature=0.9, sb=1),
]


@pytest.mark.parametrize("case", ROW_CASES,
                         ids=lambda c: f"{c['app']}-{c['lattice']}-{c['nx']}-Q{c['nspins']}-int{8 * c['sb']}")
def test_row_pair_kernel_matches_oracle(sg, case):
    seed = 8642
    n = case["nx"] * case["ny"] * case["nz"]
    spin = oracle.init_spins(seed, n, 1, case["nspins"])
    cfg = oracle.make_cfg(case["lattice"], case["nx"], case["ny"], case["nz"], case["app"], case["nspins"],
                          case["temperature"], 1, 1, 0, seed)
    ref = spin.copy()
    na, nt, hashes = oracle.color_sweeps(cfg, ref, 0, 4)
    lat = sg.Lattice(case["lattice"], case["nx"], case["ny"], case["nz"], case["app"], case["nspins"],
                     spin_bytes=case["sb"], seed=seed, variant=0)
    lat.set_temperature(case["temperature"])
    lat.upload(spin)
    got = []
    for s in range(4):
        lat.sweep(1)
        got.append(oracle.spin_hash(lat.download()))
    assert got == [int(h) for h in hashes]
    assert (lat.stats()["naccept"], lat.stats()["nattempt"]) == (na, nt)
    lat.close()


@pytest.mark.parametrize("procs,nsector", [((2, 2, 1), 4), ((3, 1, 1), 2), ((2, 1, 1), 1)])
def test_processor_grid_sectors_match_oracle(sg, procs, nsector):
    """`processors Px Py 1` + `sector`: sector k of every sub-domain is one set
    (the reference's parallel ordering, src/app_lattice.cpp:648-699)."""
    case = dict(lattice="sq/8n", nx=24, ny=20, nz=1, app="potts", nspins=9, temperature=0.8, nsector=nsector)
    seed = 4242
    n = 24 * 20
    spin = oracle.init_spins(seed, n, 1, 9)
    cfg = oracle.make_cfg("sq/8n", 24, 20, 1, "potts", 9, 0.8, nsector, 1, 0, seed, procs=procs)
    ref = spin.copy()
    na, nt, hashes = oracle.color_sweeps(cfg, ref, 0, 4)
    lat = make_lattice(sg, case, seed=seed, procs=procs)
    lat.set_temperature(0.8)
    lat.upload(spin)
    lat.sweep(4)
    assert lat.download().tolist() == ref.tolist()
    assert lat.stats()["naccept"] == na


def test_invalid_spin_rejected(sg):
    lat = sg.Lattice("sq/4n", 8, 8, 1, "potts", 5)
    bad = np.full(64, 3, dtype=np.int32)
    bad[17] = 6
    with pytest.raises(sg.SpkGpuError) as ei:
        lat.upload(bad)
    assert ei.value.code == -6


def test_sweep_before_temperature_is_an_error(sg):
    lat = sg.Lattice("sq/4n", 8, 8, 1, "ising", 2)
    with pytest.raises(sg.SpkGpuError) as ei:
        lat.sweep(1)
    assert ei.value.code == -3


def test_energy_matches_oracle(sg):
    seed = 5
    spin = oracle.init_spins(seed, 20 * 20 * 20, 1, 40)
    lat = sg.Lattice("sc/26n", 20, 20, 20, "potts", 40, seed=seed)
    lat.upload(spin)
    cfg = oracle.make_cfg("sc/26n", 20, 20, 20, "potts", 40)
    assert lat.energy() == oracle.energy(cfg, spin)


def test_philox_rate_calibration(sg):
    """the draw-side ceiling the bench reports: Philox blocks/s of the device"""
    assert sg.philox_rate(0, 256) > 1e10


@pytest.mark.parametrize("lattice,nx,ny,nz,sb", [("sq/4n", 64, 48, 1, 1), ("sq/8n", 30, 10, 1, 2),
                                                 ("sc/26n", 6, 6, 6, 4), ("sc/6n", 64, 4, 4, -1),
                                                 ("sq/4n", 10, 6, 1, 1)])
def test_pinned_host_buffers_equal_pageable(sg, lattice, nx, ny, nz, sb):
    """uploads and downloads through registered pinned host memory (read and
    written by the conversion kernels directly) equal the staged path for
    pageable memory, including the invalid-value check"""
    import torch

    app, q = ("ising", 2) if sb == -1 else ("potts", 9)
    n = nx * ny * nz
    spin = oracle.init_spins(77, n, 1, q)
    pinned = torch.from_numpy(spin.copy()).pin_memory()
    out_pinned = torch.zeros(n, dtype=torch.int32).pin_memory()
    lat = sg.Lattice(lattice, nx, ny, nz, app, q, spin_bytes=sb, seed=5)
    lat.set_temperature(0.8)
    lat.upload(pinned.numpy())
    lat.sweep(2)
    lat.download(out_pinned.numpy())
    ref = sg.Lattice(lattice, nx, ny, nz, app, q, spin_bytes=sb, seed=5)
    ref.set_temperature(0.8)
    ref.upload(spin)
    ref.sweep(2)
    assert out_pinned.numpy().tolist() == ref.download().tolist()
    bad = pinned.clone().pin_memory()
    bad[n - 1] = q + 1  # in the tail or the last 16-byte group
    with pytest.raises(sg.SpkGpuError):
        lat.upload(bad.numpy())
    lat.close()
    ref.close()


def test_pinned_ensemble_buffers_equal_pageable(sg):
    import torch

    L, T = [32, 64, 96], [2.0, 2.4, 2.8]
    n = sum(l * l for l in L)
    spin = oracle.init_spins(9, n, 1, 2)
    out = []
    for pin in (False, True):
        ens = sg.Ensemble(L, T, "ising", 2, seed=3, exchange_every=2)
        src = torch.from_numpy(spin.copy()).pin_memory().numpy() if pin else spin
        ens.upload(src)
        ens.run(4)
        dst = torch.zeros(n, dtype=torch.int32).pin_memory().numpy() if pin else np.zeros(n, dtype=np.int32)
        ens.download(dst)
        out.append(dst.tolist())
        ens.close()
    assert out[0] == out[1]


@pytest.mark.parametrize("T", [2.269, 0.0, 1e30])
def test_fused_warp_sweeps_in_one_call_match_oracle(sg, T):
    """Ising int8 on sq/4n through the warp tile, 7 sweeps in one call, then 3
    more in another call: equal to the oracle"""
    seed, nx, ny = 8080, 96, 64
    spin = oracle.init_spins(seed, nx * ny, 1, 2)
    cfg = oracle.make_cfg("sq/4n", nx, ny, 1, "ising", 2, T, seed=seed)
    ref = spin.copy()
    na, nt, hashes = oracle.color_sweeps(cfg, ref, 0, 10)
    lat = sg.Lattice("sq/4n", nx, ny, 1, "ising", 2, spin_bytes=1, seed=seed, variant=2)
    lat.set_temperature(T)
    lat.upload(spin)
    lat.sweep(7)
    assert oracle.spin_hash(lat.download()) == int(hashes[6])
    lat.sweep(3)
    assert oracle.spin_hash(lat.download()) == int(hashes[9])
    st = lat.stats()
    assert (st["naccept"], st["nattempt"]) == (na, nt)
    lat.close()
