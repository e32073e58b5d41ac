"""The configuration sizes of the path, checked through size-independent
properties where the oracle would take too long: two kernels or two storage
forms of the same draws must agree exactly on the device-computed energy,
change count and site sum; the smallest configuration runs against the
oracle in full.  Lattices beyond 2^31 sites exercise 64-bit indexing."""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    import spparks_gb300

    spparks_gb300.load_library()
    return spparks_gb300


def fingerprint(lat):
    st = lat.stats()
    return lat.energy(), lat.site_stats()["sum"], st["naccept"], st["nattempt"]


def test_c0_plain_ising_128_int32_100_sweeps_equals_oracle(sg):
    """128^2 sq/4n Ising, int32, kT = 2.269, 100 colour sweeps: bit-identical
    to the oracle after every sweep"""
    seed = 56789
    spin = oracle.init_spins(seed, 128 * 128, 1, 2)
    cfg = oracle.make_cfg("sq/4n", 128, 128, 1, "ising", 2, 2.269, seed=seed)
    ref = spin.copy()
    na, nt, hashes = oracle.color_sweeps(cfg, ref, 0, 100)
    lat = sg.Lattice("sq/4n", 128, 128, 1, "ising", 2, spin_bytes=4, seed=seed)
    lat.set_temperature(2.269)
    lat.upload(spin)
    got = []
    for _ in range(100):
        lat.sweep(1)
        got.append(oracle.spin_hash(lat.download()))
    assert got == [int(h) for h in hashes]
    assert (lat.stats()["naccept"], lat.stats()["nattempt"]) == (na, nt)


def test_c1_neighonly_sc26n_256_int16_rows_equal_phase_kernel(sg):
    """256^3 sc/26n potts/neighonly Q = 100, int16, kT = 0.5: the row-pair
    kernel and the per-colour phase kernel give the same lattice"""
    out = []
    for variant in (0, 1):
        lat = sg.Lattice("sc/26n", 256, 256, 256, "potts/neighonly", 100, spin_bytes=2, seed=56789, variant=variant)
        lat.set_temperature(0.5)
        lat.init_spins(1, 100)
        lat.sweep(2)
        out.append(fingerprint(lat))
        lat.close()
    assert out[0] == out[1]
    assert out[0][2] > 0


def test_c2_ensemble_512_replicas_both_forms_agree(sg, monkeypatch):
    """the full 512-replica ensemble: every execution form (persistent, one
    launch per sweep with 1, 2 or 4 tiles per CTA, one tile per warp) gives the same sites,
    temperatures, energies and counters after two exchange periods"""
    import bench

    L, T = bench.ensemble_config(seed=bench.SEED)
    spins = bench.init_spins(L, seed=bench.SEED)
    res = []
    for mode in sg.ENSEMBLE_MODES:
        monkeypatch.setenv("SPKGPU_ENSEMBLE_MODE", mode)
        ens = sg.Ensemble(L, T, "ising", 2, seed=bench.SEED, exchange_every=10)
        ens.upload(spins)
        ens.run(20)
        out = ens.download()
        res.append((oracle.spin_hash(out), ens.temperatures().tolist(), ens.energies().tolist(), ens.stats()))
        ens.close()
    assert all(r == res[0] for r in res[1:])
    assert res[0][3]["exchange_tries"] > 0


def test_c4_packed_sc6n_1536_equals_int8(sg):
    """1536^3 (3.6e9 sites) sc/6n Ising, kT = 4.5115: the bit-packed multispin
    sweep and the int8 per-colour sweep give the same energy, change count
    and magnetisation"""
    out = []
    for sb in (-1, 1):
        lat = sg.Lattice("sc/6n", 1536, 1536, 1536, "ising", 2, spin_bytes=sb, seed=56789)
        lat.set_temperature(4.5115)
        lat.init_spins(1, 2)
        lat.sweep(2)
        out.append(fingerprint(lat))
        lat.close()
    assert out[0] == out[1]
    assert out[0][3] == 2 * 1536 ** 3


def test_single_lattice_beyond_2_31_sites(sg):
    """a 49152^2 int8 Ising lattice (2.4e9 sites): the fused tile sweep and the
    per-colour phase kernel agree; the 32-bit cluster labelling refuses it"""
    out = []
    for variant in (0, 1):
        lat = sg.Lattice("sq/4n", 49152, 49152, 1, "ising", 2, spin_bytes=1, seed=24680, variant=variant)
        lat.set_temperature(2.5)
        lat.init_spins(1, 2)
        lat.sweep(1)
        out.append(fingerprint(lat))
        if variant == 1:
            with pytest.raises(sg.SpkGpuError) as ei:
                lat.clusters()
            assert ei.value.code == -8
        lat.close()
    assert out[0] == out[1]
    assert out[0][3] == 49152 ** 2
