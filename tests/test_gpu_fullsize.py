"""The configurations at their full sizes against the oracle.

C0, C1, C2 and C3 run in full on the oracle (C2 spread over host processes
between exchange rounds, C3 for one whole pass over its four sectors).  C4
(3.6e9 sites) is too large for a full oracle run: a sample of sites,
including every wrap face, is checked one site at a time against the
oracle's per-site rule, from the values the site and its neighbours hold
before and after the sweep on the device.  Size-independent properties
(two kernels or two storage forms of the same draws agree exactly) cover
the rest; lattices beyond 2^31 sites exercise 64-bit indexing."""

import multiprocessing as mp
import os

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


def test_c1_neighonly_sc26n_256_int16_equals_oracle(sg):
    """256^3 sc/26n potts/neighonly Q = 100, int16, kT = 0.5, 2 sweeps: the
    row-pair kernel bit-identical to the oracle after each sweep"""
    seed, n = 56789, 256 ** 3
    spin = oracle.init_spins(seed, n, 1, 100)
    lat = sg.Lattice("sc/26n", 256, 256, 256, "potts/neighonly", 100, spin_bytes=2, seed=seed)
    lat.set_temperature(0.5)
    lat.init_spins(1, 100)
    assert np.array_equal(lat.download(), spin)
    got = []
    for _ in range(2):
        lat.sweep(1)
        got.append(oracle.spin_hash(lat.download()))
    cfg = oracle.make_cfg("sc/26n", 256, 256, 256, "potts/neighonly", 100, 0.5, seed=seed)
    na, nt, hashes = oracle.color_sweeps(cfg, spin, 0, 2)
    assert got == [int(h) for h in hashes]
    st = lat.stats()
    assert (st["naccept"], st["nattempt"]) == (na, nt) and na > 0
    lat.close()


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


def test_c2_ensemble_512_replicas_equals_oracle(sg):
    """the full 512-replica ensemble (9.8e7 sites), 20 sweeps with two
    exchange rounds, in the execution form the autotuner keeps: every
    replica's sites, its temperature, the change count and the exchange
    decisions equal the oracle's restatement of the ensemble"""
    import bench

    L, T = bench.ensemble_config(seed=bench.SEED)
    spins = bench.init_spins(L, seed=bench.SEED)
    ens = sg.Ensemble(L, T, "ising", 2, seed=bench.SEED, exchange_every=10)
    ens.upload(spins)
    ens.run(20)
    out = ens.download()
    st = ens.stats()
    temps = ens.temperatures()
    ref = [ens.replica(spins, r).copy() for r in range(len(L))]
    orc = oracle.EnsembleOracle(L, T, "ising", 2, seed=bench.SEED, every=10)
    with mp.get_context("spawn").Pool(max(1, min(32, os.cpu_count() or 1))) as pool:
        orc.run(ref, 20, pool=pool)
    bad = [r for r in range(len(L)) if not np.array_equal(ens.replica(out, r), ref[r])]
    assert not bad, f"{len(bad)} replicas differ, first {bad[:5]}"
    assert temps.tolist() == orc.temperatures()
    assert st["naccept"] == orc.naccept
    assert (st["exchange_tries"], st["exchange_accepts"]) == (orc.tries, orc.accepts)
    ens.close()


def test_c3_tree_kmc_2048_serial_one_pass_equals_oracle(sg):
    """2048^2 sq/8n Potts Q = 50, kT = 1, solve_style tree, sector yes (four
    sectors of 2^20 sites), one processor, FP64 propensities: one whole pass
    over the four sectors (t = 0.1, below the adaptive step, so the run's end
    bounds the sector time) gives the oracle's lattice, events, passes and
    clock.  The FP32-propensity run of the same pass states its errors
    against all-FP64 propensities, both below 1e-6."""
    seed, nx = 56789, 2048
    spin = oracle.init_spins(seed, nx * nx, 1, 50)
    cfg = oracle.make_cfg("sq/8n", nx, nx, 1, "potts", 50, 1.0, 4, seed=seed)
    km = oracle.Kmc(cfg)
    ref = spin.copy()
    npass, _, _ = km.run(ref, 0.1)
    assert npass == 1 and km.naccept > 10 ** 6
    lat = sg.Lattice("sq/8n", nx, nx, 1, "potts", 50, nsector=4, seed=seed)
    lat.set_temperature(1.0)
    lat.upload(spin)
    lat.kmc_setup(fp64=True)
    st = lat.kmc_run(0.0, 0.1)
    assert st["naccept"] == km.naccept and st["npass"] == npass
    assert oracle.spin_hash(lat.download()) == oracle.spin_hash(ref)
    assert st["time"] == pytest.approx(km.time, rel=1e-12)
    assert st["total_propensity"] == pytest.approx(km.total_propensity(), rel=1e-12)
    lat.close()
    lat = sg.Lattice("sq/8n", nx, nx, 1, "potts", 50, nsector=4, seed=seed)
    lat.set_temperature(1.0)
    lat.upload(spin)
    lat.kmc_setup(fp64=False)
    st32 = lat.kmc_run(0.0, 0.1)
    assert st32["npass"] == 1 and st32["time"] == pytest.approx(0.1, rel=1e-12)
    assert 0.0 < st32["prop_rel_err"] < 1e-6 and 0.0 <= st32["dt_rel_err"] < 1e-6
    assert abs(st32["naccept"] - km.naccept) < 1e-2 * km.naccept
    lat.close()


class _DeviceBytes:
    """A device buffer seen by torch through the CUDA array interface."""

    def __init__(self, ptr, nbytes):
        self.__cuda_array_interface__ = {"shape": (nbytes,), "typestr": "|u1", "data": (ptr, False),
                                         "version": 3}


def _packed_values(words, ids):
    """site values (1 or 2) of bit-packed Ising sites: bit b of word w is
    site 64 w + b"""
    import torch

    w = words[ids >> 6]
    return (1 + ((w >> (ids & 63)) & 1)).to(torch.int32)


def test_c4_packed_sc6n_1536_sampled_sites_equal_oracle(sg):
    """1536^3 (3.6e9 sites) sc/6n Ising bit-packed, kT = 4.5115, one sweep:
    for 6e6 sites (4e6 uniform, 2e6 on the six wrap faces) the new value
    equals the oracle's per-site rule applied to the site's old value and
    its neighbours' values at its turn (colour 1: old; colour 2: new), with
    the site's own Philox word; the initial values equal the oracle's too"""
    import ctypes

    import torch

    n_side = 1536
    n = n_side ** 3
    seed, T = 56789, 4.5115
    lat = sg.Lattice("sc/6n", n_side, n_side, n_side, "ising", 2, spin_bytes=-1, seed=seed)
    lat.set_temperature(T)
    lat.init_spins(1, 2)
    ptr, nbytes = ctypes.c_void_p(), ctypes.c_int64()
    assert lat.lib.spkgpu_device_spins(lat.h, ctypes.byref(ptr), ctypes.byref(nbytes)) == 0
    assert nbytes.value == n // 8
    words = torch.as_tensor(_DeviceBytes(ptr.value, nbytes.value), device="cuda").view(torch.int64)

    rng = np.random.default_rng(4)
    face = []
    for axis in range(3):
        for edge in (0, n_side - 1):
            c = rng.integers(0, n_side, size=(3, 2 ** 20 // 3))
            c[axis] = edge
            face.append(c[0] + n_side * (c[1] + n_side * c[2]))
    ids = np.unique(np.concatenate([rng.integers(0, n, 4 * 10 ** 6)] + face))
    cfg = oracle.make_cfg("sc/6n", n_side, n_side, n_side, "ising", 2, T, seed=seed)
    nb = oracle.neighbors_many(cfg, ids)
    x, y, z = ids % n_side, (ids // n_side) % n_side, ids // (n_side * n_side)
    color1 = ((x + y + z) % 2) == 0
    assert all(oracle.lib().spko_color(cfg, int(i)) == (1 if c else 2) for i, c in zip(ids[:1000], color1[:1000]))
    dev_ids = torch.from_numpy(ids).cuda()
    dev_nb = torch.from_numpy(nb).cuda()
    old_self = _packed_values(words, dev_ids).cpu().numpy()
    old_nb = _packed_values(words, dev_nb).cpu().numpy()
    assert np.array_equal(old_self, oracle.init_values(seed, ids, 1, 2))
    lat.sweep(1)
    lat.synchronize()
    new_self = _packed_values(words, dev_ids).cpu().numpy()
    new_nb = _packed_values(words, dev_nb).cpu().numpy()
    seen = np.where(color1[:, None], old_nb, new_nb)
    want = oracle.site_updates(cfg, ids, old_self, seen, 0)
    bad = np.nonzero(want != new_self)[0]
    assert bad.size == 0, f"{bad.size} of {ids.size} sampled sites differ, first ids {ids[bad[:5]].tolist()}"
    assert np.count_nonzero(new_self != old_self) > 0
    lat.close()


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
