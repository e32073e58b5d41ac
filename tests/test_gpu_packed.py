"""GPU parity of the bit-packed (64 sites per uint64) Ising path on sc/6n:
identical lattices to the oracle and to the int8 path under the same Philox
draws, per sweep."""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    import spparks_gb300

    spparks_gb300.load_library()
    return spparks_gb300


def test_pack_roundtrip_and_energy(sg):
    nx, ny, nz = 128, 6, 4
    spin = oracle.init_spins(77, nx * ny * nz, 1, 2)
    lat = sg.Lattice("sc/6n", nx, ny, nz, "ising", 2, spin_bytes=-1, seed=77)
    lat.upload(spin)
    assert np.array_equal(lat.download(), spin)
    cfg = oracle.make_cfg("sc/6n", nx, ny, nz, "ising", 2)
    assert lat.energy() == oracle.energy(cfg, spin)


@pytest.mark.parametrize("nx,ny,nz,T", [(64, 8, 6, 4.5115), (128, 4, 4, 2.2557), (64, 6, 10, 0.0), (192, 4, 2, 9.0),
                                        (64, 4, 4, 1e30)])
def test_packed_matches_oracle_and_int8(sg, nx, ny, nz, T):
    seed = 4711
    n = nx * ny * nz
    spin = oracle.init_spins(seed, n, 1, 2)
    cfg = oracle.make_cfg("sc/6n", nx, ny, nz, "ising", 2, T, seed=seed)
    ref = spin.copy()
    na, nt, hashes = oracle.color_sweeps(cfg, ref, 0, 5)
    packed = sg.Lattice("sc/6n", nx, ny, nz, "ising", 2, spin_bytes=-1, seed=seed)
    plain = sg.Lattice("sc/6n", nx, ny, nz, "ising", 2, spin_bytes=1, seed=seed)
    for lat in (packed, plain):
        lat.set_temperature(T)
        lat.upload(spin)
    got = []
    for _ in range(5):
        packed.sweep(1)
        plain.sweep(1)
        a = packed.download()
        assert np.array_equal(a, plain.download())
        got.append(oracle.spin_hash(a))
    assert got == [int(h) for h in hashes]
    assert (packed.stats()["naccept"], packed.stats()["nattempt"]) == (na, nt)


def test_packed_rejects_bad_input(sg):
    with pytest.raises(sg.SpkGpuError):
        sg.Lattice("sc/6n", 96, 4, 4, "ising", 2, spin_bytes=-1)   # nx not a multiple of 64
    with pytest.raises(sg.SpkGpuError):
        sg.Lattice("sq/4n", 64, 64, 1, "ising", 2, spin_bytes=-1)  # packed is sc/6n only
    lat = sg.Lattice("sc/6n", 64, 2, 2, "ising", 2, spin_bytes=-1)
    bad = np.ones(256, dtype=np.int32)
    bad[100] = 3
    with pytest.raises(sg.SpkGpuError) as ei:
        lat.upload(bad)
    assert ei.value.code == -6


@pytest.mark.parametrize("lattice,nx,ny,nz,app,q,sb", [("sc/6n", 64, 4, 4, "ising", 2, -1), ("sc/6n", 64, 4, 4, "ising", 2, 1),
                                                       ("sq/8n", 32, 16, 1, "potts", 50, 2), ("sc/26n", 8, 8, 8, "potts", 100, 4)])
def test_device_init_matches_oracle(sg, lattice, nx, ny, nz, app, q, sb):
    lat = sg.Lattice(lattice, nx, ny, nz, app, q, spin_bytes=sb, seed=31337)
    lat.init_spins(1, q)
    assert np.array_equal(lat.download(), oracle.init_spins(31337, nx * ny * nz, 1, q))
