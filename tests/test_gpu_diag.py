"""Device diagnostics against the oracle: site sum/min/max (diag_style array)
and connected-component clusters (diag_style cluster) for every lattice
style, site-value width and the bit-packed Ising layout, on initial and swept
lattices."""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    import spparks_gb300

    spparks_gb300.load_library()
    return spparks_gb300


CASES = [
    ("sq/4n", 64, 48, 1, "ising", 2, 1),
    ("sq/4n", 32, 32, 1, "potts", 3, 4),
    ("sq/8n", 40, 24, 1, "potts", 5, 2),
    ("sc/6n", 16, 12, 10, "ising", 2, 4),
    ("sc/6n", 64, 8, 6, "ising", 2, -1),   # bit-packed
    ("sc/26n", 12, 10, 8, "potts/neighonly", 6, 2),
    ("sq/4n", 2, 2, 1, "potts", 2, 4),     # neighbours wrap onto each other
    ("sq/8n", 8, 2, 1, "potts", 2, 4),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{c[1]}x{c[2]}x{c[3]}-{c[4]}-sb{c[6]}")
@pytest.mark.parametrize("T,sweeps", [(0.0, 0), (1.2, 6)])
def test_diagnostics_match_oracle(sg, case, T, sweeps):
    lattice, nx, ny, nz, app, q, sb = case
    seed = 24680
    n = nx * ny * nz
    spin = oracle.init_spins(seed, n, 1, q)
    cfg = oracle.make_cfg(lattice, nx, ny, nz, app, q, T, seed=seed)
    lat = sg.Lattice(lattice, nx, ny, nz, app, q, spin_bytes=sb, seed=seed)
    lat.set_temperature(T)
    lat.upload(spin)
    if sweeps:
        oracle.color_sweeps(cfg, spin, 0, sweeps)
        lat.sweep(sweeps)
        assert lat.download().tolist() == spin.tolist()
    st = lat.site_stats()
    assert (st["sum"], st["min"], st["max"]) == (int(spin.sum()), int(spin.min()), int(spin.max()))
    got, ref = lat.clusters(), oracle.clusters(cfg, spin)
    assert got["ncluster"] == ref["ncluster"]
    assert got["mean_volume"] == ref["mean_volume"]
    # <R>: sum of volume^(1/d) in a different order (per-block partial sums)
    assert got["mean_radius"] == pytest.approx(ref["mean_radius"], rel=1e-12)
    lat.close()


def test_single_cluster_and_all_distinct(sg):
    lat = sg.Lattice("sq/8n", 32, 32, 1, "potts", 1024, spin_bytes=4, seed=1)
    lat.upload(np.full(1024, 7, dtype=np.int32))
    c = lat.clusters()
    assert (c["ncluster"], c["mean_volume"], c["mean_radius"]) == (1, 1024.0, 32.0)
    lat.upload(np.arange(1, 1025, dtype=np.int32))
    c = lat.clusters()
    assert (c["ncluster"], c["mean_volume"], c["mean_radius"]) == (1024, 1.0, 1.0)
    lat.close()
