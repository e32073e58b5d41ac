"""Pins the oracle restatement (oracle/spk_oracle.c) before it is trusted as
the GPU path's checker: against the published Philox known-answer vectors,
the reference's own example logs, and fixtures produced by the reference
itself (tests/golden/make_golden.py)."""

import numpy as np
import pytest

import oracle
from conftest import fixture_count

# Philox4x32-10 known-answer vectors published with the Random123 library
PHILOX_KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]


@pytest.mark.parametrize("ctr,key,expect", PHILOX_KAT)
def test_philox_known_answers(ctr, key, expect):
    assert oracle.philox(ctr, key) == expect


def cfg_from_case(case, rng=oracle.RNG_PHILOX, seed=None):
    return oracle.make_cfg(case["lattice"], case["nx"], case["ny"], case["nz"], case["app"], case["nspins"],
                           case["temperature"], case.get("nsector", 1), case.get("nloop", 1), rng,
                           case.get("seed", 0) if seed is None else seed, case.get("mask", False))


def test_neighbor_order_matches_reference_offsets():
    # CreateSites::offsets_2d/3d order: dx outer, dy, dz inner
    c = oracle.make_cfg("sq/4n", 8, 8)
    i = 3 + 8 * 4
    assert oracle.neighbors(c, i) == [2 + 32, 3 + 24, 3 + 40, 4 + 32]
    c6 = oracle.make_cfg("sc/6n", 4, 4, 4)
    i = 1 + 4 * (1 + 4 * 1)
    x, y, z = 1, 1, 1
    idx = lambda a, b, d: a + 4 * (b + 4 * d)
    assert oracle.neighbors(c6, i) == [idx(0, 1, 1), idx(1, 0, 1), idx(1, 1, 0), idx(1, 1, 2), idx(1, 2, 1),
                                       idx(2, 1, 1)]
    c26 = oracle.make_cfg("sc/26n", 4, 4, 4)
    nb = oracle.neighbors(c26, 0)
    assert len(nb) == 26 and nb[0] == idx(3, 3, 3) and nb[-1] == idx(1, 1, 1)


@pytest.mark.parametrize("k", range(fixture_count("sweeps")))
def test_sweeps_match_reference(ref_fixtures, k):
    fx = ref_fixtures["sweeps"][k]
    case = fx["case"]
    cfg = cfg_from_case(case)
    spin = np.array(fx["snaps"]["init"]["spins"], dtype=np.int32)
    assert spin.tolist() == oracle.init_spins(case["seed"], spin.size, 1, case["nspins"]).tolist()
    mask = np.zeros(spin.size, dtype=np.uint8) if case.get("mask") else None
    na, nt, hashes = oracle.color_sweeps(cfg, spin, 0, case["nsweeps"], mask=mask)
    ref = fx["sweeps"]
    assert [format(int(h), "016x") for h in hashes] == [r[3] for r in ref]
    assert na == ref[-1][1] and nt == ref[-1][2]
    assert spin.tolist() == fx["snaps"]["final"]["spins"]


@pytest.mark.parametrize("k", range(fixture_count("ensemble")))
def test_ensemble_replicas_match_reference(ref_fixtures, k):
    """a replica of a batched ensemble (its own Philox stream word) against
    the reference driven by that stream"""
    fx = ref_fixtures["ensemble"][k]
    case = fx["case"]
    cfg = oracle.make_cfg(case["lattice"], case["nx"], case["ny"], case["nz"], case["app"], case["nspins"],
                          case["temperature"], seed=case["seed"], stream_base=case["stream_base"])
    spin = np.array(fx["snaps"]["init"]["spins"], dtype=np.int32)
    assert spin.tolist() == oracle.init_spins(case["init_seed"], spin.size, 1, case["nspins"]).tolist()
    na, nt, hashes = oracle.color_sweeps(cfg, spin, 0, case["nsweeps"])
    assert [format(int(h), "016x") for h in hashes] == [r[3] for r in fx["sweeps"]]
    assert na == fx["sweeps"][-1][1] and nt == fx["sweeps"][-1][2]
    assert spin.tolist() == fx["snaps"]["final"]["spins"]


@pytest.mark.parametrize("lattice,nx,ny,nz,app,q,T", [
    ("sc/6n", 8, 8, 8, "ising", 2, 4.5), ("sq/4n", 16, 8, 1, "ising", 2, 2.0), ("sq/8n", 16, 16, 1, "potts", 5, 1.0),
    ("sc/26n", 6, 6, 6, "potts/neighonly", 9, 0.5), ("sq/4n", 8, 8, 1, "potts/neigh", 6, 0.7)])
def test_single_site_updates_reproduce_a_colour_sweep(lattice, nx, ny, nz, app, q, T):
    """the oracle's single-site rule, given each site's value and the values
    its neighbours hold at its turn (lower colours already swept), gives the
    same lattice as the oracle's whole colour sweep: the basis of the sampled
    checks of lattices too large for a full oracle run"""
    cfg = oracle.make_cfg(lattice, nx, ny, nz, app, q, T, seed=11)
    n = nx * ny * nz
    s0 = oracle.init_spins(11, n, 1, q)
    s1 = s0.copy()
    oracle.color_sweeps(cfg, s1, 3, 1)
    ids = np.arange(n)
    nb = oracle.neighbors_many(cfg, ids)
    col = np.array([oracle.lib().spko_color(cfg, int(i)) for i in ids])
    seen = np.where(col[nb] < col[:, None], s1[nb], s0[nb])
    assert np.array_equal(oracle.site_updates(cfg, ids, s0, seen, 3), s1)


@pytest.mark.parametrize("k", range(5))
def test_kmc_matches_reference(ref_fixtures, k):
    fx = ref_fixtures["kmc"][k]
    case = fx["case"]
    cfg = cfg_from_case(case)
    cfg.nsector = 4 if case["lattice"].startswith("sq") else 8
    spin = np.array(fx["snaps"]["init"]["spins"], dtype=np.int32)
    km = oracle.Kmc(cfg)
    recs = []
    for r, t in enumerate(case["runs"]):
        npass, hashes, times = km.run(spin, t)
        recs += [(format(int(h), "016x"), float(tm)) for h, tm in zip(hashes, times)]
        assert spin.tolist() == fx["snaps"][f"run{r}"]["spins"]
    ref = fx["sweeps"]
    assert [h for h, _ in recs] == [r[3] for r in ref]
    for (_, tm), r in zip(recs, ref):
        assert tm == pytest.approx(r[4], rel=1e-12)
    assert km.naccept == ref[-1][1]


@pytest.mark.parametrize("k", range(3))
def test_strict_matches_unmodified_reference(ref_fixtures, k):
    """sweep color/strict with the reference's own RanMars/Park-Miller seeding:
    ranmaster draw 1 -> set site range, 2-3 -> ranapp, 4-5 -> ranstrict and the
    per-site seeds (src/app_lattice.cpp:274-295, src/set.cpp:598-624)."""
    fx = ref_fixtures["strict"][k]
    case = fx["case"]
    cfg = cfg_from_case(case, rng=oracle.RNG_STRICT, seed=0)
    n = case["nx"] * case["ny"] * case["nz"]
    u = oracle.ranmars_draws(case["master_seed"], 5)
    spin = oracle.set_range(oracle.park_seed(u[0]), n, 1, case["nspins"])
    assert spin.tolist() == fx["snaps"]["init"]["spins"]
    seeds = oracle.strict_siteseeds(u[4], n)
    sweep = 0
    for r in range(case["nruns"]):
        oracle.color_sweeps(cfg, spin, sweep, case["sweeps_per_run"], siteseeds=seeds)
        sweep += case["sweeps_per_run"]
        assert spin.tolist() == fx["snaps"][f"run{r}"]["spins"]
        assert oracle.energy(cfg, spin) == fx["energies"][r]


def example_run(example_logs, which, rows):
    """Reproduces the reference example (sweep random + sector yes, T=0) with the
    oracle's RanMars/Park-Miller restatement: ranmaster draw 1 -> set site range,
    draws 2-3 -> ranapp (src/app_lattice.cpp:274-278)."""
    if which == "ising":
        cfg = oracle.make_cfg("sq/4n", 50, 50, 1, "ising", 2, 0.0, nsector=4)
        q = 2
    else:
        cfg = oracle.make_cfg("sc/26n", 20, 20, 20, "potts", 100, 0.0, nsector=8)
        q = 100
    n = oracle.nsites(cfg)
    u = oracle.ranmars_draws(56789, 3)
    spin = oracle.set_range(oracle.park_seed(u[0]), n, 1, q)
    # ranapp = RandomPark(u[1]) then reset(u[2], me=0, 100): the reset wins
    ranapp = np.array([oracle.lib().spko_park_reset(u[2], 0, 100)], dtype=np.int32)
    log = example_logs[which]["rows"]
    assert oracle.energy(cfg, spin) == log[0]["energy"]
    done = 0
    na = oracle.ctypes.c_int64(0)
    nt = oracle.ctypes.c_int64(0)
    for row in log[1:rows + 1]:
        oracle.lib().spko_random_sector_sweeps(oracle.ctypes.byref(cfg), oracle._ptr(spin, oracle.ctypes.c_int32),
                                               oracle._ptr(ranapp, oracle.ctypes.c_int32), row["nsweeps"] - done,
                                               oracle.ctypes.byref(na), oracle.ctypes.byref(nt))
        done = row["nsweeps"]
        assert (na.value, nt.value - na.value) == (row["naccept"], row["nreject"])
        assert oracle.energy(cfg, spin) == row["energy"]


def test_example_log_ising(example_logs):
    example_run(example_logs, "ising", 10)


def test_example_log_potts(example_logs):
    example_run(example_logs, "potts", 2)


def parse_diag_script(lines):
    """Lattice, app and diagnostics of a diag log case script."""
    spec = {"diags": []}
    for line in lines:
        w = line.split()
        if w[0] == "seed":
            spec["seed"] = int(w[1])
        elif w[0] == "app_style":
            spec["app"] = w[1]
            spec["q"] = int(w[2]) if len(w) > 2 else 2
        elif w[0] == "lattice":
            spec["lattice"] = w[1]
        elif w[0] == "region":
            b = [float(v) for v in w[3:9]]
            spec["n"] = (int(b[1] - b[0]), int(b[3] - b[2]), max(1, int(b[5] - b[4])))
        elif w[0] == "temperature":
            spec["T"] = float(w[1])
        elif w[0] == "diag_style":
            if w[1] == "array":
                spec["diags"] += [("array", w[k], w[k + 1]) for k in range(2, len(w), 2)]
            else:
                spec["diags"].append((w[1],))
    return spec


def diag_tokens(cfg, spin, diags):
    """The diag columns the reference prints (%10g / %10d) for a lattice."""
    out = []
    for d in diags:
        if d[0] == "energy":
            out.append("%g" % oracle.energy(cfg, spin))
        elif d[0] == "cluster":
            c = oracle.clusters(cfg, spin)
            out += ["%d" % c["ncluster"], "%g" % c["mean_volume"], "%g" % c["mean_radius"]]
        else:
            v = {"mean": float(np.sum(spin, dtype=np.int64)) / spin.size, "sum": float(np.sum(spin, dtype=np.int64)),
                 "min": float(spin.min()), "max": float(spin.max())}[d[2]]
            out.append("%g" % v)
    return out


@pytest.mark.parametrize("k", range(3))
def test_diagnostics_match_unmodified_reference_log(ref_fixtures, k):
    """energy, `diag_style array` and `diag_style cluster` columns of an
    unmodified reference run (sweep color/strict) from the oracle: the t = 0
    row pins the cluster analysis on the `set site range` lattice, the later
    rows on the lattices the strict sweeps produce."""
    fx = ref_fixtures["diag_logs"][k]
    sp = parse_diag_script(fx["case"]["lines"])
    nx, ny, nz = sp["n"]
    cfg = oracle.make_cfg(sp["lattice"], nx, ny, nz, sp["app"], sp["q"], sp["T"], rng=oracle.RNG_STRICT, seed=0)
    n = nx * ny * nz
    u = oracle.ranmars_draws(sp["seed"], 5)
    spin = oracle.set_range(oracle.park_seed(u[0]), n, 1, sp["q"])
    seeds = oracle.strict_siteseeds(u[4], n)
    done = naccept = nattempt = 0
    for row in fx["rows"]:
        sweeps = int(row[3]) - done
        if sweeps:
            na, nt, _ = oracle.color_sweeps(cfg, spin, done, sweeps, siteseeds=seeds)
            naccept, nattempt, done = naccept + na, nattempt + nt, done + sweeps
        assert [int(row[1]), int(row[2])] == [naccept, nattempt - naccept]
        assert diag_tokens(cfg, spin, sp["diags"]) == row[5:], fx["case"]["name"]


def test_ising_sweep_takes_one_word_per_site():
    """At kT = 1e30 every Ising move is accepted (floor(exp(-dE/T) 2^31) = 2^31), so after one sweep site s
    holds the proposal of its own word: word s&3 of the block with counter (s>>2, s>>34, sweep, pass), value 1
    iff the word is below 2^31.  Rows of 6 sites make blocks straddle rows."""
    seed = 4242
    c = oracle.make_cfg("sq/4n", 6, 4, 1, "ising", 2, 1e30, seed=seed)
    spin = np.full(24, 2, dtype=np.int32)
    oracle.color_sweeps(c, spin, 7, 1)
    want = [1 if oracle.philox([s >> 2, 0, 7, 0], [seed, 0])[s & 3] < 2**31 else 2 for s in range(24)]
    assert spin.tolist() == want


def test_potts_sweep_takes_two_words_per_site():
    """The Potts-family apps keep two words per site: at kT = 1e30 site s proposes
    (int)(Q (x+1) 2^-32) + 1 from word 2(s&1) of the block with counter (s>>1, s>>33, sweep, pass)."""
    seed, q = 99, 5
    c = oracle.make_cfg("sq/4n", 6, 4, 1, "potts", q, 1e30, seed=seed)
    spin = np.full(24, 1, dtype=np.int32)
    oracle.color_sweeps(c, spin, 3, 1)
    want = [min(q, (q * (oracle.philox([s >> 1, 0, 3, 0], [seed, 0])[2 * (s & 1)] + 1)) // 2**32 + 1)
            for s in range(24)]
    assert spin.tolist() == want
