"""GPU parity of the fused sq/4n tile sweep and of the batched ensemble
(persistent cooperative kernel, graph replays, on-device replica exchange)
against the oracle."""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    import spparks_gb300

    spparks_gb300.load_library()
    return spparks_gb300


@pytest.mark.parametrize("app,q,T", [("ising", 2, 2.269), ("potts", 20, 0.7), ("potts/neighonly", 9, 0.4),
                                     ("potts/neigh", 5, 1.1), ("ising", 2, 0.0), ("ising", 2, 1e30),
                                     ("potts", 7, 0.0), ("potts/neighonly", 5, 0.0)])
@pytest.mark.parametrize("nx,ny,sb", [(64, 64, 1), (96, 96, 1), (96, 32, 2), (32, 64, 4)])
def test_fused_tile_sweep_matches_oracle(sg, app, q, T, nx, ny, sb):
    seed = 8642
    spin = oracle.init_spins(seed, nx * ny, 1, q)
    cfg = oracle.make_cfg("sq/4n", nx, ny, 1, app, q, T, seed=seed)
    ref = spin.copy()
    na, nt, hashes = oracle.color_sweeps(cfg, ref, 0, 6)
    lat = sg.Lattice("sq/4n", nx, ny, 1, app, q, spin_bytes=sb, seed=seed, variant=2)
    lat.set_temperature(T)
    lat.upload(spin)
    got = []
    for _ in range(6):
        lat.sweep(1)
        got.append(oracle.spin_hash(lat.download()))
    assert got == [int(h) for h in hashes]
    st = lat.stats()
    assert (st["naccept"], st["nattempt"]) == (na, nt)
    # the fused path issues one launch per sweep
    assert lat.launch_count() <= 2 + 6 + 6


@pytest.mark.parametrize("app,q,T", [("ising", 2, 2.269), ("potts", 20, 0.7), ("potts/neighonly", 9, 0.4),
                                     ("potts/neigh", 5, 1.1), ("ising", 2, 0.0), ("ising", 2, 1e30)])
@pytest.mark.parametrize("nx,ny,sb", [(32, 32, 1), (64, 96, 2), (128, 128, 4), (96, 64, 1)])
def test_resident_sweeps_match_oracle(sg, app, q, T, nx, ny, sb):
    """sq/4n lattices that fit one CTA's shared memory: every sweep of a
    call in one launch (calls of 1, 5 and 4 sweeps), equal to the oracle at
    the end of each call, with the same change and attempt counts"""
    seed = 4321
    spin = oracle.init_spins(seed, nx * ny, 1, q)
    cfg = oracle.make_cfg("sq/4n", nx, ny, 1, app, q, T, seed=seed)
    ref = spin.copy()
    na, nt, hashes = oracle.color_sweeps(cfg, ref, 0, 10)
    lat = sg.Lattice("sq/4n", nx, ny, 1, app, q, spin_bytes=sb, seed=seed)
    lat.set_temperature(T)
    lat.upload(spin)
    done = 0
    for calls in (1, 5, 4):
        before = lat.launch_count()
        lat.sweep(calls)
        assert lat.launch_count() - before == 1  # one launch per call
        done += calls
        assert oracle.spin_hash(lat.download()) == int(hashes[done - 1]), (calls, done)
    st = lat.stats()
    assert (st["naccept"], st["nattempt"]) == (na, nt)
    lat.close()


def ensemble_case(seed=777):
    L = [32, 64, 32, 96, 64, 32, 64]
    T = [2.0, 2.5, 3.1, 1.7, 1.9, 2.6, 3.3]
    spins = [oracle.init_spins(seed + r, l * l, 1, 2) for r, l in enumerate(L)]
    return L, T, spins


@pytest.fixture(params=["persistent", "launches", "launches2", "launches4", "warps"])
def mode(request, monkeypatch):
    """every execution form of the ensemble, forced past the autotuner (the
    warp form is Ising only: a Potts ensemble then takes the autotuner's)"""
    monkeypatch.setenv("SPKGPU_ENSEMBLE_MODE", request.param)
    return request.param


@pytest.mark.parametrize("every,nsweeps,chunks", [(0, 7, [3, 4]), (2, 8, [2, 6]), (3, 12, [12]), (1, 5, [2, 3]),
                                                  (4, 13, [3, 2, 8])])
def test_ensemble_matches_oracle(sg, mode, every, nsweeps, chunks):
    L, T, spins = ensemble_case()
    seed = 99
    ens = sg.Ensemble(L, T, "ising", 2, seed=seed, exchange_every=every)
    assert ens.mode()["mode"] == mode
    ens.upload(np.concatenate(spins))
    ref = [s.copy() for s in spins]
    orc = oracle.EnsembleOracle(L, T, "ising", 2, seed=seed, every=every)
    for c in chunks:
        ens.run(c)
        orc.run(ref, c)
    got = ens.download()
    for r in range(len(L)):
        assert np.array_equal(ens.replica(got, r), ref[r]), f"replica {r}"
    st = ens.stats()
    assert st["naccept"] == orc.naccept
    assert st["nattempt"] == sum(l * l for l in L) * nsweeps
    assert (st["exchange_tries"], st["exchange_accepts"]) == (orc.tries, orc.accepts)
    assert ens.temperatures().tolist() == orc.temperatures()
    if every:
        assert ens.energies().tolist() == orc.last_bonds


def test_ensemble_potts(sg, mode):
    L = [32, 64, 64]
    T = [0.6, 0.9, 0.8]
    spins = [oracle.init_spins(5 + r, l * l, 1, 12) for r, l in enumerate(L)]
    ens = sg.Ensemble(L, T, "potts", 12, seed=4, exchange_every=2)
    ens.upload(np.concatenate(spins))
    orc = oracle.EnsembleOracle(L, T, "potts", 12, seed=4, every=2)
    ref = [s.copy() for s in spins]
    ens.run(6)
    orc.run(ref, 6)
    got = ens.download()
    for r in range(3):
        assert np.array_equal(ens.replica(got, r), ref[r])
    assert ens.temperatures().tolist() == orc.temperatures()
    assert ens.stats()["naccept"] == orc.naccept


def test_autotuner_times_both_forms_then_caches(sg, monkeypatch):
    monkeypatch.delenv("SPKGPU_ENSEMBLE_MODE", raising=False)
    L, T = [64, 96, 32, 64, 32], [1.8, 2.2, 2.6, 3.0, 3.4]  # a replica set no other test uses
    first = sg.Ensemble(L, T, "ising", 2, seed=1, exchange_every=5).mode()
    assert first["mode"] in sg.ENSEMBLE_MODES
    assert all(v is not None and v > 0 for v in first["tune_ms"].values())
    again = sg.Ensemble(L, T, "ising", 2, seed=2, exchange_every=5).mode()
    assert again["mode"] == first["mode"]
    assert all(v is None for v in again["tune_ms"].values())  # cached: nothing timed


def test_ensemble_extreme_temperatures(sg, mode):
    """thresholds at both ends in every execution form: kT = 0.01 (every
    uphill threshold 0) and 1e30 (exp(-dE/kT) rounds to 1: threshold 2^32,
    every draw passes), with exchanges between them"""
    L = [64, 32, 64, 32]
    T = [0.01, 1e30, 50.0, 1.5]
    spins = [oracle.init_spins(60 + r, l * l, 1, 2) for r, l in enumerate(L)]
    ens = sg.Ensemble(L, T, "ising", 2, seed=12, exchange_every=2)
    ens.upload(np.concatenate(spins))
    orc = oracle.EnsembleOracle(L, T, "ising", 2, seed=12, every=2)
    ref = [x.copy() for x in spins]
    ens.run(6)
    orc.run(ref, 6)
    got = ens.download()
    for r in range(len(L)):
        assert np.array_equal(ens.replica(got, r), ref[r]), f"replica {r}"
    assert ens.stats()["naccept"] == orc.naccept
    assert ens.temperatures().tolist() == orc.temperatures()
    ens.close()


def test_ensemble_rejects_bad_sizes(sg):
    with pytest.raises(sg.SpkGpuError):
        sg.Ensemble([48], [2.0])
    with pytest.raises(sg.SpkGpuError):
        sg.Ensemble([32], [0.0])


def test_run_io_pipeline_equals_sequential_steps(sg):
    """spkgpu_ensemble_run_io with page-locked buffers: three overlapping
    steps, each from its own input, give the outputs, counters and
    temperatures of upload / run / download in turn; pageable buffers take
    the sequential path with the same results"""
    import torch

    L, T = [64, 32, 96, 64], [1.9, 2.3, 2.7, 3.1]
    n = sum(l * l for l in L)
    inputs = [oracle.init_spins(40 + k, n, 1, 2) for k in range(3)]
    seq = sg.Ensemble(L, T, "ising", 2, seed=8, exchange_every=3)
    want = []
    for x in inputs:
        seq.upload(x)
        seq.run(6)
        want.append(seq.download().tolist())
    want_state = (seq.stats(), seq.temperatures().tolist())
    seq.close()
    for pinned in (True, False):
        ens = sg.Ensemble(L, T, "ising", 2, seed=8, exchange_every=3)
        if pinned:
            ins = [torch.from_numpy(x.copy()).pin_memory().numpy() for x in inputs]
            outs = [torch.zeros(n, dtype=torch.int32).pin_memory().numpy() for _ in inputs]
        else:
            ins = [x.copy() for x in inputs]
            outs = [np.zeros(n, dtype=np.int32) for _ in inputs]
        for x, y in zip(ins, outs):
            ens.run_io(x, y, 6)
        ens.synchronize()
        assert [y.tolist() for y in outs] == want
        assert (ens.stats(), ens.temperatures().tolist()) == want_state
        ens.close()


def test_run_io_reports_invalid_input_at_synchronize(sg):
    import torch

    L, T = [32, 64], [2.0, 2.5]
    n = sum(l * l for l in L)
    x = torch.from_numpy(oracle.init_spins(5, n, 1, 2)).pin_memory()
    x[17] = 3
    y = torch.zeros(n, dtype=torch.int32).pin_memory()
    ens = sg.Ensemble(L, T, "ising", 2, seed=8, exchange_every=0)
    ens.run_io(x.numpy(), y.numpy(), 2)
    with pytest.raises(sg.SpkGpuError) as ei:
        ens.synchronize()
    assert ei.value.code == -6  # SPKGPU_ERR_INVALID_SPIN
    ens.synchronize()  # the flag is cleared once reported
    ens.close()


def test_ensemble_replicas_match_reference_fixtures(sg, ref_fixtures, monkeypatch):
    """replicas of one ensemble (no exchange) against the reference built
    with the Philox shim and driven by each replica's stream word: every
    execution form, the headline warp tile included, bit-identical after
    every sweep"""
    fxs = ref_fixtures["ensemble"]
    cases = [fx["case"] for fx in fxs]
    L = [c["nx"] for c in cases]
    T = [c["temperature"] for c in cases]
    assert all(c["stream_base"] == (r + 1) << 8 and c["seed"] == cases[0]["seed"] for r, c in enumerate(cases))
    init = np.concatenate([np.array(fx["snaps"]["init"]["spins"], dtype=np.int32) for fx in fxs])
    nsweeps = cases[0]["nsweeps"]
    for mode in sg.ENSEMBLE_MODES:
        monkeypatch.setenv("SPKGPU_ENSEMBLE_MODE", mode)
        ens = sg.Ensemble(L, T, "ising", 2, seed=cases[0]["seed"], exchange_every=0)
        assert ens.mode()["mode"] == mode
        ens.upload(init)
        for s in range(nsweeps):
            ens.run(1)
            out = ens.download()
            for r, fx in enumerate(fxs):
                assert format(oracle.spin_hash(ens.replica(out, r)), "016x") == fx["sweeps"][s][3], (mode, r, s)
        assert ens.stats()["naccept"] == sum(fx["sweeps"][-1][1] for fx in fxs)
        ens.close()


def test_persistent_grid_barrier_gives_up_and_reports_a_device_error(sg, monkeypatch):
    """The persistent form's grid barrier waits a bounded number of times.
    With SPKGPU_ENSEMBLE_BARRIER_TEST one CTA never arrives and the limit is
    2000 waits: the other CTAs give up, set the error word and leave, so the
    run ends on its own and spkgpu_ensemble_synchronize reports
    SPKGPU_ERR_DEVICE.  The context stays usable: a new ensemble on the same
    device then gives the oracle's results."""
    L, T = [64, 96, 128], [1.8, 2.3, 2.9]
    spins = [oracle.init_spins(90 + r, l * l, 1, 2) for r, l in enumerate(L)]
    monkeypatch.setenv("SPKGPU_ENSEMBLE_MODE", "persistent")
    monkeypatch.setenv("SPKGPU_ENSEMBLE_BARRIER_TEST", "2000,1")
    ens = sg.Ensemble(L, T, "ising", 2, seed=17, exchange_every=2)
    assert ens.mode()["mode"] == "persistent"
    ens.upload(np.concatenate(spins))
    with pytest.raises(sg.SpkGpuError) as ei:
        ens.run(4)
        ens.synchronize()
    assert ei.value.code == -7  # SPKGPU_ERR_DEVICE
    ens.close()
    monkeypatch.delenv("SPKGPU_ENSEMBLE_BARRIER_TEST")
    ens = sg.Ensemble(L, T, "ising", 2, seed=17, exchange_every=2)
    ens.upload(np.concatenate(spins))
    ens.run(4)
    got = ens.download()
    orc = oracle.EnsembleOracle(L, T, "ising", 2, seed=17, every=2)
    ref = [x.copy() for x in spins]
    orc.run(ref, 4)
    assert all(np.array_equal(ens.replica(got, r), ref[r]) for r in range(len(L)))
    assert ens.stats()["naccept"] == orc.naccept
    ens.close()
