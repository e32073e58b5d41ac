"""Statistical parity of the Philox GPU path with the unmodified reference:
over independent seeds, the final energy, magnetisation (mean site value, and
|m| = |2*mean - 3| for Ising) and mean cluster volume <N> of `sweep color`
runs (ising, potts, potts/neighonly) and of tree-KMC runs over sectors agree
with the reference's own runs (its RandomPark/RanMars streams;
tests/golden/reference_stats.json, made by make_reference_stats.py) within
three standard errors of the difference of the two sample means."""

import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_stats.json"
REF = json.loads(GOLDEN.read_text())


@pytest.fixture(scope="module")
def sg():
    import spparks_gb300

    spparks_gb300.load_library()
    return spparks_gb300


def within_3_sigma(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    se = np.sqrt(a.var(ddof=1) / a.size + b.var(ddof=1) / b.size)
    return abs(a.mean() - b.mean()) <= 3.0 * se, a.mean(), b.mean(), se


CASES = [(c, None) for c in REF["configs"] if not c.get("kmc")] + \
        [(c, fp64) for c in REF["configs"] if c.get("kmc") for fp64 in (True, False)]


@pytest.mark.parametrize("cfg,fp64", CASES,
                         ids=lambda v: v["name"] if isinstance(v, dict) else ("" if v is None else f"fp64={v}"))
def test_statistics_match_unmodified_reference(sg, cfg, fp64):
    """colour sweeps for the sweep configurations; for the tree-KMC one, runs
    to the same time with FP64 propensities and with FP32 propensities (FP64
    tree sums and clock)"""
    nx, ny, nz = cfg["n"]
    got = {"energy": [], "mean_i1": [], "mean_volume": []}
    for k in range(REF["nseeds"]):
        kmc = cfg.get("kmc", False)
        lat = sg.Lattice(cfg["lattice"], nx, ny, nz, cfg["app"], cfg["q"], spin_bytes=1, seed=5000 + 11 * k,
                         nsector=4 if kmc else 1)
        lat.set_temperature(cfg["T"])
        lat.init_spins(1, cfg["q"])
        if kmc:
            lat.kmc_setup(fp64=fp64)
            assert lat.kmc_run(0.0, cfg["run"])["time"] == pytest.approx(cfg["run"], rel=1e-12)
        else:
            lat.sweep(cfg["nsweeps"])
        got["energy"].append(lat.energy())
        got["mean_i1"].append(lat.site_stats()["mean"])
        got["mean_volume"].append(lat.clusters()["mean_volume"])
        lat.close()
    checks = {key: within_3_sigma(got[key], cfg[key]) for key in got}
    if cfg["app"] == "ising":
        checks["|m|"] = within_3_sigma(np.abs(2 * np.asarray(got["mean_i1"]) - 3),
                                       np.abs(2 * np.asarray(cfg["mean_i1"]) - 3))
    bad = {k: v[1:] for k, v in checks.items() if not v[0]}
    assert not bad, f"{cfg['name']}: (gpu mean, reference mean, standard error) {bad}"
