"""Statistical parity of the Philox GPU path with the unmodified reference:
over independent seeds, the final energy, magnetisation (mean site value, and
|m| = |2*mean - 3| for Ising) and mean cluster volume <N> of `sweep color`
runs agree with the reference's own runs (its RandomPark/RanMars streams;
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


@pytest.mark.parametrize("cfg", REF["configs"], ids=lambda c: c["name"])
def test_statistics_match_unmodified_reference(sg, cfg):
    nx, ny, nz = cfg["n"]
    got = {"energy": [], "mean_i1": [], "mean_volume": []}
    for k in range(REF["nseeds"]):
        lat = sg.Lattice(cfg["lattice"], nx, ny, nz, cfg["app"], cfg["q"], spin_bytes=1, seed=5000 + 11 * k)
        lat.set_temperature(cfg["T"])
        lat.init_spins(1, cfg["q"])
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
