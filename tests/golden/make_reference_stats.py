"""Statistics of the unmodified reference over independent seeds, for the
statistical parity test of the Philox GPU path (tests/test_gpu_statistics.py).

Runs ``oracle/_ref/spk_serial`` (the reference built from its own sources by
``oracle/ref/Makefile``, its own RandomPark / RanMars streams) with `sweep
color`, or `solve_style tree` with `sector yes` for the KMC configuration, for
NSEEDS seeds per configuration and records, from the last stats
row of each run, the energy (diag_style energy), the mean site value
(diag_style array i1 mean; Ising magnetisation 2*mean - 3) and the mean
cluster volume <N> (diag_style cluster).  Writes reference_stats.json.

    python tests/golden/make_reference_stats.py [--ref /path/to/spparks]
"""

from __future__ import annotations

import argparse
import json
import subprocess
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
NSEEDS = 64

CONFIGS = [
    dict(name="ising_sq4n_64_T3.0", app="ising", q=2, lattice="sq/4n", n=(64, 64, 1), T=3.0, run=50.0),
    dict(name="ising_sq4n_64_T2.0", app="ising", q=2, lattice="sq/4n", n=(64, 64, 1), T=2.0, run=50.0),
    dict(name="potts_sq8n_48_Q10_T0.4", app="potts", q=10, lattice="sq/8n", n=(48, 48, 1), T=0.4, run=20.0),
    dict(name="ising_sc6n_16_T4.0", app="ising", q=2, lattice="sc/6n", n=(16, 16, 16), T=4.0, run=20.0),
    # potts/neighonly on sc/26n (the C1 path): dt_sweep = 1/26, so run 19.5/26 is 19 sweeps
    dict(name="neighonly_sc26n_12_Q20_T0.5", app="potts/neighonly", q=20, lattice="sc/26n", n=(12, 12, 12),
         T=0.5, run=19.5 / 26),
    # rejection-free KMC with the tree solver over four sectors (the C3 path), run to t = 2
    dict(name="kmc_potts_sq8n_32_Q10_T0.8", app="potts", q=10, lattice="sq/8n", n=(32, 32, 1), T=0.8, run=2.0,
         kmc=True),
]


def script(cfg, seed):
    nx, ny, nz = cfg["n"]
    dim = 3 if cfg["lattice"].startswith("sc") else 2
    zrange = f"0 {nz}" if dim == 3 else "-0.5 0.5"
    app = "ising" if cfg["app"] == "ising" else f"{cfg['app']} {cfg['q']}"
    return [f"seed {seed}", f"app_style {app}", f"dimension {dim}", f"lattice {cfg['lattice']} 1.0",
            f"region box block 0 {nx} 0 {ny} {zrange}", "create_box box", "create_sites box",
            f"set site range 1 {cfg['q']}"] + (["solve_style tree", "sector yes"] if cfg.get("kmc") else
                                                  ["sweep color"]) + [f"temperature {cfg['T']}", "diag_style energy",
            "diag_style array i1 mean", "diag_style cluster", f"stats {cfg['run']}", f"run {cfg['run']}"]


def last_row(binary, lines):
    with tempfile.TemporaryDirectory(dir=str(ROOT / "oracle" / "_ref")) as d:
        (Path(d) / "in.case").write_text("\n".join(lines) + "\n")
        subprocess.run([str(binary), "-in", "in.case", "-screen", "none", "-log", "log.case"], cwd=d, check=True,
                       capture_output=True)
        text = (Path(d) / "log.case").read_text().splitlines()
    header, row = None, None
    for line in text:
        p = line.split()
        if p[:4] == ["Time", "Naccept", "Nreject", "Nsweeps"]:
            header = p
        elif header is not None and len(p) == len(header) and p[0][0].isdigit():
            row = p
    return dict(zip(header, row))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    args = ap.parse_args()
    subprocess.check_call(["make", "-s", "-C", str(ROOT / "oracle" / "ref"), "-j8", f"REF={Path(args.ref) / 'src'}"])
    binary = ROOT / "oracle" / "_ref" / "spk_serial"
    out = {"nseeds": NSEEDS, "configs": []}
    for cfg in CONFIGS:
        rows = [last_row(binary, script(cfg, 1000 + 7 * k)) for k in range(NSEEDS)]
        sweeps = {int(r["Nsweeps"]) for r in rows}
        # a colour sweep run has the same sweep count for every seed; a KMC
        # run ends at the same time, after a seed-dependent number of passes
        assert cfg.get("kmc") or len(sweeps) == 1, sweeps
        assert all(abs(float(r["Time"]) - cfg["run"]) < 1e-9 for r in rows) or not cfg.get("kmc")
        out["configs"].append({
            **cfg, "script": script(cfg, "SEED"), "nsweeps": None if cfg.get("kmc") else sweeps.pop(),
            "energy": [float(r["Energy"]) for r in rows],
            "mean_i1": [float(r["mean(i1)"]) for r in rows],
            "mean_volume": [float(r["<N>"]) for r in rows],
        })
        print(cfg["name"], "sweeps", out["configs"][-1]["nsweeps"], "mean energy",
              sum(out["configs"][-1]["energy"]) / NSEEDS)
    (HERE / "reference_stats.json").write_text(json.dumps(out, indent=1))
    print("wrote", HERE / "reference_stats.json")


if __name__ == "__main__":
    main()
