"""Generate the golden parity fixtures from the reference itself.

Runs the reference SPPARKS built from its own sources by ``oracle/ref/Makefile``
(``oracle/_ref/runner_philox``: stock apps and tree solver with a Philox
RandomPark shim; ``oracle/_ref/runner_plain`` and ``spk_serial``: unmodified)
on small cases and writes ``tests/golden/*.json``.  It also copies the
Naccept/Nreject/Energy columns of the reference's example logs
(examples/ising, examples/potts), which are the reference's own golden
vectors for its rejection path.

Usage (needs the reference sources; not run by the tests):
    python tests/golden/make_golden.py [--ref /path/to/spparks]
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

DT_SWEEP = {"ising": lambda q, z: 0.5, "potts": lambda q, z: 1.0 / q,
            "potts/neighonly": lambda q, z: 1.0 / z, "potts/neigh": lambda q, z: 1.0 / z}
MAXNEIGH = {"sq/4n": 4, "sq/8n": 8, "sc/6n": 6, "sc/26n": 26}


def geometry_lines(lattice, nx, ny, nz):
    if lattice.startswith("sq"):
        return ["dimension 2", f"lattice {lattice} 1.0", f"region box block 0 {nx} 0 {ny} -0.5 0.5",
                "create_box box", "create_sites box"]
    return ["dimension 3", f"lattice {lattice} 1.0", f"region box block 0 {nx} 0 {ny} 0 {nz}",
            "create_box box", "create_sites box"]


def app_line(app, q):
    return "app_style ising" if app == "ising" else f"app_style {app} {q}"


def run_time(case):
    """A run time that yields exactly case['nsweeps'] passes whatever the
    rounding of dt_sweep: stop half a sweep before the last one ends."""
    dt = DT_SWEEP[case["app"]](case["nspins"], MAXNEIGH[case["lattice"]])
    nloop = case.get("nloop", 1)
    return (case["nsweeps"] - 0.5) * dt * nloop


def sweep_script(case):
    c = case
    lines = ["seed 56789", app_line(c["app"], c["nspins"])]
    lines += geometry_lines(c["lattice"], c["nx"], c["ny"], c["nz"])
    if "init_seed" in c:
        lines += [f"#! seed {c['init_seed']}", f"#! init_spins 1 {c['nspins']}", "#! snap init",
                  f"#! seed {c['seed']}"]
    else:
        lines += [f"#! seed {c['seed']}", f"#! init_spins 1 {c['nspins']}", "#! snap init"]
    if "stream_base" in c:
        lines.append(f"#! stream {c['stream_base']}")
    lines.append("sweep color" + (" mask yes" if c.get("mask") else ""))
    if c.get("nsector", 1) > 1:
        s = "sector yes" if c["nsector"] in (4, 8) and not c.get("nsector_explicit") else f"sector {c['nsector']}"
        if c.get("nloop", 1) > 1:
            s += f" nstop {c['nloop']}"
        lines.append(s)
    lines.append(f"temperature {c['temperature']!r}")
    lines += ["#! record on", f"run {run_time(c)!r}", "#! snap final"]
    return lines


def kmc_script(case):
    c = case
    lines = ["seed 56789", app_line(c["app"], c["nspins"])]
    lines += geometry_lines(c["lattice"], c["nx"], c["ny"], c["nz"])
    lines += [f"#! seed {c['seed']}", f"#! init_spins 1 {c['nspins']}", "#! snap init",
              "solve_style tree", "sector yes", f"temperature {c['temperature']!r}", "#! record on"]
    for k, t in enumerate(c["runs"]):
        lines += [f"run {t!r}", f"#! snap run{k}"]
    return lines


def strict_script(case):
    c = case
    lines = ["seed %d" % c["master_seed"], app_line(c["app"], c["nspins"])]
    lines += geometry_lines(c["lattice"], c["nx"], c["ny"], c["nz"])
    lines += [f"set site range 1 {c['nspins']}", "#! snap init", "sweep color/strict",
              f"temperature {c['temperature']!r}"]
    dt = DT_SWEEP[c["app"]](c["nspins"], MAXNEIGH[c["lattice"]])
    for k in range(c["nruns"]):
        lines += [f"run {(c['sweeps_per_run'] - 0.5) * dt!r}", f"#! snap run{k}", "#! energy"]
    return lines


def parse_output(text):
    out = {"sweeps": [], "snaps": {}, "energies": []}
    for line in text.splitlines():
        p = line.split()
        if not p:
            continue
        if p[0] == "sweep":
            out["sweeps"].append([int(p[1]), int(p[2]), int(p[3]), p[4], float(p[5])])
        elif p[0] == "snap":
            n = int(p[3])
            out["snaps"][p[1]] = {"hash": p[2], "spins": [int(v) for v in p[4:4 + n]]}
        elif p[0] == "energy":
            out["energies"].append(float(p[1]))
    return out


def run_runner(binary, lines):
    with tempfile.NamedTemporaryFile("w", suffix=".in", delete=False, dir=str(ROOT / "oracle" / "_ref")) as f:
        f.write("\n".join(lines) + "\n")
        path = f.name
    try:
        res = subprocess.run([str(binary), path], capture_output=True, text=True, check=True,
                             cwd=str(ROOT / "oracle" / "_ref"))
    finally:
        os.unlink(path)
    return parse_output(res.stdout)


SWEEP_CASES = [
    dict(name="ising_sq4n_16_T2269", app="ising", nspins=2, lattice="sq/4n", nx=16, ny=16, nz=1,
         temperature=2.269, seed=56789, nsweeps=12),
    dict(name="ising_sq4n_16_T0", app="ising", nspins=2, lattice="sq/4n", nx=16, ny=12, nz=1,
         temperature=0.0, seed=11, nsweeps=6),
    dict(name="ising_sc6n_8_T22557", app="ising", nspins=2, lattice="sc/6n", nx=8, ny=6, nz=4,
         temperature=2.2557, seed=99, nsweeps=6),
    dict(name="potts_sq8n_16_Q8", app="potts", nspins=8, lattice="sq/8n", nx=16, ny=16, nz=1,
         temperature=1.0, seed=7, nsweeps=8),
    dict(name="potts_sc26n_8_Q100", app="potts", nspins=100, lattice="sc/26n", nx=8, ny=8, nz=8,
         temperature=0.5, seed=5, nsweeps=4),
    dict(name="neighonly_sc26n_8_Q100", app="potts/neighonly", nspins=100, lattice="sc/26n", nx=8, ny=8,
         nz=8, temperature=0.5, seed=56789, nsweeps=6),
    dict(name="neighonly_sq8n_12_Q5", app="potts/neighonly", nspins=5, lattice="sq/8n", nx=12, ny=8,
         nz=1, temperature=0.3, seed=3, nsweeps=10),
    dict(name="neigh_sq4n_16_Q20", app="potts/neigh", nspins=20, lattice="sq/4n", nx=16, ny=16, nz=1,
         temperature=0.8, seed=21, nsweeps=8),
    dict(name="potts_sq4n_sector4_Q16", app="potts", nspins=16, lattice="sq/4n", nx=16, ny=16, nz=1,
         temperature=0.7, seed=4, nsweeps=5, nsector=4),
    dict(name="ising_sc26n_sector8", app="ising", nspins=2, lattice="sc/26n", nx=8, ny=8, nz=8,
         temperature=3.0, seed=8, nsweeps=3, nsector=8),
    dict(name="neighonly_sq4n_sector2_nstop2", app="potts/neighonly", nspins=10, lattice="sq/4n", nx=12,
         ny=8, nz=1, temperature=0.6, seed=12, nsweeps=4, nsector=2, nsector_explicit=True, nloop=2),
    dict(name="potts_sq4n_mask_sector4_T0", app="potts", nspins=4, lattice="sq/4n", nx=16, ny=16, nz=1,
         temperature=0.0, seed=13, nsweeps=6, nsector=4, mask=True),
    dict(name="ising_sq4n_mask_T1", app="ising", nspins=2, lattice="sq/4n", nx=8, ny=8, nz=1,
         temperature=1.0, seed=14, nsweeps=4, mask=True),
    # edge cases: periodic extents of 2 (a site meets the same neighbour site more than once) and Q = 1 (no
    # site can change)
    dict(name="ising_sq4n_2x2", app="ising", nspins=2, lattice="sq/4n", nx=2, ny=2, nz=1,
         temperature=2.0, seed=31, nsweeps=8),
    dict(name="potts_sq8n_2x2_Q5", app="potts", nspins=5, lattice="sq/8n", nx=2, ny=2, nz=1,
         temperature=1.0, seed=32, nsweeps=6),
    dict(name="neighonly_sc26n_2x2x2_Q10", app="potts/neighonly", nspins=10, lattice="sc/26n", nx=2, ny=2,
         nz=2, temperature=0.5, seed=33, nsweeps=6),
    dict(name="potts_sq4n_Q1", app="potts", nspins=1, lattice="sq/4n", nx=16, ny=16, nz=1,
         temperature=1.0, seed=34, nsweeps=3),
    dict(name="neighonly_sq8n_Q1", app="potts/neighonly", nspins=1, lattice="sq/8n", nx=8, ny=8, nz=1,
         temperature=0.5, seed=35, nsweeps=3),
    # lattices the int8 warp tile takes (sides multiples of 32): the single-lattice warp sweep is pinned to
    # the reference directly
    dict(name="ising_sq4n_64_T2269", app="ising", nspins=2, lattice="sq/4n", nx=64, ny=64, nz=1,
         temperature=2.269, seed=56789, nsweeps=8),
    dict(name="ising_sq4n_96x64_T19", app="ising", nspins=2, lattice="sq/4n", nx=96, ny=64, nz=1,
         temperature=1.9, seed=4242, nsweeps=6),
]

# replicas of a batched ensemble (no exchange): replica r draws from Philox stream word (r+1) << 8, so the
# ensemble's warp-tile sweep is pinned to the reference directly
ENSEMBLE_SEED = 31
ENSEMBLE_CASES = [
    dict(name="ensemble_r0_ising_64_T20", app="ising", nspins=2, lattice="sq/4n", nx=64, ny=64, nz=1,
         temperature=2.0, seed=ENSEMBLE_SEED, init_seed=701, stream_base=1 << 8, nsweeps=6),
    dict(name="ensemble_r1_ising_96_T26", app="ising", nspins=2, lattice="sq/4n", nx=96, ny=96, nz=1,
         temperature=2.6, seed=ENSEMBLE_SEED, init_seed=702, stream_base=2 << 8, nsweeps=6),
    dict(name="ensemble_r2_ising_32_T15", app="ising", nspins=2, lattice="sq/4n", nx=32, ny=32, nz=1,
         temperature=1.5, seed=ENSEMBLE_SEED, init_seed=703, stream_base=3 << 8, nsweeps=6),
]

KMC_CASES = [
    dict(name="kmc_potts_sq8n_16_Q10", app="potts", nspins=10, lattice="sq/8n", nx=16, ny=16, nz=1,
         temperature=1.0, seed=31, runs=[1.5, 0.75]),
    dict(name="kmc_ising_sq4n_16", app="ising", nspins=2, lattice="sq/4n", nx=16, ny=16, nz=1,
         temperature=2.0, seed=32, runs=[2.0]),
    dict(name="kmc_potts_sc26n_8_Q50", app="potts", nspins=50, lattice="sc/26n", nx=8, ny=8, nz=8,
         temperature=0.8, seed=33, runs=[0.6]),
    # edge cases: Q = 1 (every propensity zero: one pass, nothing changes) and a 4x4 lattice (sectors of 2x2,
    # repeated neighbour sites)
    dict(name="kmc_potts_sq8n_8_Q1", app="potts", nspins=1, lattice="sq/8n", nx=8, ny=8, nz=1,
         temperature=1.0, seed=36, runs=[0.5]),
    dict(name="kmc_potts_sq8n_4x4_Q4", app="potts", nspins=4, lattice="sq/8n", nx=4, ny=4, nz=1,
         temperature=0.9, seed=37, runs=[1.0, 0.5]),
]

# tree KMC with stats and energy between passes (Philox shim): the log's rows
KMC_LOG_CASES = [
    dict(name="kmclog_potts_sq8n_16_Q10", app="potts", nspins=10, lattice="sq/8n", nx=16, ny=16, nz=1,
         temperature=1.0, seed=41, runs=[1.0, 0.5], stats=0.2),
    dict(name="kmclog_ising_sc6n_8", app="ising", nspins=2, lattice="sc/6n", nx=8, ny=8, nz=8,
         temperature=3.0, seed=42, runs=[0.6], stats=0.1),
]


def kmc_log_script(case):
    lines = kmc_script(case)
    k = lines.index("solve_style tree")
    return ["log kmc.log"] + lines[:k] + ["diag_style energy", f"stats {case['stats']!r}"] + lines[k:]


STRICT_CASES = [
    dict(name="strict_ising_sq4n_16", app="ising", nspins=2, lattice="sq/4n", nx=16, ny=16, nz=1,
         temperature=2.269, master_seed=56789, nruns=3, sweeps_per_run=4),
    dict(name="strict_neighonly_sc26n_6", app="potts/neighonly", nspins=100, lattice="sc/26n", nx=6,
         ny=6, nz=6, temperature=0.5, master_seed=4321, nruns=2, sweeps_per_run=3),
    dict(name="strict_potts_sq8n_12_Q4", app="potts", nspins=4, lattice="sq/8n", nx=12, ny=12, nz=1,
         temperature=0.9, master_seed=777, nruns=2, sweeps_per_run=5),
]


LOG_CASES = [
    dict(name="log_strict_ising_sq4n_50", lines=[
        "seed 56789", "app_style ising", "dimension 2", "lattice sq/4n 1.0", "region box block 0 50 0 50 -0.5 0.5",
        "create_box box", "create_sites box", "set site range 1 2", "sweep color/strict", "diag_style energy",
        "temperature 2.269", "stats 5.0", "run 50.0"]),
    dict(name="log_strict_neighonly_sc26n_12", lines=[
        "seed 4242", "app_style potts/neighonly 100", "dimension 3", "lattice sc/26n 1.0",
        "region box block 0 12 0 12 0 12", "create_box box", "create_sites box", "set site range 1 100",
        "sweep color/strict", "diag_style energy", "temperature 0.5", "stats 0.2", "run 1.0"]),
    dict(name="log_strict_potts_sq8n_20_two_runs", lines=[
        "seed 777", "app_style potts 8", "dimension 2", "lattice sq/8n 1.0", "region box block 0 20 0 20 -0.5 0.5",
        "create_box box", "create_sites box", "set site range 1 8", "sweep color/strict", "diag_style energy",
        "temperature 0.9", "stats 0.5", "run 2.0", "temperature 0.3", "run 1.0"]),
]


# unmodified reference runs with the site diagnostics: the t = 0 row pins the
# oracle's cluster analysis on the initial `set site range` lattice, every
# row pins the GPU driver's diag columns
DIAG_LOG_CASES = [
    dict(name="diag_strict_potts_sq8n_32", lines=[
        "seed 2468", "app_style potts 10", "dimension 2", "lattice sq/8n 1.0", "region box block 0 32 0 32 -0.5 0.5",
        "create_box box", "create_sites box", "set site range 1 10", "sweep color/strict", "diag_style energy",
        "diag_style array i1 mean i1 max", "diag_style cluster", "temperature 0.4", "stats 2.0", "run 10.0"]),
    dict(name="diag_strict_ising_sc6n_12", lines=[
        "seed 97531", "app_style ising", "dimension 3", "lattice sc/6n 1.0", "region box block 0 12 0 12 0 12",
        "create_box box", "create_sites box", "set site range 1 2", "sweep color/strict", "diag_style energy",
        "diag_style cluster", "diag_style array i1 mean", "temperature 3.0", "stats 1.0", "run 4.0"]),
    dict(name="diag_strict_ising_sq4n_40", lines=[
        "seed 1357", "app_style ising", "dimension 2", "lattice sq/4n 1.0", "region box block 0 40 0 40 -0.5 0.5",
        "create_box box", "create_sites box", "set site range 1 2", "sweep color/strict", "diag_style cluster",
        "diag_style array i1 sum i1 min", "temperature 1.5", "stats 5.0", "run 20.0"]),
]


# unmodified reference runs that write dumps (text and sites) or read a site
# file: the driver must write the same files and print the same stats
def _site_file():
    """a Values-only site file for a 12x12 lattice (values 1..5 by a fixed rule)"""
    rows = [f"{i + 1} {1 + (7 * i + (i // 12) * 3) % 5}" for i in range(144)]
    return "\n".join(["read_sites input", "", "2 dimension", "144 sites", "id site values",
                      "0 12 xlo xhi", "0 12 ylo yhi", "-0.5 0.5 zlo zhi", "", "Values", ""] + rows) + "\n"


IO_CASES = [
    dict(name="io_dump_strict_ising_sq4n_16", inputs={}, outputs=["dump.text", "sites.0.txt", "sites.1.txt",
                                                                  "sites.2.txt"], lines=[
        "seed 4321", "app_style ising", "dimension 2", "lattice sq/4n 1.0", "region box block 0 16 0 16 -0.5 0.5",
        "create_box box", "create_sites box", "set site range 1 2", "sweep color/strict", "temperature 2.0",
        "diag_style energy", "dump 1 text 2.0 dump.text id site x y z energy", "dump 2 sites 5.0 sites.*.txt id site",
        "stats 2.0", "run 10.0"]),
    dict(name="io_dump_strict_potts_sc26n_6", inputs={}, outputs=["d3.txt"], lines=[
        "seed 8642", "app_style potts 6", "dimension 3", "lattice sc/26n 1.0", "region box block 0 6 0 6 0 6",
        "create_box box", "create_sites box", "set site range 1 6", "sweep color/strict", "temperature 0.7",
        "dump 1 text 0.5 d3.txt id site energy", "dump_modify 1 delay 1.0", "stats 0.5", "run 2.0", "run 1.0"]),
    dict(name="io_read_sites_strict_potts_sq8n_12", inputs={"in.sites": _site_file()}, outputs=["final.0.txt"],
         lines=[
        "seed 97", "app_style potts 5", "dimension 2", "lattice sq/8n 1.0", "region box block 0 12 0 12 -0.5 0.5",
        "create_box box", "create_sites box", "read_sites in.sites", "sweep color/strict", "temperature 0.5",
        "diag_style energy", "stats 1.0", "dump 1 sites 3.0 final.*.txt id site", "dump_modify 1 delay 3.0",
        "run 3.0"]),
]


def spk_serial_io(binary, case):
    """Stats table and the written files of a reference run."""
    with tempfile.TemporaryDirectory(dir=str(ROOT / "oracle" / "_ref")) as d:
        for name, text in case["inputs"].items():
            (Path(d) / name).write_text(text)
        (Path(d) / "in.case").write_text("\n".join(case["lines"]) + "\n")
        subprocess.run([str(binary), "-in", "in.case", "-screen", "none", "-log", "log.case"], cwd=d, check=True,
                       capture_output=True)
        log = (Path(d) / "log.case").read_text()
        files = {name: (Path(d) / name).read_text() for name in case["outputs"]}
    header, rows = None, []
    for line in log.splitlines():
        p = line.split()
        if p[:4] == ["Time", "Naccept", "Nreject", "Nsweeps"]:
            header = p
            continue
        if header is not None and len(p) == len(header) and p[0][0].isdigit():
            rows.append(p[:4] + ["-"] + p[5:])  # CPU seconds vary from run to run
    return header, rows, files


def spk_serial_table(binary, lines):
    """Header tokens and the stats rows (as printed tokens) of a reference run."""
    with tempfile.TemporaryDirectory(dir=str(ROOT / "oracle" / "_ref")) as d:
        inp = Path(d) / "in.case"
        inp.write_text("\n".join(lines) + "\n")
        subprocess.run([str(binary), "-in", "in.case", "-screen", "none", "-log", "log.case"], cwd=d, check=True,
                       capture_output=True)
        text = (Path(d) / "log.case").read_text().splitlines()
    header, rows = None, []
    for line in text:
        p = line.split()
        if p[:4] == ["Time", "Naccept", "Nreject", "Nsweeps"]:
            header = p
            continue
        if header is not None:
            if len(p) == len(header) and p[0][0].isdigit():
                rows.append(p[:4] + ["-"] + p[5:])  # CPU seconds vary from run to run
                continue
            if rows:
                break
    return header, rows


def spk_serial_stats(binary, lines):
    """Stats rows (Time Naccept Nreject Nsweeps Energy) printed by the reference."""
    with tempfile.TemporaryDirectory(dir=str(ROOT / "oracle" / "_ref")) as d:
        inp = Path(d) / "in.case"
        inp.write_text("\n".join(lines) + "\n")
        subprocess.run([str(binary), "-in", "in.case", "-screen", "none", "-log", "log.case"], cwd=d, check=True,
                       capture_output=True)
        text = (Path(d) / "log.case").read_text().splitlines()
    rows, grab = [], False
    for line in text:
        p = line.split()
        if p[:4] == ["Time", "Naccept", "Nreject", "Nsweeps"]:
            grab = True
            continue
        if grab:
            if len(p) == 6:
                try:
                    rows.append([float(p[0]), int(p[1]), int(p[2]), int(p[3]), float(p[5])])
                    continue
                except ValueError:
                    pass
            grab = False
    return rows


def example_log_rows(path):
    rows = []
    lines = Path(path).read_text().splitlines()
    for k, line in enumerate(lines):
        if line.split()[:4] == ["Time", "Naccept", "Nreject", "Nsweeps"]:
            for row in lines[k + 1:]:
                p = row.split()
                if len(p) != 6:
                    break
                rows.append({"time": float(p[0]), "naccept": int(p[1]), "nreject": int(p[2]),
                             "nsweeps": int(p[3]), "energy": float(p[5])})
            break
    return rows


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    args = ap.parse_args()
    refsrc = Path(args.ref) / "src"
    subprocess.check_call(["make", "-s", "-C", str(ROOT / "oracle" / "ref"), "-j8", f"REF={refsrc}"])
    philox = ROOT / "oracle" / "_ref" / "runner_philox"
    plain = ROOT / "oracle" / "_ref" / "runner_plain"

    fixtures = {"sweeps": [], "kmc": [], "strict": [], "ensemble": []}
    for group, cases in (("sweeps", SWEEP_CASES), ("ensemble", ENSEMBLE_CASES)):
        for case in cases:
            lines = sweep_script(case)
            res = run_runner(philox, lines)
            assert len(res["sweeps"]) == case["nsweeps"], (case["name"], len(res["sweeps"]))
            fixtures[group].append({"case": case, "script": lines, **res})
            print(group, "case", case["name"], "final", res["snaps"]["final"]["hash"])
    for case in KMC_CASES:
        lines = kmc_script(case)
        res = run_runner(philox, lines)
        fixtures["kmc"].append({"case": case, "script": lines, **res})
        print("kmc case", case["name"], "passes", len(res["sweeps"]))
    for case in STRICT_CASES:
        lines = strict_script(case)
        res = run_runner(plain, lines)
        fixtures["strict"].append({"case": case, "script": lines, **res})
        print("strict case", case["name"], [res["snaps"][f"run{k}"]["hash"] for k in range(case["nruns"])])

    serial = ROOT / "oracle" / "_ref" / "spk_serial"
    fixtures["logs"] = []
    for case in LOG_CASES:
        rows = spk_serial_stats(serial, case["lines"])
        fixtures["logs"].append({"case": case, "rows": rows})
        print("log case", case["name"], len(rows), "rows")
    fixtures["diag_logs"] = []
    for case in DIAG_LOG_CASES:
        header, rows = spk_serial_table(serial, case["lines"])
        fixtures["diag_logs"].append({"case": case, "header": header, "rows": rows})
        print("diag log case", case["name"], header, len(rows), "rows")
    fixtures["kmc_logs"] = []
    for case in KMC_LOG_CASES:
        lines = kmc_log_script(case)
        res = run_runner(philox, lines)
        log = ROOT / "oracle" / "_ref" / "kmc.log"
        header, rows = None, []
        for line in log.read_text().splitlines():
            p = line.split()
            if p[:4] == ["Time", "Naccept", "Nreject", "Nsweeps"]:
                header = p
                continue
            if header is not None and len(p) == len(header) and p[0][0].isdigit():
                rows.append(p[:4] + ["-"] + p[5:])
        log.unlink()
        fixtures["kmc_logs"].append({"case": case, "script": lines, "header": header, "rows": rows, **res})
        print("kmc log case", case["name"], len(rows), "rows")
    fixtures["io"] = []
    for case in IO_CASES:
        header, rows, files = spk_serial_io(serial, case)
        fixtures["io"].append({"case": case, "header": header, "rows": rows, "files": files})
        print("io case", case["name"], len(rows), "rows", sorted(files))
    (HERE / "reference_philox.json").write_text(json.dumps(fixtures, indent=1))
    logs = {
        "ising": {"script": (Path(args.ref) / "examples/ising/in.ising").read_text().splitlines(),
                  "rows": example_log_rows(Path(args.ref) / "examples/ising/log.ising.11Nov09.linux.1")},
        "potts": {"script": (Path(args.ref) / "examples/potts/in.potts").read_text().splitlines(),
                  "rows": example_log_rows(Path(args.ref) / "examples/potts/log.potts.11Nov09.linux.1")},
    }
    (HERE / "example_logs.json").write_text(json.dumps(logs, indent=1))
    print("wrote", HERE / "reference_philox.json", HERE / "example_logs.json")


if __name__ == "__main__":
    main()
