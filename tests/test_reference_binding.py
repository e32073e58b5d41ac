"""The reference-side binding of the GB300 path: the GPU app styles of
spparks_gb300/reference_app (ising/gpu, potts/gpu, potts/neighonly/gpu),
compiled with the reference's own sources into oracle/_ref/spk_serial_gpu and
linked to libspkgpu.so, as a maintainer would add them to SPPARKS.

On the CPU: the binary builds and lists the three styles.  On the GPU: input
scripts run through the reference's own driver with a GPU style print the
same stats rows as the stock style (sweep color/strict, where the device
consumes the reference's own per-site Park-Miller seeds; CPU time column
excepted), and tree KMC over sectors and Philox colour sweeps run through the same
output schedule."""

import subprocess
import tempfile
from pathlib import Path

import pytest

import oracle

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def binaries():
    import spparks_gb300

    spparks_gb300.load_library()  # builds libspkgpu.so if needed
    if not (oracle.build_reference() and oracle.build_reference_gpu()):
        pytest.skip("no reference sources here to build the binding with")
    return oracle.REF_OUT / "spk_serial", oracle.REF_OUT / "spk_serial_gpu"


def test_binding_builds_and_registers_the_gpu_styles(binaries):
    _, gpu = binaries
    with tempfile.TemporaryDirectory() as d:
        out = subprocess.run([str(gpu), "-h"], cwd=d, capture_output=True, text=True).stdout
    line = next(l for l in out.splitlines() if l.startswith("App styles:"))
    for style in ("ising/gpu", "potts/gpu", "potts/neighonly/gpu", "ising", "potts"):
        assert style in line.split(), style


def stats_rows(binary, lines):
    """(header, rows) of the stats table a run of `lines` logs."""
    with tempfile.TemporaryDirectory() as d:
        (Path(d) / "in.case").write_text("\n".join(lines) + "\n")
        res = subprocess.run([str(binary), "-in", "in.case", "-screen", "none", "-log", "log.case"], cwd=d,
                             capture_output=True, text=True, timeout=600)
        assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
        text = (Path(d) / "log.case").read_text().splitlines()
    header, rows = None, []
    for line in text:
        p = line.split()
        if p[:4] == ["Time", "Naccept", "Nreject", "Nsweeps"]:
            header = p
        elif header is not None and len(p) == len(header) and p[0][0].isdigit():
            rows.append(p)
    return header, rows


def geometry(lattice, n):
    nx, ny, nz = n
    if lattice.startswith("sq"):
        return ["dimension 2", f"lattice {lattice} 1.0", f"region box block 0 {nx} 0 {ny} -0.5 0.5"]
    return ["dimension 3", f"lattice {lattice} 1.0", f"region box block 0 {nx} 0 {ny} 0 {nz}"]


STRICT_CASES = [
    dict(name="ising_sq4n_64", app="ising", lattice="sq/4n", n=(64, 64, 1), q=2, T=2.0, sweep="color/strict",
         run=[20.0, 10.0], stats=5.0),
    dict(name="potts_sq8n_48_Q10", app="potts 10", lattice="sq/8n", n=(48, 48, 1), q=10, T=0.4,
         sweep="color/strict", run=[8.0], stats=2.0),
    dict(name="neighonly_sc26n_12_Q20", app="potts/neighonly 20", lattice="sc/26n", n=(12, 12, 12), q=20, T=0.5,
         sweep="color/strict", run=[10 / 26], stats=4 / 26),
    dict(name="potts_sq4n_mask_T0", app="potts 4", lattice="sq/4n", n=(32, 32, 1), q=4, T=0.0,
         sweep="color/strict mask yes", run=[6.0], stats=1.0),
]


def case_lines(c, gpu):
    style, *args = c["app"].split()
    app = " ".join([style + ("/gpu" if gpu else "")] + args)
    lines = ["seed 56789", f"app_style {app}"] + geometry(c["lattice"], c["n"])
    lines += ["create_box box", "create_sites box", f"set site range 1 {c['q']}", f"sweep {c['sweep']}",
              f"temperature {c['T']}", "diag_style energy", "diag_style cluster", f"stats {c['stats']!r}"]
    lines += [f"run {t!r}" for t in c["run"]]
    return lines


@pytest.mark.gpu
@pytest.mark.parametrize("c", STRICT_CASES, ids=lambda c: c["name"])
def test_gpu_style_equals_stock_style_with_color_strict(binaries, c):
    stock, gpu = binaries
    h0, r0 = stats_rows(stock, case_lines(c, False))
    h1, r1 = stats_rows(gpu, case_lines(c, True))
    assert h0 == h1 and len(r0) == len(r1) > 1
    cpu = h0.index("CPU")
    def strip(rows):
        return [[v for k, v in enumerate(row) if k != cpu] for row in rows]

    assert strip(r0) == strip(r1)


@pytest.mark.gpu
def test_gpu_style_tree_kmc_and_color_sweeps_run(binaries):
    """tree KMC over sectors and Philox colour sweeps through the GPU styles:
    the runs start and end where the stock style's do and accept events"""
    stock, gpu = binaries
    base = ["seed 4321", "app_style {app}"] + geometry("sq/8n", (32, 32, 1)) + \
        ["create_box box", "create_sites box", "set site range 1 10"]
    kmc = base + ["solve_style tree", "sector yes", "temperature 0.8", "diag_style energy", "stats 0.25",
                  "run 1.0", "run 0.5"]
    h0, r0 = stats_rows(stock, [l.format(app="potts 10") for l in kmc])
    h1, r1 = stats_rows(gpu, [l.format(app="potts/gpu 10") for l in kmc])
    # the adaptive sector time follows each run's own events, so only the
    # start and the ends of the two runs fall at the same times
    assert h0 == h1
    for rows in (r0, r1):
        assert rows[0][0] == "0" and {"1", "1.5"} <= {r[0] for r in rows} and rows[-1][0] == "1.5"
    assert int(r1[-1][1]) > 1000
    sweeps = base + ["sweep color", "temperature 0.8", "stats 2.0", "run 10.0"]
    h0, r0 = stats_rows(stock, [l.format(app="potts 10") for l in sweeps])
    h1, r1 = stats_rows(gpu, [l.format(app="potts/gpu 10") for l in sweeps])
    assert [r[0] for r in r0] == [r[0] for r in r1] and [r[3] for r in r0] == [r[3] for r in r1]
    assert int(r1[-1][1]) > 0
