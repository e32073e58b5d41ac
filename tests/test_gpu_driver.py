"""The reference's input scripts through the GB300 driver (the reference's
library interface, libspkgpu.so): stats columns, lattices and energies equal
the reference's own output for the same script."""

import tempfile
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def sg():
    import spparks_gb300

    spparks_gb300.load_library()
    return spparks_gb300


def stats_rows(text):
    rows, grab = [], False
    for line in text.splitlines():
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


@pytest.mark.parametrize("k", range(3))
def test_script_stats_match_reference_log(sg, ref_fixtures, k):
    fx = ref_fixtures["logs"][k]
    with tempfile.TemporaryDirectory() as d:
        log = Path(d) / "log.spkgpu"
        spk = sg.SPPARKS(cmdargs=["-screen", "none", "-log", str(log)])
        for line in fx["case"]["lines"]:
            spk.command(line)
        spk.close()
        got = stats_rows(log.read_text())
    ref = fx["rows"]
    # the reference prints the first row of each run; so does the driver
    assert [r[1:] for r in got] == [r[1:] for r in ref]
    for g, r in zip(got, ref):
        assert float(f"{g[0]:.6g}") == pytest.approx(r[0], rel=1e-5)


@pytest.mark.parametrize("k", range(3))
def test_strict_script_through_driver(sg, ref_fixtures, k):
    fx = ref_fixtures["strict"][k]
    spk = sg.SPPARKS(cmdargs=["-screen", "none", "-log", "none"])
    r = 0
    for line in fx["script"]:
        if line.startswith("#!"):
            if line.startswith("#! snap run"):
                assert spk.sites().tolist() == fx["snaps"][f"run{r}"]["spins"]
            elif line.startswith("#! energy"):
                assert spk.energy() == fx["energies"][r]
                r += 1
            continue
        spk.command(line)
    spk.close()


@pytest.mark.parametrize("kind,k", [("sweeps", 0), ("sweeps", 3), ("sweeps", 8), ("sweeps", 11), ("kmc", 0)])
def test_philox_script_through_driver(sg, ref_fixtures, kind, k):
    """Philox-shim reference scripts: `seed S` keys the draws; the initial
    values are written through extract("site") like a library caller would."""
    fx = ref_fixtures[kind][k]
    spk = sg.SPPARKS(cmdargs=["-screen", "none", "-log", "none"])
    philox_seed = fx["case"]["seed"]
    for line in fx["script"]:
        if line.startswith("#!"):
            if line.startswith("#! snap init"):
                spk.set_sites(fx["snaps"]["init"]["spins"])
            elif line.startswith("#! snap"):
                tag = line.split()[2]
                assert spk.sites().tolist() == fx["snaps"][tag]["spins"], tag
            continue
        if line.startswith("seed "):
            line = f"seed {philox_seed}"
        spk.command(line)
    spk.close()


def stats_table(text):
    header, rows = None, []
    for line in text.splitlines():
        p = line.split()
        if p[:4] == ["Time", "Naccept", "Nreject", "Nsweeps"]:
            header = p
            continue
        if header is not None and len(p) == len(header) and p[0][0].isdigit():
            rows.append(p)
    return header, rows


@pytest.mark.parametrize("k", range(3))
def test_diag_columns_match_reference_log(sg, ref_fixtures, k):
    """`diag_style energy | array | cluster` columns printed by the driver from
    the device diagnostics equal the unmodified reference's (color/strict)."""
    fx = ref_fixtures["diag_logs"][k]
    with tempfile.TemporaryDirectory() as d:
        log = Path(d) / "log.spkgpu"
        spk = sg.SPPARKS(cmdargs=["-screen", "none", "-log", str(log)])
        for line in fx["case"]["lines"]:
            spk.command(line)
        spk.close()
        header, rows = stats_table(log.read_text())
    assert header == fx["header"]
    drop_cpu = lambda r: r[:4] + r[5:]  # noqa: E731
    assert [drop_cpu(r) for r in rows] == [drop_cpu(r) for r in fx["rows"]]


@pytest.mark.parametrize("k", range(3))
def test_dumps_and_read_sites_match_reference(sg, ref_fixtures, k, tmp_path, monkeypatch):
    """`dump text|sites` (with `dump_modify delay`) and `read_sites` through
    the driver: the stats rows and every file the unmodified reference writes
    (color/strict runs) are reproduced exactly."""
    fx = ref_fixtures["io"][k]
    monkeypatch.chdir(tmp_path)
    for name, text in fx["case"]["inputs"].items():
        (tmp_path / name).write_text(text)
    log = tmp_path / "log.spkgpu"
    spk = sg.SPPARKS(cmdargs=["-screen", "none", "-log", str(log)])
    for line in fx["case"]["lines"]:
        spk.command(line)
    spk.close()
    header, rows = stats_table(log.read_text())
    assert header == fx["header"]
    drop_cpu = lambda r: r[:4] + r[5:]  # noqa: E731
    assert [drop_cpu(r) for r in rows] == [drop_cpu(r) for r in fx["rows"]]
    for name, text in fx["files"].items():
        assert (tmp_path / name).read_text() == text, name


@pytest.mark.parametrize("k", range(2))
def test_kmc_stats_between_passes_match_reference_log(sg, ref_fixtures, k, tmp_path, monkeypatch):
    """tree KMC with `stats` and `diag_style energy`: the rows the reference
    (Philox shim) prints between passes, from runs paused at each output
    time (spkgpu_kmc_run_until) and continued."""
    fx = ref_fixtures["kmc_logs"][k]
    monkeypatch.chdir(tmp_path)
    spk = sg.SPPARKS(cmdargs=["-screen", "none", "-log", "none"])
    for line in fx["script"]:
        if line.startswith("#!"):
            if line.startswith("#! snap init"):
                spk.set_sites(fx["snaps"]["init"]["spins"])
            elif line.startswith("#! snap"):
                tag = line.split()[2]
                assert spk.sites().tolist() == fx["snaps"][tag]["spins"], tag
            continue
        if line.startswith("seed "):
            line = f"seed {fx['case']['seed']}"
        spk.command(line)
    spk.close()
    header, rows = stats_table((tmp_path / "kmc.log").read_text())
    assert header == fx["header"]
    drop_cpu = lambda r: r[:4] + r[5:]  # noqa: E731
    assert [drop_cpu(r) for r in rows] == [drop_cpu(r) for r in fx["rows"]]
