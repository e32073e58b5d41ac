"""Host-side checks of the input-script driver behind the reference's library
interface (spparks_open_no_mpi / spparks_command / spparks_extract): command
parsing, refusals and the reference-compatible `set site range` values.  No
command here reaches the GPU."""

import numpy as np
import pytest

import oracle
import spparks_gb300 as sg


@pytest.fixture
def spk():
    from spparks_gb300 import build

    build.build()
    s = sg.SPPARKS(cmdargs=["-screen", "none", "-log", "none"])
    yield s
    s.close()


def setup_lines(nx=16, ny=16, app="ising"):
    return ["seed 56789", f"app_style {app}", "dimension 2", "lattice sq/4n 1.0",
            f"region box block 0 {nx} 0 {ny} -0.5 0.5", "create_box box", "create_sites box"]


def test_set_site_range_matches_reference(spk, ref_fixtures):
    """`seed` + `set site range` give the unmodified reference's initial values
    (RanMars master stream, Park-Miller irandom per site ID)."""
    fx = ref_fixtures["strict"][0]
    c = fx["case"]
    for line in setup_lines(c["nx"], c["ny"]):
        spk.command(line.replace("56789", str(c["master_seed"])))
    spk.command(f"set site range 1 {c['nspins']}")
    assert spk.sites().tolist() == fx["snaps"]["init"]["spins"]
    assert spk.extract("nlocal", 0) == c["nx"] * c["ny"]
    assert spk.extract("dimension", 0) == 2


def test_commands_outside_the_gpu_path_are_refused(spk):
    for line in setup_lines():
        spk.command(line)
    with pytest.raises(sg.SpkGpuError, match="serial site order"):
        spk.command("sweep random")
    with pytest.raises(sg.SpkGpuError):
        spk.command("bogus_command 1")
    with pytest.raises(sg.SpkGpuError, match="Illegal sector command"):
        spk.command("sector 3")
    spk.command("dump 1 text 10.0 dump.ising")  # output-only: accepted with a warning


def test_run_needs_a_solver_and_valid_sites(spk):
    for line in setup_lines():
        spk.command(line)
    spk.command("temperature 1.0")
    with pytest.raises(sg.SpkGpuError, match="solver"):
        spk.command("run 1.0")
    spk.command("sweep color")
    # create_sites leaves every value 0: outside 1..2
    with pytest.raises(sg.SpkGpuError, match="invalid values"):
        spk.command("run 1.0")


def test_set_site_range_equals_oracle_restatement(spk):
    for line in setup_lines(32, 8, "potts 7").__iter__():
        spk.command(line)
    spk.command("set site range 1 7")
    u = oracle.ranmars_draws(56789, 1)
    assert spk.sites().tolist() == oracle.set_range(oracle.park_seed(u[0]), 256, 1, 7).tolist()


def test_dump_one_and_read_sites_match_reference_files(spk, ref_fixtures, tmp_path, monkeypatch):
    """Before any run (no device work): `dump_one` writes the reference's
    first text snapshot of the `set site range` lattice byte for byte, and a
    `dump sites` file read back with `read_sites` restores the same values."""
    monkeypatch.chdir(tmp_path)
    fx = ref_fixtures["io"][0]
    lines = [ln for ln in fx["case"]["lines"] if not ln.startswith(("run", "stats"))]
    for line in lines:
        spk.command(line)
    spk.command("dump_one 1")
    first = fx["files"]["dump.text"].split("ITEM: TIMESTEP")[1]
    assert (tmp_path / "dump.text").read_text() == "ITEM: TIMESTEP" + first
    spk.command("dump_one 2")
    assert (tmp_path / "sites.0.txt").read_text() == fx["files"]["sites.0.txt"]
    before = spk.sites().copy()
    spk.command("set site value 1")
    spk.command("read_sites sites.0.txt")
    assert spk.sites().tolist() == before.tolist()


def test_read_sites_refuses_explicit_lattices(spk, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    for line in setup_lines(8, 8, "ising"):
        spk.command(line)
    (tmp_path / "s.txt").write_text("x\n\n2 dimension\n64 sites\n4 max neighbors\n\nSites\n\n")
    with pytest.raises(sg.SpkGpuError, match="create_sites"):
        spk.command("read_sites s.txt")
