"""CPU-side checks of the C-ABI library: it loads without a GPU, exports every
symbol that include/*.h declares, and rejects bad descriptions before any
device call."""

import ctypes
import re
from pathlib import Path

import pytest

import spparks_gb300 as sg

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b((?:spkgpu|spparks)_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from spparks_gb300 import build

    build.build()
    return sg.load_library()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "spkgpu_create" in names and "spkgpu_sweep" in names and len(names) >= 20


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert missing == []
    assert set(sg.EXPORTS) <= set(declared_symbols())


def test_version_and_invalid_descriptions(lib):
    assert lib.spkgpu_version() == 1
    bad = [
        dict(nx=7),                      # odd extent cannot be coloured
        dict(app=sg.ISING, nspins=3),    # Ising is two-state
        dict(nsector=3),
        dict(lattice=sg.SQ_4N, nsector=8),  # 2d with 8 sectors
        dict(rng=sg.RNG_STRICT, nsector=4),  # color/strict with sectors
        dict(nspins=200, spin_bytes=1),
        dict(variant=3),
    ]
    for b in bad:
        d = sg.Desc()
        d.lattice, d.nx, d.ny, d.nz = sg.SQ_4N, 8, 8, 1
        d.app, d.nspins, d.spin_bytes, d.nsector, d.nloop = sg.POTTS, 5, 0, 1, 1
        d.procs[0] = d.procs[1] = d.procs[2] = 1
        d.rng, d.mask, d.seed, d.device, d.variant = 0, 0, 1, 0, 0
        for k, v in b.items():
            setattr(d, k, v)
        h = ctypes.c_void_p()
        assert lib.spkgpu_create(ctypes.byref(d), ctypes.byref(h)) == -1, b
        assert not h.value


def test_null_handle_calls_fail_cleanly(lib):
    assert lib.spkgpu_sweep(None, 1) == -1
    assert lib.spkgpu_destroy(None) == -1
    assert lib.spkgpu_last_error(None) == b"null handle"


def test_noalloc_rejects_bad_arguments_before_any_device_call(lib):
    f = lib.spkgpu_sweep_sq4_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                  ctypes.c_int32, ctypes.c_double, ctypes.c_uint32, ctypes.c_int64, ctypes.c_int32,
                  ctypes.c_void_p, ctypes.c_void_p]
    # (pointer, nx, ny, spin_bytes, app, nspins, T): never dereferenced on these paths
    bad = [
        (0x10000, 64, 64, 1, sg.ISING, 2, -1.0),     # negative temperature
        (0x10004, 64, 64, 1, sg.ISING, 2, 2.0),      # not 8-byte aligned
        (0x10000, 48, 64, 1, sg.ISING, 2, 2.0),      # extent not a multiple of 32
        (0x10000, 64, 64, 1, sg.ISING, 3, 2.0),      # Ising is two-state
        (0x10000, 64, 64, 3, sg.POTTS, 5, 2.0),      # no 3-byte site values
        (None, 64, 64, 1, sg.ISING, 2, 2.0),
    ]
    for p, nx, ny, sb, app, q, T in bad:
        assert f(p, nx, ny, sb, app, q, T, 1, 0, 1, None, None) == -1, (p, nx, ny, sb, app, q, T)
