"""spkgpu_sweep_sq4_noalloc, called through the C ABI.

Callers that cannot allocate device memory (they own all of it through their
own pool, or cannot afford the synchronisation cudaMalloc/cudaFree may cause)
hand their device lattice to this entry point, which keeps its sweep buffer
in a fixed static device array.  Its result must equal the regular entry
point's (spkgpu_create + spkgpu_sweep) exactly - site values are integers, so
the tolerance is zero - over two calls in a row that continue the sweep index.
This file is collected last so that a run stopping at the first failure has
already run every other test."""

import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

ERR_ARG, TOO_LARGE = -1, -8
NOALLOC_MAX_BYTES = 4 << 20  # SPKGPU_NOALLOC_MAX_BYTES


@pytest.fixture(scope="module")
def lib():
    import spparks_gb300

    return spparks_gb300.load_library()


@pytest.mark.parametrize("app,q,T,nx,ny,sb,calls,offset", [
    ("ising", 2, 2.269, 64, 64, 1, (3, 4), 0),
    # 8-byte but not 16-byte aligned: the 64-thread tile instead of the warp tile
    ("ising", 2, 2.269, 96, 64, 1, (2, 3), 8),
    ("potts", 30, 0.8, 96, 32, 4, (2, 3), 0),
    ("potts/neighonly", 7, 0.5, 32, 64, 2, (1, 2), 0),
])
def test_noalloc_matches_regular_entry_point(lib, app, q, T, nx, ny, sb, calls, offset):
    import torch

    import spparks_gb300 as sg

    seed = 2468
    n = nx * ny
    spin = oracle.init_spins(seed, n, 1, q)
    ref = sg.Lattice("sq/4n", nx, ny, 1, app, q, spin_bytes=sb, seed=seed)
    ref.set_temperature(T)
    ref.upload(spin)
    dtype = {1: torch.int8, 2: torch.int16, 4: torch.int32}[sb]
    store = torch.zeros(n + 16, dtype=dtype).cuda()
    dev = store[offset:offset + n]
    dev.copy_(torch.from_numpy(spin).to(dtype).cuda())
    assert dev.data_ptr() % 16 == (offset * dev.element_size()) % 16
    torch.cuda.synchronize()
    sweep0 = 0
    before = 0
    for ns in calls:
        na = ctypes.c_int64(-1)
        rc = lib.spkgpu_sweep_sq4_noalloc(ctypes.c_void_p(dev.data_ptr()), nx, ny, sb, sg.APP_STYLES[app], q, T,
                                          seed, sweep0, ns, None, ctypes.byref(na))
        assert rc == 0
        ref.sweep(ns)
        st = ref.stats()
        assert np.array_equal(dev.to(torch.int32).cpu().numpy(), ref.download())
        assert na.value == st["naccept"] - before
        before = st["naccept"]
        sweep0 += ns
    ref.close()


def test_noalloc_rejects_lattices_beyond_the_static_array(lib):
    import spparks_gb300 as sg

    na = ctypes.c_int64(0)
    # 4096 x 2048 int8 = 8 MiB > 4 MiB: rejected before any device work
    rc = lib.spkgpu_sweep_sq4_noalloc(ctypes.c_void_p(16), 4096, 2048, 1, sg.ISING, 2, 2.0, 1, 0, 1, None,
                                      ctypes.byref(na))
    assert rc == TOO_LARGE


def _regular(app, q, T, nx, ny, sb, seed, spin, nsweeps):
    import spparks_gb300 as sg

    ref = sg.Lattice("sq/4n", nx, ny, 1, app, q, spin_bytes=sb, seed=seed)
    ref.set_temperature(T)
    ref.upload(spin)
    ref.sweep(nsweeps)
    out, na = ref.download(), ref.stats()["naccept"]
    ref.close()
    return out, na


def test_noalloc_at_the_size_limit_and_without_waiting(lib):
    """A 2048 x 2048 int8 lattice fills the static array exactly and is
    accepted.  Three sweeps run on a side stream with naccept = NULL (the call
    returns without waiting); a zero-sweep call then changes nothing and
    reports zero."""
    import torch

    import spparks_gb300 as sg

    nx = ny = 2048
    assert nx * ny == NOALLOC_MAX_BYTES
    seed, T = 1357, 2.269
    spin = oracle.init_spins(seed, nx * ny, 1, 2)
    dev = torch.from_numpy(spin).to(torch.int8).cuda()
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    rc = lib.spkgpu_sweep_sq4_noalloc(ctypes.c_void_p(dev.data_ptr()), nx, ny, 1, sg.ISING, 2, T, seed, 0, 3,
                                      ctypes.c_void_p(side.cuda_stream), None)
    assert rc == 0
    side.synchronize()
    want, _ = _regular("ising", 2, T, nx, ny, 1, seed, spin, 3)
    got = dev.to(torch.int32).cpu().numpy()
    assert np.array_equal(got, want)
    na = ctypes.c_int64(-1)
    rc = lib.spkgpu_sweep_sq4_noalloc(ctypes.c_void_p(dev.data_ptr()), nx, ny, 1, sg.ISING, 2, T, seed, 3, 0,
                                      ctypes.c_void_p(side.cuda_stream), ctypes.byref(na))
    assert rc == 0 and na.value == 0
    assert np.array_equal(dev.to(torch.int32).cpu().numpy(), want)


def test_noalloc_refuses_a_counter_read_inside_a_capture(lib):
    """Reading the change count back waits for the stream, which a stream
    capture cannot hold: the call is refused before it enqueues anything,
    and the same call without the counter is then captured and replayed."""
    import torch

    import spparks_gb300 as sg

    nx, ny, seed, T = 64, 64, 97, 2.0
    spin = oracle.init_spins(seed, nx * ny, 1, 2)
    dev = torch.from_numpy(spin).to(torch.int8).cuda()
    na = ctypes.c_int64(-1)
    # the set-up call (address lookup) before any capture
    assert lib.spkgpu_sweep_sq4_noalloc(ctypes.c_void_p(dev.data_ptr()), nx, ny, 1, sg.ISING, 2, T, seed, 0, 0,
                                        None, ctypes.byref(na)) == 0
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side):
        refused = lib.spkgpu_sweep_sq4_noalloc(ctypes.c_void_p(dev.data_ptr()), nx, ny, 1, sg.ISING, 2, T, seed,
                                               0, 2, ctypes.c_void_p(side.cuda_stream), ctypes.byref(na))
        captured = lib.spkgpu_sweep_sq4_noalloc(ctypes.c_void_p(dev.data_ptr()), nx, ny, 1, sg.ISING, 2, T, seed,
                                                0, 2, ctypes.c_void_p(side.cuda_stream), None)
    assert refused == ERR_ARG and captured == 0
    # the capture recorded the work without running it
    assert np.array_equal(dev.to(torch.int32).cpu().numpy(), spin)
    g.replay()
    torch.cuda.synchronize()
    want, _ = _regular("ising", 2, T, nx, ny, 1, seed, spin, 2)
    assert np.array_equal(dev.to(torch.int32).cpu().numpy(), want)
