"""nf_stream_candidates_noalloc: the candidate dump staged in a fixed device
array instead of a per-call allocation. It must give the same candidates as
nf_stream_candidates, bit for bit (tolerance 0: the same kernel arithmetic on
the same Philox counters), call after call, and refuse sizes above its
65 536-candidate staging array.

The file sorts last so that it also runs after every other test of a session;
it passes alone in a fresh process as well (the first call on the device does
the address look-up)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX = 65536


def _both(sim, k0, n):
    a = sim.stream(k0, n)
    b = sim.stream_noalloc(k0, n)
    return a, b


def test_noalloc_matches_allocating_dump_uniform_density(gpu):
    cfg = dict(gpu.configs.SMALL)
    with gpu.Simulation(cfg) as sim:
        # Two calls in a row through the no-allocation path, the first one
        # before anything else touched the handle's device state.
        b1 = sim.stream_noalloc(0, MAX)
        b2 = sim.stream_noalloc(987654321, 4000)
        a1 = sim.stream(0, MAX)
        a2 = sim.stream(987654321, 4000)
    assert np.array_equal(a1.view(np.uint32), b1.view(np.uint32))
    assert np.array_equal(a2.view(np.uint32), b2.view(np.uint32))
    assert np.isfinite(b1).all() and np.isfinite(b2).all()


def test_noalloc_matches_allocating_dump_density_mesh(gpu):
    cfg = dict(gpu.configs.MEDIUM)
    with gpu.Simulation(cfg, mesh=gpu.configs.gaussian_mesh()) as sim:
        # The mesh is uploaded by the allocating path; before that the
        # no-allocation path reports a state error instead of allocating.
        with pytest.raises(gpu.NanoFillerError) as ei:
            sim.stream_noalloc(0, 16)
        assert ei.value.status == 10 and "density mesh" in str(ei.value)
        a1, b1 = _both(sim, 5, MAX)
        a2, b2 = _both(sim, 2**40 + 17, 1)
        b3 = sim.stream_noalloc(5, MAX)  # again, after a different call
    assert np.array_equal(a1.view(np.uint32), b1.view(np.uint32))
    assert np.array_equal(a2.view(np.uint32), b2.view(np.uint32))
    assert np.array_equal(b1.view(np.uint32), b3.view(np.uint32))
    assert (b1[:, 9] < 1.0).any() and (b1[:, 9] > 0).all()  # rho varies over the mesh


def test_noalloc_limits(gpu):
    with gpu.Simulation(dict(gpu.configs.SMALL)) as sim:
        with pytest.raises(gpu.NanoFillerError) as ei:
            sim.stream_noalloc(0, MAX + 1)
        assert ei.value.status == 5 and "65536" in str(ei.value)
        assert sim.stream_noalloc(0, 0).shape == (0, 10)
        # NULL destinations are skipped, as in nf_stream_candidates.
        x = np.zeros(100, np.float32)
        L = gpu.load()
        st = L.nf_stream_candidates_noalloc(sim._h, 0, 100, x.ctypes.data_as(C.c_void_p), *([None] * 9))
        assert st == 0
        assert np.array_equal(x, sim.stream(0, 100)[:, 0])


def test_noalloc_makes_no_allocation(gpu):
    """The property the entry point exists for: after the handle is set up,
    calls through it leave the library's count of requested blocks unchanged,
    while the allocating dump requests a staging block on every call."""
    with gpu.Simulation(dict(gpu.configs.SMALL)) as sim:
        sim.stream_noalloc(0, 16)  # device code loaded, handle descriptors on the device
        n0 = gpu.allocations()
        for k0 in (0, 1 << 20, 1 << 33):
            sim.stream_noalloc(k0, MAX)
        assert gpu.allocations() == n0
        sim.stream(0, MAX)
        assert gpu.allocations() > n0

