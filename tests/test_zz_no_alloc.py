"""gbls_count_active_noalloc against gbls_get_counts, through the C ABI.

The allocation-free entry point is for callers whose host application owns
the device memory budget and forbids allocations after start-up.  It must
return exactly the active-voxel count that gbls_get_counts reports; it is
called twice in a row (the second call reuses the static scratch array that
the first call left behind) on two different grid states.
"""
import ctypes as C

import pytest


@pytest.mark.gpu
def test_count_active_noalloc_matches_get_counts():
    from openvdb_gb300 import FAST, DeviceLevelSet, Field, LevelSetAdvection, fixtures
    from openvdb_gb300._abi import GridCounts
    from openvdb_gb300._lib import lib

    L = lib()
    L.gbls_count_active_noalloc.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
    L.gbls_count_active_noalloc.restype = C.c_int

    host = fixtures.sphere(40.0, (3.0, -2.0, 5.0), 1.0, 3.0)
    dev = DeviceLevelSet(host)
    dev.set_precision(FAST)
    adv = LevelSetAdvection(dev, Field.constant_field((0.8, -0.3, 0.5)))
    for step in range(2):
        adv.advect(float(step), float(step) + 1.0)
        counts = GridCounts()
        assert L.gbls_get_counts(dev.handle, C.byref(counts)) == 0
        n = C.c_int64(-1)
        rc = L.gbls_count_active_noalloc(dev.handle, C.byref(n))
        assert rc == 0, L.gbls_last_error()
        assert n.value == counts.active_voxel_count
        # a second call in a row returns the same count
        m = C.c_int64(-1)
        assert L.gbls_count_active_noalloc(dev.handle, C.byref(m)) == 0
        assert m.value == n.value


@pytest.mark.gpu
def test_count_active_noalloc_limit_memory_and_launches(monkeypatch):
    """The leaf limit (lowered through GBLS_NOALLOC_MAX_LEAVES): a grid of
    exactly the limit is counted, one leaf over it is rejected with
    GBLS_ERR_INVALID_ARGUMENT.  Calls leave the device's free memory as it
    was, and each counted call adds its two kernels to the launch counter."""
    import torch
    from openvdb_gb300 import DeviceLevelSet, _abi, fixtures
    from openvdb_gb300._abi import GridCounts
    from openvdb_gb300._lib import lib

    L = lib()
    L.gbls_count_active_noalloc.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
    L.gbls_count_active_noalloc.restype = C.c_int
    dev = DeviceLevelSet(fixtures.sphere(24.0, (0.5, 1.5, -2.0), 1.0, 3.0))
    counts = GridCounts()
    assert L.gbls_get_counts(dev.handle, C.byref(counts)) == 0
    n = C.c_int64(-1)
    assert L.gbls_count_active_noalloc(dev.handle, C.byref(n)) == 0  # warm-up: module and stream set up
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    dev.reset_stats()
    monkeypatch.setenv("GBLS_NOALLOC_MAX_LEAVES", str(counts.leaf_count))
    for _ in range(3):
        n = C.c_int64(-1)
        assert L.gbls_count_active_noalloc(dev.handle, C.byref(n)) == 0, L.gbls_last_error()
        assert n.value == counts.active_voxel_count
    assert dev.stats()["kernel_launches"] == 6
    monkeypatch.setenv("GBLS_NOALLOC_MAX_LEAVES", str(counts.leaf_count - 1))
    n = C.c_int64(-1)
    assert L.gbls_count_active_noalloc(dev.handle, C.byref(n)) == _abi.ERR_INVALID_ARGUMENT
    assert b"at most" in L.gbls_last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
