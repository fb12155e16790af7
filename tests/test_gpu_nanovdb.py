"""NanoVDB on the device (gbls_nanovdb_export_device,
gbls_nanovdb_export_index_device, gbls_create_from_nanovdb).

The device writers must produce, byte for byte, what the host writers
produce for the downloaded grid -- and those are pinned to the reference's
nanovdb::tools::createNanoGrid by tests/test_nanovdb.py -- in every
statistics, checksum, channel and tile mode, for grids with several root
entries, negative origins, root tiles and translated maps, after an
advection has reshaped the tree, and for batch instances.  A device buffer
read back into a handle must give the grid it was written from.
"""
import ctypes as C

import numpy as np
import pytest

from openvdb_gb300 import DeviceLevelSet, fixtures
from openvdb_gb300._lib import GblsError, lib
from openvdb_gb300.grid import bitwise_equal, compare
from openvdb_gb300.levelset import DeviceBatch
from openvdb_gb300.nanovdb import (export_device, export_index_device, from_device, from_nanovdb, to_nanovdb,
                                   to_nanovdb_index)

STATS = ["disable", "bbox", "minmax", "all"]
CHECKSUMS = ["disable", "partial", "full"]


def _grids():
    centers, radii = fixtures.sixty_four_spheres(seed=11, n=8, domain=256.0, rmin=10.0, rmax=30.0)
    union = fixtures.union_of_spheres(centers, radii, 1.0, 3.0)
    tiles = union.copy()
    tiles.root_tile_origins = np.array([[-8192, 4096, 0], [8192, 0, 0]], np.int32)
    tiles.root_tile_values = np.array([3.0, -3.0], np.float32)
    moved = fixtures.sphere(12.0, (3.5, -7.25, 1.0))
    moved.translation = (0.25, -1.0, 3.5)
    moved.map_type = 1
    return {"sphere": fixtures.sphere(12.0, (3.5, -7.25, 1.0)),
            "torus": fixtures.torus(20.0, 6.0, (-40.0, 5.0, 9.0)),
            "union": union,
            "root_tiles": tiles,
            "translated": moved,
            "big": fixtures.sphere(300.0, (0.0, 0.0, 0.0), half_width=2.0)}


GRIDS = None


def grids():
    global GRIDS
    if GRIDS is None:
        GRIDS = _grids()
    return GRIDS


def _host(t):
    return t.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["sphere", "torus", "union", "root_tiles", "translated", "big"])
def test_float_grid_bytes_equal_host_writer(name):
    ls = DeviceLevelSet(grids()[name])
    g = ls.to_host()
    for stats in STATS:
        for checksum in CHECKSUMS:
            dev = _host(export_device(ls, name, stats, checksum))
            host = to_nanovdb(g, name, stats, checksum)
            assert dev.size == host.size
            diff = np.flatnonzero(dev != host)
            assert diff.size == 0, (stats, checksum, diff[:8])
    ls.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["sphere", "union", "root_tiles", "translated", "big"])
def test_index_grid_bytes_equal_host_writer(name):
    ls = DeviceLevelSet(grids()[name])
    g = ls.to_host()
    for channel in (False, True):
        for stats in (False, True):
            for tiles in (False, True):
                for checksum in CHECKSUMS:
                    dev = _host(export_index_device(ls, name, channel, stats, tiles, checksum))
                    host = to_nanovdb_index(g, name, channel, stats, tiles, checksum)
                    assert dev.size == host.size
                    diff = np.flatnonzero(dev != host)
                    assert diff.size == 0, (channel, stats, tiles, checksum, diff[:8])
    ls.close()


@pytest.mark.gpu
def test_after_advection_and_tracking():
    """New leaves from dilation, pruned leaves and node tables rebuilt by the
    tracker: the device writers still agree with the host writers."""
    from openvdb_gb300 import PARITY, LevelSetAdvection
    from openvdb_gb300.fields import Field
    c, r = fixtures.sixty_four_spheres(seed=3, n=6, domain=128.0, rmin=8.0, rmax=20.0)
    ls = DeviceLevelSet(fixtures.union_of_spheres(c, r, 1.0, 3.0))
    ls.set_precision(PARITY)
    adv = LevelSetAdvection(ls, Field.deformation(domain=128.0, period=20.0, scale=1.0))
    adv.advect(0.0, 2.0)
    g = ls.to_host()
    for stats in STATS:
        assert np.array_equal(_host(export_device(ls, "a", stats, "full")), to_nanovdb(g, "a", stats, "full"))
    assert np.array_equal(_host(export_index_device(ls, "a", True, True, True, "full")),
                          to_nanovdb_index(g, "a", True, True, True, "full"))
    ls.close()


@pytest.mark.gpu
def test_batch_instances():
    gs = grids()
    b = DeviceBatch([gs["sphere"], gs["torus"], gs["union"]])
    for i in range(3):
        g = b.to_host(i)
        assert np.array_equal(_host(export_device(b, "i", "all", "full", instance=i)), to_nanovdb(g, "i", "all", "full"))
        assert np.array_equal(_host(export_index_device(b, "i", True, True, False, "partial", instance=i)),
                              to_nanovdb_index(g, "i", True, True, False, "partial"))
    with pytest.raises(GblsError):
        export_device(b, "i", instance=3)
    with pytest.raises(GblsError):
        export_device(b, "i", instance=-1)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["sphere", "union", "root_tiles", "translated", "big"])
def test_device_buffer_round_trip(name):
    """Device export -> device import, and host buffer -> device import."""
    g = grids()[name]
    ls = DeviceLevelSet(g)
    buf = export_device(ls, name, "all", "full")
    back = from_device(buf)
    out = back.to_host()
    assert bitwise_equal(out, g), compare(out, g)
    assert back.voxel_size == g.voxel_size and back.background == np.float32(g.background)
    host_back = from_device(to_nanovdb(g, name)).to_host()
    assert bitwise_equal(host_back, g), compare(host_back, g)
    assert bitwise_equal(from_nanovdb(_host(buf)), g)
    ls.close()
    back.close()


@pytest.mark.gpu
def test_device_import_advects_like_the_source():
    """A level set imported from a device NanoVDB buffer advects bit for bit
    like the grid it was written from."""
    from openvdb_gb300 import PARITY, LevelSetAdvection, digest
    from openvdb_gb300.fields import Field
    c, r = fixtures.sixty_four_spheres(seed=5, n=5, domain=128.0, rmin=8.0, rmax=20.0)
    g = fixtures.union_of_spheres(c, r, 1.0, 3.0)
    a, b = DeviceLevelSet(g), from_device(export_device(DeviceLevelSet(g), "g"))
    out = []
    for ls in (a, b):
        ls.set_precision(PARITY)
        LevelSetAdvection(ls, Field.deformation(domain=128.0, period=20.0, scale=1.0)).advect(0.0, 1.0)
        out.append(digest(ls.to_host()))
    assert out[0] == out[1]


@pytest.mark.gpu
def test_rejects_bad_output_buffers():
    import torch
    L = lib()
    ls = DeviceLevelSet(grids()["sphere"])
    n = C.c_int64()
    assert L.gbls_nanovdb_export_device(ls.handle, -1, b"s", 3, 1, None, 0, C.byref(n)) == 0
    buf = torch.zeros(n.value + 64, dtype=torch.uint8, device="cuda")
    # too small, misaligned, host memory
    assert L.gbls_nanovdb_export_device(ls.handle, -1, b"s", 3, 1, C.c_void_p(buf.data_ptr()), n.value - 1,
                                        C.byref(n)) == 1
    assert L.gbls_nanovdb_export_device(ls.handle, -1, b"s", 3, 1, C.c_void_p(buf.data_ptr() + 16), n.value,
                                        C.byref(n)) == 1
    host = np.zeros(n.value, np.uint8)
    assert L.gbls_nanovdb_export_device(ls.handle, -1, b"s", 3, 1, C.c_void_p(host.ctypes.data), n.value,
                                        C.byref(n)) == 1
    assert int(buf.sum()) == 0
    with pytest.raises(GblsError):
        export_device(ls, "x" * 300)
    assert L.gbls_nanovdb_export_index_device(ls.handle, -1, b"s", 2, 1, 1, 1, None, 0, C.byref(n)) == 8
    ls.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["union_float", "tiles_float", "negative_float", "union_index", "tiles_index",
                                  "negative_index"])
def test_device_probe_matches_reference_accessor(case):
    """Device-written buffer -> device ReadAccessor: the reference's own
    accessor's values, value indices and active flags on the same bytes."""
    import hashlib
    import os
    import sys
    import torch
    from openvdb_gb300.nanovdb import probe
    here = os.path.join(os.path.dirname(__file__), "golden")
    sys.path.insert(0, here)
    import make_nanovdb_probe as mp
    gold = np.load(os.path.join(here, "nanovdb_probe.npz"))
    grid, kind, args = mp.CASES[case]
    ls = DeviceLevelSet(mp.make_grid(grid))
    if kind == "float":
        buf = export_device(ls, case, STATS[args[0]], CHECKSUMS[args[1]])
    else:
        buf = export_index_device(ls, case, False, args[0], args[1], "partial")
    assert hashlib.sha256(_host(buf).tobytes()).digest() == gold[case + "/sha256"].tobytes()
    ijk = torch.from_numpy(gold[case + "/ijk"]).cuda()
    vals, act = probe(buf, ijk)
    exp = gold[case + "/values"]
    got = _host(vals)
    got = got.view(np.uint32) if kind == "float" else got.view(np.uint64)
    assert np.array_equal(got, exp), np.flatnonzero(got != exp)[:8]
    assert np.array_equal(_host(act), gold[case + "/active"])
    ls.close()


@pytest.mark.gpu
def test_device_probe_bounds_checks_truncated_buffers():
    import torch
    from openvdb_gb300.nanovdb import probe
    ls = DeviceLevelSet(grids()["sphere"])
    buf = export_device(ls, "s")
    ijk = torch.tensor([[0, 0, 0], [12, 0, 0], [15, -7, 1]], dtype=torch.int32, device="cuda")
    v, a = probe(buf, ijk)
    assert int(a.sum()) >= 1
    for cut in (700, 900, buf.numel() // 2):
        with pytest.raises(GblsError):
            probe(buf[:cut], ijk)
    ls.close()
