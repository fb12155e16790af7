"""NanoVDB buffers of level sets (nanovdb::tools::createNanoGrid for FloatGrids).

to_nanovdb(grid) returns the NanoGrid<float> buffer (NanoVDB 32.9,
breadth-first) of a HostGrid as a uint8 numpy array: byte for byte what
createNanoGrid(openvdb::FloatGrid, StatsMode, CheckMode) writes
(nanovdb/tools/CreateNanoGrid.h:162-168), so NanoVDB readers, renderers and
GPU samplers take it unchanged.  to_device(grid) places the same buffer in
device memory (a torch uint8 tensor) for CUDA consumers of NanoVDB.
"""
import ctypes as C

import numpy as np

from ._lib import check, lib

STATS = {"disable": 0, "bbox": 1, "minmax": 2, "all": 3}
CHECKSUM = {"disable": 0, "partial": 1, "full": 2}


def to_nanovdb(grid, name="", stats="all", checksum="partial"):
    """NanoGrid<float> buffer of `grid` (a HostGrid) named `name`."""
    L = lib()
    d = grid.desc()
    n = C.c_int64()
    s, c = STATS[stats], CHECKSUM[checksum]
    nm = name.encode()
    check(L.gbls_nanovdb_export(C.byref(d), nm, s, c, None, 0, C.byref(n)), host=True)
    buf = np.empty(n.value, np.uint8)
    check(L.gbls_nanovdb_export(C.byref(d), nm, s, c, buf.ctypes.data, n.value, C.byref(n)), host=True)
    return buf


def to_nanovdb_index(grid, name="", channel=True, include_stats=True, include_tiles=True,
                     checksum="partial"):
    """NanoGrid<ValueOnIndex> buffer of `grid` (createNanoGrid<FloatGrid,
    ValueOnIndex>(grid, channels, includeStats, includeTiles)); with
    `channel` the values follow as the blind-data array "channel_0"."""
    L = lib()
    d = grid.desc()
    n = C.c_int64()
    args = (name.encode(), int(bool(channel)), int(bool(include_stats)), int(bool(include_tiles)),
            CHECKSUM[checksum])
    check(L.gbls_nanovdb_export_index(C.byref(d), *args, None, 0, C.byref(n)), host=True)
    buf = np.empty(n.value, np.uint8)
    check(L.gbls_nanovdb_export_index(C.byref(d), *args, buf.ctypes.data, n.value, C.byref(n)), host=True)
    return buf


def from_nanovdb(buffer):
    """HostGrid of a NanoGrid<float> buffer (bytes or a uint8 array)."""
    from .fixtures import _from_native
    a = np.ascontiguousarray(np.frombuffer(bytes(buffer), np.uint8) if isinstance(buffer, (bytes, bytearray))
                             else buffer, dtype=np.uint8)
    h = C.c_void_p()
    check(lib().gbls_nanovdb_import(a.ctypes.data, a.size, C.byref(h)), host=True)
    return _from_native(h)


def to_device(grid, name="", stats="all", checksum="partial", device="cuda"):
    """The same buffer as a torch uint8 tensor on `device`."""
    import torch
    return torch.from_numpy(to_nanovdb(grid, name, stats, checksum)).to(device)
