""".vdb files of level-set FloatGrids (OpenVDB file format 225), on the host.

Mirrors the reference's file interface for the grids the device path holds
(Tree_float_5_4_3 narrow-band level sets):

* write(filename, grids, names)   -- io::File::write (io/File.h:130) /
                                     pyopenvdb.write
* read(filename, gridname=None)   -- io::File::readGrid (io/File.h:150) /
                                     pyopenvdb.read; the first grid when no
                                     name is given
* grid_info(filename)             -- io::File::getGrids metadata: one
                                     (unique name, grid type, class) per grid
* File(filename)                  -- the same as methods, io::File style

Grids are HostGrid objects (the exchange layout of the C ABI); a grid read
from a file goes to the device with DeviceLevelSet(grid).  Data is written
with active-mask compression only, which every OpenVDB build reads;
Blosc- or zlib-compressed files are rejected (GblsError, status
GBLS_ERR_UNSUPPORTED), as are other grid types and active tiles.
"""
import ctypes as C
import os

from . import _abi
from ._lib import check, lib
from .fixtures import _from_native


def _path(filename):
    return os.fsencode(os.fspath(filename))


def write(filename, grids, names=None):
    """Write one grid or a list of grids; `names` defaults to empty names
    (made unique as io::Archive::write does)."""
    if not isinstance(grids, (list, tuple)):
        grids = [grids]
        names = [names] if isinstance(names, str) else names
    n = len(grids)
    if names is None:
        names = [""] * n
    if len(names) != n:
        raise ValueError("one name per grid")
    descs = (_abi.GridDesc * max(n, 1))()
    for i, g in enumerate(grids):
        descs[i] = g.desc()
    cnames = (C.c_char_p * max(n, 1))(*[(s or "").encode() for s in names])
    check(lib().gbls_vdb_write(_path(filename), n, descs, cnames), host=True)


def grid_info(filename):
    """[(unique name, grid type, grid class)] of the file's grids."""
    L = lib()
    count = C.c_int32()
    check(L.gbls_vdb_grid_count(_path(filename), C.byref(count)), host=True)
    out = []
    for i in range(count.value):
        name, typ, cls = (C.create_string_buffer(4096) for _ in range(3))
        check(L.gbls_vdb_grid_info(_path(filename), i, name, 4096, typ, 4096, cls, 4096), host=True)
        out.append((name.value.decode(), typ.value.decode(), cls.value.decode()))
    return out


def read(filename, gridname=None, index=0):
    """The grid named `gridname` (unique name first, then grid name), else
    the `index`-th grid, as a HostGrid."""
    h = C.c_void_p()
    name = gridname.encode() if gridname is not None else None
    check(lib().gbls_vdb_read(_path(filename), name, int(index), C.byref(h)), host=True)
    return _from_native(h)


class File:
    """io::File for level-set FloatGrids: getGrids metadata, readGrid, write."""

    def __init__(self, filename):
        self.filename = os.fspath(filename)

    def gridNames(self):
        return [n for n, _, _ in grid_info(self.filename)]

    def readGrid(self, name):
        return read(self.filename, name)

    def write(self, grids, names=None):
        write(self.filename, grids, names)
