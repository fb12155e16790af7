""".vdb files of level-set FloatGrids (host code, no GPU).

The writer's bytes are compared with the same grid written by the
reference's own serialisers (io::GridDescriptor, MetaMap, math::Transform,
the tree's writeTopology / writeBuffers and io::writeCompressedValues, built
from the reference sources into oracle/_ref), the reader is compared with
the reference's deserialisers on files from both sides (half-float storage
included), and the per-node record kinds of the active-mask compression are
all exercised by planting inactive values in leaves.  The reference tests are
skipped where the oracle library is not built; the round trips run
everywhere.
"""
import os
import struct

import numpy as np
import pytest

from openvdb_gb300 import HostGrid, digest, fixtures, vdbfile
from openvdb_gb300._lib import GblsError

UUID_AT, UUID_LEN = 21, 36  # magic 8 + versions 12 + offsets flag 1


def _refpy():
    refpy = pytest.importorskip("oracle.refpy")
    if not refpy.available():
        pytest.skip("reference oracle library not built on this host")
    return refpy


def _same(a, b):
    assert digest(a) == digest(b)
    assert (a.map_type, tuple(a.translation), a.voxel_size) == (b.map_type, tuple(b.translation), b.voxel_size)


def _clone(g, **kw):
    args = dict(voxel_size=g.voxel_size, background=g.background, translation=g.translation,
                map_type=g.map_type)
    for k in ("leaf_origins", "leaf_masks", "leaf_values", "lower_origins", "lower_tiles",
              "upper_origins", "upper_tiles", "root_tile_origins", "root_tile_values"):
        args[k] = getattr(g, k).copy()
    args.update(kw)
    return HostGrid(**args)


def _planted(g):
    """Inactive leaf values other than +-background, one leaf per record
    kind of io/Compression.h (one odd value; odd value + background; two odd
    values; three distinct values), plus a leaf with every voxel active."""
    h = _clone(g)
    bg = np.float32(h.background)
    inactive = [~np.unpackbits(h.leaf_masks[i].view(np.uint8), bitorder="little").astype(bool)
                for i in range(5)]
    v = h.leaf_values
    v[0][inactive[0]] = 0.25                      # NO_MASK_AND_ONE_INACTIVE_VAL
    idx = np.flatnonzero(inactive[1])
    v[1][idx] = bg
    v[1][idx[::2]] = 0.5                          # MASK_AND_ONE_INACTIVE_VAL
    idx = np.flatnonzero(inactive[2])
    v[2][idx] = 0.75
    v[2][idx[::3]] = -0.125                       # MASK_AND_TWO_INACTIVE_VALS
    idx = np.flatnonzero(inactive[3])
    v[3][idx[0::3]], v[3][idx[1::3]], v[3][idx[2::3]] = 1.0, 2.0, 3.0   # NO_MASK_AND_ALL_VALS
    h.leaf_masks[4][:] = np.uint64(0xFFFFFFFFFFFFFFFF)                # no inactive values
    return h


def _grids():
    sphere = fixtures.sphere(20.0, (1.5, -3.0, 7.0), 0.5, 3.0)
    union = fixtures.union_of_spheres(np.array([[0, 0, 0], [30, 5, -12], [-4100, 17, 9]], np.float32),
                                      np.array([12, 9, 6], np.float32), 1.0, 3.0)
    shifted = _clone(sphere, translation=(0.25, -1.0, 3.5), map_type=1)
    return {"sphere": sphere, "union": union, "translated": shifted, "planted": _planted(sphere)}


GRIDS = None


def grids():
    global GRIDS
    if GRIDS is None:
        GRIDS = _grids()
    return GRIDS


@pytest.mark.parametrize("name", ["sphere", "union", "translated", "planted"])
def test_round_trip(tmp_path, name):
    g = grids()[name]
    p = tmp_path / "g.vdb"
    vdbfile.write(p, g, name)
    _same(vdbfile.read(p, name), g)
    assert vdbfile.grid_info(p) == [(name, "Tree_float_5_4_3", "level set")]


def test_planted_leaves_cover_every_record_kind(tmp_path):
    g = grids()["planted"]
    p = tmp_path / "g.vdb"
    vdbfile.write(p, g, "planted")
    data = p.read_bytes()
    at = struct.unpack_from("<q", data, UUID_AT + UUID_LEN + 4 + 4 + (4 + 7) + (4 + 16) + 4 + 8)[0]
    kinds = []
    for leaf in range(5):  # buffers: value mask, record kind, extras, active values
        mask = np.frombuffer(data, np.uint64, 8, at)
        kind = data[at + 64]
        at += 65 + 4 * (kind in (2, 4, 5)) + 4 * (kind == 5) + 64 * (kind in (3, 4, 5))
        at += 4 * (512 if kind == 6 else int(np.unpackbits(mask.view(np.uint8)).sum()))
        kinds.append(kind)
    assert kinds == [2, 4, 5, 6, 0]


def test_several_grids_and_unique_names(tmp_path):
    gs = grids()
    p = tmp_path / "many.vdb"
    vdbfile.write(p, [gs["sphere"], gs["union"], gs["planted"], gs["translated"]], ["a", "b", "a", ""])
    names = [n for n, _, _ in vdbfile.grid_info(p)]
    assert names == ["a\x1e0", "b", "a\x1e1", "\x1e0"]  # io::Archive::write's suffixes
    _same(vdbfile.read(p, "b"), gs["union"])
    _same(vdbfile.read(p, "a"), gs["sphere"])             # grid name: the first match
    _same(vdbfile.read(p, "a\x1e1"), gs["planted"])       # unique name
    _same(vdbfile.read(p, index=3), gs["translated"])
    assert vdbfile.File(p).gridNames() == names


def test_empty_grid(tmp_path):
    g = HostGrid(voxel_size=0.1, background=0.3)
    p = tmp_path / "e.vdb"
    vdbfile.write(p, g, "empty")
    _same(vdbfile.read(p), g)


@pytest.mark.parametrize("name", ["sphere", "union", "translated", "planted"])
def test_bytes_equal_reference_writer(tmp_path, name):
    refpy = _refpy()
    g = grids()[name]
    mine, ref = tmp_path / "mine.vdb", tmp_path / "ref.vdb"
    vdbfile.write(mine, g, name)
    refpy.RefGrid.from_host(g).write_vdb(str(ref), name)
    a, b = mine.read_bytes(), ref.read_bytes()
    assert len(a) == len(b)
    assert a[:UUID_AT] == b[:UUID_AT] and a[UUID_AT + UUID_LEN:] == b[UUID_AT + UUID_LEN:]


def test_empty_grid_bytes_equal_reference_writer(tmp_path):
    refpy = _refpy()
    g = HostGrid(voxel_size=0.1, background=0.3)
    mine, ref = tmp_path / "mine.vdb", tmp_path / "ref.vdb"
    vdbfile.write(mine, g, "empty")
    refpy.RefGrid.from_host(g).write_vdb(str(ref), "empty")
    a, b = mine.read_bytes(), ref.read_bytes()
    assert a[:UUID_AT] + a[UUID_AT + UUID_LEN:] == b[:UUID_AT] + b[UUID_AT + UUID_LEN:]


@pytest.mark.parametrize("name", ["sphere", "union", "translated", "planted"])
def test_reference_reads_our_file(tmp_path, name):
    refpy = _refpy()
    g = grids()[name]
    p = tmp_path / "mine.vdb"
    vdbfile.write(p, g, name)
    _same(refpy.RefGrid.read_vdb(str(p), name).to_host(), g)


@pytest.mark.parametrize("half", [False, True])
@pytest.mark.parametrize("name", ["sphere", "union", "planted"])
def test_we_read_reference_file(tmp_path, name, half):
    refpy = _refpy()
    g = grids()[name]
    p = tmp_path / "ref.vdb"
    refpy.RefGrid.from_host(g).write_vdb(str(p), name, half=half)
    expect = refpy.RefGrid.read_vdb(str(p), name).to_host()
    if not half:
        _same(expect, g)
    got = vdbfile.read(p, name)
    _same(got, expect)
    assert vdbfile.grid_info(p)[0][1] == ("Tree_float_5_4_3_HalfFloat" if half else "Tree_float_5_4_3")


def _status(fn):
    with pytest.raises(GblsError) as e:
        fn()
    return e.value.code


def test_errors(tmp_path):
    g = grids()["sphere"]
    p = tmp_path / "g.vdb"
    vdbfile.write(p, g, "s")
    data = p.read_bytes()
    bad = tmp_path / "bad.vdb"
    bad.write_bytes(b"not a vdb file at all")
    assert _status(lambda: vdbfile.read(bad)) == 3                       # RuntimeError: not a VDB file
    bad.write_bytes(data[: len(data) // 2])
    assert _status(lambda: vdbfile.read(bad)) == 3                       # truncated
    assert _status(lambda: vdbfile.read(p, "nope")) == 1                 # no such grid
    assert _status(lambda: vdbfile.read(tmp_path / "missing.vdb")) == 3  # cannot open
    # the grid's compression flags (right after the three stream offsets): Blosc
    at = UUID_AT + UUID_LEN + 4 + 4 + (4 + 1) + (4 + 16) + 4 + 24
    assert struct.unpack_from("<I", data, at)[0] == 2
    bad.write_bytes(data[:at] + struct.pack("<I", 6) + data[at + 4:])
    assert _status(lambda: vdbfile.read(bad)) == 8
    # another grid type
    bad.write_bytes(data.replace(b"Tree_float_5_4_3", b"Tree_int32_5_4_3"))
    assert _status(lambda: vdbfile.read(bad)) == 8
    # descriptors must be in tree order
    rev = _clone(g, leaf_origins=g.leaf_origins[::-1].copy())
    assert _status(lambda: vdbfile.write(tmp_path / "o.vdb", rev, "r")) == 1
