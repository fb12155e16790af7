"""NanoVDB export (host code, no GPU).

Every statistics mode (Disable, BBox, MinMax, All) and both checksum modes
are compared byte for byte with the reference's own
nanovdb::tools::createNanoGrid of the same FloatGrid (compiled from the
reference sources into oracle/_ref; serial statistics).  Grids: a sphere,
a union across several root entries with negative origins, explicit root
tiles, a translated map, planted inactive values, an empty grid, and voxel
sizes on both sides of the matrix inverse's Gauss-Jordan branch.  The
header checks below run everywhere.
"""
import struct
import zlib

import numpy as np
import pytest

from openvdb_gb300 import HostGrid, digest, fixtures
from openvdb_gb300.nanovdb import to_nanovdb

import test_vdbfile as tv


def _refpy():
    refpy = pytest.importorskip("oracle.refpy")
    if not refpy.available():
        pytest.skip("reference oracle library not built on this host")
    return refpy


def _grids():
    g = dict(tv.grids())
    g["empty"] = HostGrid(voxel_size=0.1, background=0.3)
    g["root_tiles"] = tv._clone(g["union"], root_tile_origins=np.array([[-8192, 4096, 0], [8192, 0, 0]], np.int32),
                                root_tile_values=np.array([3.0, -3.0], np.float32))  # tree (Coord) order
    g["dx_0.001_translated"] = tv._clone(g["sphere"], voxel_size=0.001, translation=(0.25, -1.0, 3.5), map_type=1)
    g["dx_0.003"] = tv._clone(g["sphere"], voxel_size=0.003)
    return g


GRIDS = None


def grids():
    global GRIDS
    if GRIDS is None:
        GRIDS = _grids()
    return GRIDS


NAMES = ["sphere", "union", "translated", "planted", "empty", "root_tiles", "dx_0.001_translated", "dx_0.003"]


@pytest.mark.parametrize("checksum", ["disable", "partial", "full"])
@pytest.mark.parametrize("stats", ["disable", "bbox", "minmax", "all"])
@pytest.mark.parametrize("name", NAMES)
def test_bytes_equal_reference(name, stats, checksum):
    refpy = _refpy()
    g = grids()[name]
    mine = to_nanovdb(g, name, stats, checksum)
    ref = refpy.RefGrid.from_host(g).nanovdb(name, ["disable", "bbox", "minmax", "all"].index(stats),
                                             ["disable", "partial", "full"].index(checksum))
    assert mine.size == ref.size
    assert np.array_equal(mine, ref)


def test_header_fields_and_checksum():
    g = grids()["union"]
    b = to_nanovdb(g, "union").tobytes()
    magic, checksum, version, flags, index, count, size = struct.unpack_from("<QQIIIIQ", b, 0)
    assert magic == 0x314244566F6E614E and version == (32 << 21) | (9 << 10) | 2
    assert flags == 0b111110 and (index, count, size) == (0, 1, len(b))
    assert b[40:45] == b"union" and b[45] == 0
    assert checksum >> 32 == 0xFFFFFFFF and checksum & 0xFFFFFFFF == zlib.crc32(b[16:672 + 64])
    node_offsets = struct.unpack_from("<4q", b, 672)
    node_counts = struct.unpack_from("<3I", b, 672 + 32)
    voxels = struct.unpack_from("<Q", b, 672 + 56)[0]
    assert node_counts == (len(g.leaf_origins), len(g.lower_origins), len(g.upper_origins))
    assert voxels == g.active_voxel_count()
    leaf_at = 672 + node_offsets[0]
    assert leaf_at + 2144 * len(g.leaf_origins) == len(b)
    first = np.frombuffer(b, np.float32, 512, leaf_at + 96)
    assert np.array_equal(first, g.leaf_values[0])


def test_rejects_long_names():
    from openvdb_gb300._lib import GblsError
    with pytest.raises(GblsError):
        to_nanovdb(grids()["sphere"], "x" * 300)


@pytest.mark.parametrize("name", NAMES)
def test_index_grid_full_checksum(name):
    """CheckMode::Full on an index grid without a value channel (with one, the
    reference's checksum covers its uninitialised padding)."""
    from openvdb_gb300.nanovdb import to_nanovdb_index
    refpy = _refpy()
    g = grids()[name]
    mine = to_nanovdb_index(g, name, False, True, True, checksum="full")
    ref = refpy.RefGrid.from_host(g).nanovdb_index(name, 0, True, True, checksum=2)
    assert np.array_equal(mine, ref)


@pytest.mark.parametrize("tiles", [False, True])
@pytest.mark.parametrize("stats", [False, True])
@pytest.mark.parametrize("channel", [False, True])
@pytest.mark.parametrize("name", NAMES)
def test_index_grid_bytes_equal_reference(name, channel, stats, tiles):
    """createNanoGrid<FloatGrid, ValueOnIndex>; the alignment padding after
    the value channel is uninitialised in the reference and is masked."""
    from openvdb_gb300.nanovdb import to_nanovdb_index
    refpy = _refpy()
    g = grids()[name]
    mine = to_nanovdb_index(g, name, channel, stats, tiles)
    ref = refpy.RefGrid.from_host(g).nanovdb_index(name, int(channel), stats, tiles)
    assert mine.size == ref.size
    count = int(np.frombuffer(mine.tobytes(), np.uint64, 1, 656)[0])
    pad = ((count * 4 + 31) // 32 * 32 - count * 4) if channel else 0
    assert np.array_equal(mine[: mine.size - pad], ref[: ref.size - pad])


def test_index_grid_values_and_offsets():
    """Every active value is found at its leaf's offset plus its rank."""
    from openvdb_gb300.nanovdb import to_nanovdb_index
    g = grids()["union"]
    b = to_nanovdb_index(g, "u").tobytes()
    count = struct.unpack_from("<Q", b, 656)[0]
    meta_at = struct.unpack_from("<q", b, 640)[0]
    data_at = meta_at + struct.unpack_from("<q", b, meta_at)[0]
    values = np.frombuffer(b, np.float32, count, data_at)
    leaf_at = 672 + struct.unpack_from("<q", b, 672)[0]
    for f in range(len(g.leaf_origins)):
        off, prefix = struct.unpack_from("<QQ", b, leaf_at + 96 * f + 80)
        bits = np.unpackbits(g.leaf_masks[f].view(np.uint8), bitorder="little").astype(bool)
        assert np.array_equal(values[off: off + bits.sum()], g.leaf_values[f][bits])
        sums = np.cumsum([bin(int(w)).count("1") for w in g.leaf_masks[f]])[:7]
        assert all(((prefix >> (9 * i)) & 511) == sums[i] for i in range(7))
    assert values[0] == np.float32(g.background)


@pytest.mark.parametrize("stats", ["disable", "all"])
@pytest.mark.parametrize("name", NAMES)
def test_import_round_trip(name, stats):
    """NanoGrid<float> -> exchange layout returns the grid bit for bit, also
    from the reference converter's buffer."""
    from openvdb_gb300.nanovdb import from_nanovdb
    g = grids()[name]
    back = from_nanovdb(to_nanovdb(g, name, stats))
    assert digest(back) == digest(g)
    assert np.allclose(back.translation, g.translation) and back.voxel_size == g.voxel_size
    refpy = pytest.importorskip("oracle.refpy")
    if refpy.available():
        ref = refpy.RefGrid.from_host(g).nanovdb(name, ["disable", "bbox", "minmax", "all"].index(stats), 1)
        assert digest(from_nanovdb(ref)) == digest(g)


def test_import_rejects_garbage():
    from openvdb_gb300._lib import GblsError
    from openvdb_gb300.nanovdb import from_nanovdb
    with pytest.raises(GblsError):
        from_nanovdb(b"\0" * 1000)
    buf = to_nanovdb(grids()["sphere"], "s")
    with pytest.raises(GblsError):
        from_nanovdb(buf[: buf.size // 2])


def _probe_golden():
    import os
    import sys
    here = os.path.join(os.path.dirname(__file__), "golden")
    sys.path.insert(0, here)
    import make_nanovdb_probe as mp
    return mp, np.load(os.path.join(here, "nanovdb_probe.npz"))


def _writer_bytes(mp, case):
    from openvdb_gb300.nanovdb import to_nanovdb_index
    grid, kind, args = mp.CASES[case]
    g = mp.make_grid(grid)
    if kind == "float":
        return to_nanovdb(g, case, ["disable", "bbox", "minmax", "all"][args[0]],
                          ["disable", "partial", "full"][args[1]])
    return to_nanovdb_index(g, case, False, args[0], args[1], "partial")


@pytest.mark.parametrize("case", ["union_float", "tiles_float", "negative_float", "union_index", "tiles_index",
                                  "negative_index"])
def test_probe_golden_buffers_are_the_host_writers(case):
    """The buffers the probe vectors were taken on are the host writer's
    bytes (so the device writer, equal to it, feeds the device probe the
    reference's buffer)."""
    import hashlib
    mp, gold = _probe_golden()
    b = _writer_bytes(mp, case)
    assert hashlib.sha256(b.tobytes()).digest() == gold[case + "/sha256"].tobytes()


@pytest.mark.parametrize("case", ["union_float", "tiles_index", "negative_index"])
def test_probe_golden_matches_reference(case):
    """The committed probe vectors are what the reference's ReadAccessor
    returns now."""
    refpy = _refpy()
    mp, gold = _probe_golden()
    vals, act = refpy.nano_probe(_writer_bytes(mp, case), gold[case + "/ijk"])
    exp = gold[case + "/values"]
    assert np.array_equal(vals.view(exp.dtype) if vals.dtype == np.float32 else vals, exp)
    assert np.array_equal(act, gold[case + "/active"])
