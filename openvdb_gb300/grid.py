"""Host-side level-set grid in the gbls_grid_desc exchange format.

A HostGrid holds the canonical description of an OpenVDB FloatGrid narrow
band (tree order everywhere; see include/gbls.h) in numpy arrays, and hands a
ctypes GridDesc view of them to the C ABI.
"""
import ctypes as C

import numpy as np

from . import _abi

UPPER_SLOTS = 32768
LOWER_SLOTS = 4096


def _ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class HostArena:
    """Reusable host storage for downloads, optionally page-locked.

    HostGrid.allocate(counts, arena) hands out views into buffers that grow
    on demand and are reused by the next allocation from the same arena, so
    repeated downloads touch no fresh pages.  A grid allocated from an arena
    is overwritten by the next allocation from it: uploading it first and
    downloading the result into the same arena updates the grid in place.
    """

    def __init__(self, pinned=False, headroom=1.25):
        self.pinned = bool(pinned)
        self.headroom = float(headroom)  # capacity factor of every (re)allocation
        self._bufs = {}

    def _alloc(self, nbytes):
        if self.pinned:
            import torch
            t = torch.empty(max(nbytes, 1), dtype=torch.uint8, pin_memory=True)
            return t, t.numpy()
        a = np.empty(max(nbytes, 1), np.uint8)
        return a, a

    def array(self, name, shape, dtype):
        nbytes = int(np.prod(shape, dtype=np.int64)) * np.dtype(dtype).itemsize
        held = self._bufs.get(name)
        if held is None or held[1].nbytes < nbytes:
            cap = int(nbytes * self.headroom) + 64
            held = self._alloc(cap)
            self._bufs[name] = held
        return held[1][:nbytes].view(dtype).reshape(shape)


class HostGrid:
    """Numpy arrays describing one FloatGrid level set."""

    def __init__(self, voxel_size=1.0, background=3.0, translation=(0.0, 0.0, 0.0),
                 map_type=_abi.MAP_UNIFORM_SCALE, leaf_origins=None, leaf_masks=None,
                 leaf_values=None, lower_origins=None, lower_tiles=None, upper_origins=None,
                 upper_tiles=None, root_tile_origins=None, root_tile_values=None):
        self.voxel_size = float(voxel_size)
        self.background = float(np.float32(background))
        self.translation = tuple(float(t) for t in translation)
        self.map_type = int(map_type)

        def arr(a, shape_tail, dtype):
            if a is None:
                return np.zeros((0,) + shape_tail, dtype=dtype)
            return np.ascontiguousarray(a, dtype=dtype).reshape((-1,) + shape_tail)

        self.leaf_origins = arr(leaf_origins, (3,), np.int32)
        self.leaf_masks = arr(leaf_masks, (8,), np.uint64)
        self.leaf_values = arr(leaf_values, (512,), np.float32)
        self.lower_origins = arr(lower_origins, (3,), np.int32)
        self.lower_tiles = arr(lower_tiles, (LOWER_SLOTS,), np.float32)
        self.upper_origins = arr(upper_origins, (3,), np.int32)
        self.upper_tiles = arr(upper_tiles, (UPPER_SLOTS,), np.float32)
        self.root_tile_origins = arr(root_tile_origins, (3,), np.int32)
        self.root_tile_values = arr(root_tile_values, (), np.float32).reshape(-1)

    # ---- construction from counts (to receive a download) ---------------
    @classmethod
    def allocate(cls, counts, arena=None):
        """Arrays for a download of `counts` (every element is written by the
        download); from `arena` when given, else freshly zeroed."""
        if arena is not None:
            g = cls()
            for k, tail, dt, n in (("leaf_origins", (3,), np.int32, counts.leaf_count),
                                   ("leaf_masks", (8,), np.uint64, counts.leaf_count),
                                   ("leaf_values", (512,), np.float32, counts.leaf_count),
                                   ("lower_origins", (3,), np.int32, counts.lower_count),
                                   ("lower_tiles", (LOWER_SLOTS,), np.float32, counts.lower_count),
                                   ("upper_origins", (3,), np.int32, counts.upper_count),
                                   ("upper_tiles", (UPPER_SLOTS,), np.float32, counts.upper_count),
                                   ("root_tile_origins", (3,), np.int32, counts.root_tile_count),
                                   ("root_tile_values", (), np.float32, counts.root_tile_count)):
                setattr(g, k, arena.array(k, (n,) + tail, dt))
            return g
        return cls(
            leaf_origins=np.zeros((counts.leaf_count, 3), np.int32),
            leaf_masks=np.zeros((counts.leaf_count, 8), np.uint64),
            leaf_values=np.zeros((counts.leaf_count, 512), np.float32),
            lower_origins=np.zeros((counts.lower_count, 3), np.int32),
            lower_tiles=np.zeros((counts.lower_count, LOWER_SLOTS), np.float32),
            upper_origins=np.zeros((counts.upper_count, 3), np.int32),
            upper_tiles=np.zeros((counts.upper_count, UPPER_SLOTS), np.float32),
            root_tile_origins=np.zeros((counts.root_tile_count, 3), np.int32),
            root_tile_values=np.zeros((counts.root_tile_count,), np.float32),
        )

    def desc(self):
        """A GridDesc pointing into this grid's arrays (valid while self lives)."""
        d = _abi.GridDesc()
        d.voxel_size = self.voxel_size
        d.translation[:] = self.translation
        d.map_type = self.map_type
        d.background = self.background
        d.leaf_count = len(self.leaf_origins)
        d.leaf_origins = _ptr(self.leaf_origins, C.c_int32)
        d.leaf_masks = _ptr(self.leaf_masks, C.c_uint64)
        d.leaf_values = _ptr(self.leaf_values, C.c_float)
        d.lower_count = len(self.lower_origins)
        d.lower_origins = _ptr(self.lower_origins, C.c_int32)
        d.lower_tiles = _ptr(self.lower_tiles, C.c_float)
        d.upper_count = len(self.upper_origins)
        d.upper_origins = _ptr(self.upper_origins, C.c_int32)
        d.upper_tiles = _ptr(self.upper_tiles, C.c_float)
        d.root_tile_count = len(self.root_tile_origins)
        d.root_tile_origins = _ptr(self.root_tile_origins, C.c_int32)
        d.root_tile_values = _ptr(self.root_tile_values, C.c_float)
        return d

    def copy_scalars_from(self, d):
        self.voxel_size = d.voxel_size
        self.translation = tuple(d.translation)
        self.map_type = d.map_type
        self.background = d.background

    # ---- queries ----------------------------------------------------------
    @property
    def leaf_count(self):
        return len(self.leaf_origins)

    def active_voxel_count(self):
        bits = np.unpackbits(self.leaf_masks.view(np.uint8), bitorder="little")
        return int(bits.sum())

    def active_mask_bool(self):
        """(L, 512) bool array of active voxels (voxel n = (x<<6)|(y<<3)|z)."""
        bits = np.unpackbits(self.leaf_masks.view(np.uint8).reshape(-1, 64), axis=1,
                             bitorder="little")
        return bits.astype(bool)

    def active_values(self):
        return self.leaf_values[self.active_mask_bool()]

    def active_coords(self):
        m = self.active_mask_bool()
        li, n = np.nonzero(m)
        o = self.leaf_origins[li]
        return np.stack([o[:, 0] + (n >> 6), o[:, 1] + ((n >> 3) & 7), o[:, 2] + (n & 7)], axis=1)

    def copy(self):
        g = HostGrid(self.voxel_size, self.background, self.translation, self.map_type)
        for k in ("leaf_origins", "leaf_masks", "leaf_values", "lower_origins", "lower_tiles",
                  "upper_origins", "upper_tiles", "root_tile_origins", "root_tile_values"):
            setattr(g, k, getattr(self, k).copy())
        return g


def topology_equal(a, b):
    """True when the node structure, leaf set, masks and tiles are identical."""
    return (np.array_equal(a.leaf_origins, b.leaf_origins)
            and np.array_equal(a.leaf_masks, b.leaf_masks)
            and np.array_equal(a.lower_origins, b.lower_origins)
            and np.array_equal(a.upper_origins, b.upper_origins)
            and np.array_equal(a.lower_tiles, b.lower_tiles)
            and np.array_equal(a.upper_tiles, b.upper_tiles)
            and np.array_equal(a.root_tile_origins, b.root_tile_origins)
            and np.array_equal(a.root_tile_values, b.root_tile_values))


def compare(a, b):
    """Summary of the differences between two grids (for test messages)."""
    out = {
        "leaves": (a.leaf_count, b.leaf_count),
        "active": (a.active_voxel_count(), b.active_voxel_count()),
        "topology_equal": topology_equal(a, b),
    }
    if np.array_equal(a.leaf_origins, b.leaf_origins):
        out["mask_words_differing"] = int((a.leaf_masks != b.leaf_masks).sum())
        diff = np.abs(a.leaf_values.astype(np.float64) - b.leaf_values.astype(np.float64))
        out["max_abs_value_diff"] = float(diff.max()) if diff.size else 0.0
        out["values_bitwise_equal"] = bool(np.array_equal(a.leaf_values.view(np.uint32),
                                                          b.leaf_values.view(np.uint32)))
    else:
        sa = {tuple(o) for o in a.leaf_origins.tolist()}
        sb = {tuple(o) for o in b.leaf_origins.tolist()}
        out["leaves_only_a"] = len(sa - sb)
        out["leaves_only_b"] = len(sb - sa)
    return out


def bitwise_equal(a, b):
    return (topology_equal(a, b)
            and np.array_equal(a.leaf_values.view(np.uint32), b.leaf_values.view(np.uint32))
            and a.background == b.background and a.voxel_size == b.voxel_size)


def digest(g):
    """SHA-256 over the canonical arrays of a grid (bit-exact fingerprint)."""
    import hashlib
    h = hashlib.sha256()
    h.update(np.float32(g.background).tobytes())
    h.update(np.float64(g.voxel_size).tobytes())
    for k in ("leaf_origins", "leaf_masks", "leaf_values", "lower_origins", "lower_tiles",
              "upper_origins", "upper_tiles", "root_tile_origins", "root_tile_values"):
        a = np.ascontiguousarray(getattr(g, k))
        h.update(k.encode())
        h.update(np.int64(a.size).tobytes())
        h.update(a.tobytes())
    return h.hexdigest()


def summary(g):
    """Small order-independent statistics of a grid (for messages and fixtures)."""
    act = g.active_values().astype(np.float64)
    return {
        "leaves": int(g.leaf_count),
        "active": int(act.size),
        "lower": int(len(g.lower_origins)),
        "upper": int(len(g.upper_origins)),
        "root_tiles": int(len(g.root_tile_origins)),
        "sum": float(act.sum()),
        "sum_abs": float(np.abs(act).sum()),
        "negative": int((act < 0).sum()),
    }
