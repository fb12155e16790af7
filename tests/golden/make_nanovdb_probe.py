"""Generate tests/golden/nanovdb_probe.npz from the reference implementation.

For each case a seeded level set (openvdb_gb300.fixtures) is converted by
the reference's own nanovdb::tools::createNanoGrid (compiled into
oracle/_ref by oracle/ref/build_ref.py) and probed by the reference's own
nanovdb::ReadAccessor (getValue / isActive; for ValueOnIndex grids the
LeafData<ValueOnIndex>::getValue decode, nanovdb/NanoVDB.h:4144-4170) at
seeded index coordinates: random points around the narrow band, every
voxel of a few leaves, points in root tiles and far outside.  Stored per
case: the SHA-256 of the reference's buffer (the device writer must produce
the same bytes), the coordinates, the values (float bits, or value indices)
and the active flags.  Index grids carry no value channel, whose padding the
reference leaves uninitialised.

Usage: python tests/golden/make_nanovdb_probe.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from openvdb_gb300 import fixtures  # noqa: E402

OUT = os.path.join(HERE, "nanovdb_probe.npz")

# name: (grid, kind, arguments); kind "float": (stats, checksum),
# "index": (stats, tiles)
CASES = {
    "union_float": ("union", "float", (3, 1)),
    "tiles_float": ("root_tiles", "float", (2, 1)),
    "negative_float": ("negative", "float", (0, 0)),
    "union_index": ("union", "index", (True, True)),
    "tiles_index": ("root_tiles", "index", (True, True)),
    "negative_index": ("negative", "index", (False, False)),
}


def make_grid(name):
    if name in ("union", "root_tiles"):
        c, r = fixtures.sixty_four_spheres(seed=11, n=8, domain=256.0, rmin=10.0, rmax=30.0)
        g = fixtures.union_of_spheres(c, r, 1.0, 3.0)
        if name == "root_tiles":
            g.root_tile_origins = np.array([[-8192, 4096, 0], [8192, 0, 0]], np.int32)
            g.root_tile_values = np.array([3.0, -3.0], np.float32)
        return g
    if name == "negative":
        return fixtures.sphere(30.0, (-40.5, -100.25, 7.0))
    raise KeyError(name)


def coords(g, seed):
    """Seeded probe coordinates for grid g (n x 3 int32)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    o = g.leaf_origins
    lo, hi = o.min(axis=0) - 12, o.max(axis=0) + 20
    parts = [rng.integers(lo, hi, size=(3000, 3))]
    for f in rng.choice(len(o), size=4, replace=False):  # every voxel of four leaves
        i = np.arange(512)
        parts.append(o[f] + np.stack([i >> 6, (i >> 3) & 7, i & 7], axis=1))
    parts.append(rng.integers(-12000, 12000, size=(500, 3)))
    for t in g.root_tile_origins:
        parts.append(t + rng.integers(0, 4096, size=(200, 3)))
    return np.ascontiguousarray(np.concatenate(parts).astype(np.int32))


def main():
    from oracle import refpy
    if not refpy.available():
        raise SystemExit("the reference oracle library is not built (python -m oracle.ref.build_ref)")
    out = {}
    for k, (case, (grid, kind, args)) in enumerate(CASES.items()):
        g = make_grid(grid)
        ref = refpy.RefGrid.from_host(g)
        if kind == "float":
            buf = ref.nanovdb(case, args[0], args[1])
        else:
            buf = ref.nanovdb_index(case, 0, args[0], args[1], 1)
        ijk = coords(g, 100 + k)
        vals, act = refpy.nano_probe(buf, ijk)
        out[case + "/sha256"] = np.frombuffer(hashlib.sha256(buf.tobytes()).digest(), np.uint8)
        out[case + "/ijk"] = ijk
        out[case + "/values"] = vals.view(np.uint32) if kind == "float" else vals
        out[case + "/active"] = act
        print(case, buf.size, "bytes,", len(ijk), "probes,", int(act.sum()), "active")
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
