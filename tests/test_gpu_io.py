"""Upload / download through the C ABI (gbls_create, gbls_batch_create,
gbls_download, gbls_batch_download): the device packs the host exchange
format and assembles it back, so a round trip must return the input bit for
bit (in tree order, whatever the input order), and malformed inputs must be
refused with the documented status codes.
"""
import numpy as np
import pytest

from openvdb_gb300 import DeviceLevelSet, _abi, fixtures
from openvdb_gb300._lib import GblsError
from openvdb_gb300.grid import bitwise_equal, compare
from openvdb_gb300.levelset import DeviceBatch


def _grids():
    centers, radii = fixtures.sixty_four_spheres(seed=11, n=8, domain=256.0, rmin=10.0, rmax=30.0)
    return [fixtures.sphere(12.0, (3.5, -7.25, 1.0)),
            fixtures.torus(20.0, 6.0, (-40.0, 5.0, 9.0)),
            fixtures.union_of_spheres(centers, radii, 1.0, 3.0),
            fixtures.sphere(300.0, (0.0, 0.0, 0.0), half_width=2.0)]


def _shuffled(g, seed):
    """The same grid with leaves and lower / upper nodes in a seeded random order."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = g.copy()
    p = rng.permutation(s.leaf_count)
    s.leaf_origins, s.leaf_masks, s.leaf_values = s.leaf_origins[p], s.leaf_masks[p], s.leaf_values[p]
    q = rng.permutation(len(s.lower_origins))
    s.lower_origins, s.lower_tiles = s.lower_origins[q], s.lower_tiles[q]
    r = rng.permutation(len(s.upper_origins))
    s.upper_origins, s.upper_tiles = s.upper_origins[r], s.upper_tiles[r]
    return s


@pytest.mark.gpu
@pytest.mark.parametrize("k", range(4))
def test_round_trip_bit_exact(k):
    g = _grids()[k]
    out = DeviceLevelSet(g).to_host()
    assert bitwise_equal(out, g), compare(out, g)
    out2 = DeviceLevelSet(_shuffled(g, 100 + k)).to_host()
    assert bitwise_equal(out2, g), compare(out2, g)


@pytest.mark.gpu
def test_batch_round_trip_bit_exact():
    grids = _grids()[:3]  # instances of a batch share the background
    b = DeviceBatch([grids[0], _shuffled(grids[1], 5), grids[2]])
    for i, g in enumerate(grids):
        out = b.to_host(i)
        assert bitwise_equal(out, g), (i, compare(out, g))


def _expect(g, code, text):
    with pytest.raises(GblsError) as e:
        DeviceLevelSet(g)
    assert e.value.code == code and text in str(e.value), str(e.value)


@pytest.mark.gpu
def test_rejects_malformed_inputs():
    base = fixtures.sphere(12.0, (3.5, -7.25, 1.0))
    gamma = base.background
    m = base.active_mask_bool()

    g = base.copy()  # inactive leaf value that is not +-background
    li, vi = np.argwhere(~m)[len(np.argwhere(~m)) // 2]
    g.leaf_values[li, vi] = 0.5 * gamma
    _expect(g, _abi.ERR_UNSUPPORTED, "inactive leaf value")

    g = base.copy()  # lower-node tile that is not +-background, away from any leaf
    lt = g.lower_tiles.reshape(len(g.lower_origins), -1)
    free = np.flatnonzero(lt[0] != 0.0)
    lt[0, free[len(free) // 2]] = 1.0
    _expect(g, _abi.ERR_UNSUPPORTED, "lower-node tile")

    g = base.copy()  # upper-node tile
    ut = g.upper_tiles.reshape(len(g.upper_origins), -1)
    free = np.flatnonzero(ut[0] != 0.0)
    ut[0, free[len(free) // 2]] = -1.0
    _expect(g, _abi.ERR_UNSUPPORTED, "upper-node tile")

    g = base.copy()  # duplicate leaf
    g.leaf_origins = np.concatenate([g.leaf_origins, g.leaf_origins[:1]])
    g.leaf_masks = np.concatenate([g.leaf_masks, g.leaf_masks[:1]])
    g.leaf_values = np.concatenate([g.leaf_values, g.leaf_values[:1]])
    _expect(g, _abi.ERR_INVALID_ARGUMENT, "duplicate leaf")

    g = base.copy()  # leaf without a lower node
    g.leaf_origins = g.leaf_origins.copy()
    g.leaf_origins[0] = (4096, 4096, 4096)
    _expect(g, _abi.ERR_INVALID_ARGUMENT, "leaf without lower node")

    g = base.copy()  # misaligned origin
    g.leaf_origins = g.leaf_origins.copy()
    g.leaf_origins[0, 1] += 3
    _expect(g, _abi.ERR_INVALID_ARGUMENT, "not aligned")

    # the handle is still usable after refusals
    assert bitwise_equal(DeviceLevelSet(base).to_host(), base)


@pytest.mark.gpu
def test_reupload_into_existing_handle():
    """gbls_upload replaces the level set and keeps the handle usable; a
    refused upload leaves an empty level set."""
    grids = _grids()
    dev = DeviceLevelSet(grids[0])
    for g in (grids[2], grids[1], grids[3], grids[0]):
        dev.upload(g)
        out = dev.to_host()
        assert bitwise_equal(out, g), compare(out, g)
    bad = grids[1].copy()
    bad.leaf_values = bad.leaf_values.copy()
    li, vi = np.argwhere(~bad.active_mask_bool())[0]
    bad.leaf_values[li, vi] = 0.0
    with pytest.raises(GblsError) as e:
        dev.upload(bad)
    assert e.value.code == _abi.ERR_UNSUPPORTED
    assert dev.counts().leaf_count == 0 and dev.active_voxel_count() == 0
    dev.upload(grids[2])
    assert bitwise_equal(dev.to_host(), grids[2])


@pytest.mark.gpu
def test_vdb_file_into_parity_advection(tmp_path):
    """A level set read from a .vdb file advects bit for bit like the same
    grid built in memory: the sphere12_rk2 parity case through the file
    path, checked against the reference digest, and written back out."""
    import json
    import os

    from cases import CASES, make_field, make_fixture
    from openvdb_gb300 import PARITY, LevelSetAdvection, digest, vdbfile

    name = "sphere12_rk2"
    case = CASES[name]
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "parity_cases.json")))[name]
    src = tmp_path / "in.vdb"
    vdbfile.write(src, make_fixture(case["fixture"]), "ls")
    dev = DeviceLevelSet(vdbfile.read(src, "ls"), device=0)
    dev.set_precision(PARITY)
    sp, tp, tsp, ttp, nc = case["schemes"]
    adv = LevelSetAdvection(dev, make_field(case["field"]))
    adv.setSpatialScheme(sp)
    adv.setTemporalScheme(tp)
    adv.setTrackerSpatialScheme(tsp)
    adv.setTrackerTemporalScheme(ttp)
    adv.setNormCount(nc)
    op = case["ops"][0]
    assert adv.advect(op[1], op[2]) == gold[1]["count"]
    out = dev.to_host()
    assert digest(out) == gold[1]["digest"]
    dst = tmp_path / "out.vdb"
    vdbfile.write(dst, out, "ls")
    assert digest(vdbfile.read(dst, "ls")) == gold[1]["digest"]
    dev.close()
