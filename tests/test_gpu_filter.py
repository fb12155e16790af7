"""LevelSetFilter on the device against the reference (tools/LevelSetFilter.h).

tests/golden/parity_cases.json["__filter__"] holds the digest of the full
canonical grid after every filter call of the reference compiled from source
(laplacian, mean curvature, fillet, mean and gaussian box filters, median,
offsets, with and without an alpha mask; each followed by the tracker pass).
PARITY mode must reproduce every grid bit for bit.
"""
import json
import os

import pytest

from cases import FILTER_CASES, make_fixture
from openvdb_gb300 import PARITY, DeviceLevelSet, LevelSetFilter, digest
from openvdb_gb300._lib import GblsError

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "parity_cases.json")))["__filter__"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(FILTER_CASES))
def test_filter_parity(name):
    case, gold = FILTER_CASES[name], GOLD[name]
    src = make_fixture(case["fixture"])
    assert digest(src) == gold[0]["digest"]
    dev = DeviceLevelSet(src)
    dev.set_precision(PARITY)
    f = LevelSetFilter(dev)
    tsp, ttp, nc = case["tracker"]
    f.setSpatialScheme(tsp)
    f.setTemporalScheme(ttp)
    f.setNormCount(nc)
    mask = DeviceLevelSet(make_fixture(case["mask"])) if "mask" in case else None
    if mask is not None:
        mask.set_precision(PARITY)
    calls = {0: lambda w, v, m: f.laplacian(m), 1: lambda w, v, m: f.mean(w, m), 2: lambda w, v, m: f.gaussian(w, m),
             3: lambda w, v, m: f.offset(v, m), 4: lambda w, v, m: f.meanCurvature(m), 5: lambda w, v, m: f.fillet(m),
             6: lambda w, v, m: f.median(w, m)}
    for k, op in enumerate(case["ops"]):
        m = None
        if len(op) > 3:
            f.setMaskRange(*op[3])
            f.invertMask(op[4])
            m = mask
        calls[op[0]](op[1], op[2], m)
        assert digest(dev.to_host()) == gold[k + 1]["digest"], (name, k, op, gold[k + 1]["summary"])


@pytest.mark.gpu
def test_filter_widths_beyond_the_halo_are_refused():
    from openvdb_gb300 import _abi, fixtures
    f = LevelSetFilter(DeviceLevelSet(fixtures.sphere(8.0)))
    for call in (lambda: f.median(4), lambda: f.mean(4)):
        with pytest.raises(GblsError) as e:
            call()
        assert e.value.code == _abi.ERR_UNSUPPORTED


@pytest.mark.gpu
def test_filter_mask_checks():
    """setMaskRange refuses min >= max (ValueError, as the reference); the mask
    must be another level set with the same transform."""
    from openvdb_gb300 import _abi, fixtures
    dev = DeviceLevelSet(fixtures.sphere(8.0))
    f = LevelSetFilter(dev)
    with pytest.raises(ValueError):
        f.setMaskRange(1.0, 1.0)
    with pytest.raises(GblsError) as e:
        f.laplacian(dev)
    assert e.value.code == _abi.ERR_UNSUPPORTED
    other = DeviceLevelSet(fixtures.sphere(8.0, voxel_size=0.5))
    with pytest.raises(GblsError) as e:
        f.laplacian(other)
    assert e.value.code == _abi.ERR_UNSUPPORTED
