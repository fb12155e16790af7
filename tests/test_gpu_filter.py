"""LevelSetFilter on the device against the reference (tools/LevelSetFilter.h).

tests/golden/parity_cases.json["__filter__"] holds the digest of the full
canonical grid after every filter call of the reference compiled from source
(laplacian, mean curvature, fillet, mean and gaussian box filters, median,
offsets; each followed by the tracker pass).  PARITY mode must reproduce every grid bit for bit.
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
    calls = {0: lambda w, v: f.laplacian(), 1: lambda w, v: f.mean(w), 2: lambda w, v: f.gaussian(w),
             3: lambda w, v: f.offset(v), 4: lambda w, v: f.meanCurvature(), 5: lambda w, v: f.fillet(),
             6: lambda w, v: f.median(w)}
    for k, (op, width, value) in enumerate(case["ops"]):
        calls[op](width, value)
        assert digest(dev.to_host()) == gold[k + 1]["digest"], (name, k, op, gold[k + 1]["summary"])


@pytest.mark.gpu
def test_filter_widths_beyond_the_halo_are_refused():
    from openvdb_gb300 import _abi, fixtures
    f = LevelSetFilter(DeviceLevelSet(fixtures.sphere(8.0)))
    for call in (lambda: f.median(4), lambda: f.mean(4)):
        with pytest.raises(GblsError) as e:
            call()
        assert e.value.code == _abi.ERR_UNSUPPORTED
