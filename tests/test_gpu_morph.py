"""LevelSetMorphing on the device against the reference (tools/LevelSetMorph.h).

tests/golden/parity_cases.json["__morph__"] holds, per case, the digest of
the full canonical grid after every LevelSetMorphing::advect(t0, t1) call of
the reference compiled from source (tests/golden/make_golden.py) and the
number of CFL substeps.  PARITY mode must reproduce every grid bit for bit;
FAST mode (FP32 WENO weights) must keep the topology and the substep counts
and stay within 1e-3 of the band width: the sphere-to-torus case pinches a
hole through the sphere, where the FP32 and FP64 weights drift apart more
than under advection (measured: 4.1e-4 of the band width there).
"""
import json
import os

import numpy as np
import pytest

from cases import MORPH_CASES, make_fixture
from openvdb_gb300 import FAST, PARITY, DeviceLevelSet, LevelSetMorphing, digest
from openvdb_gb300.grid import compare, topology_equal

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "parity_cases.json")))["__morph__"]


def _run(name, mode):
    case = MORPH_CASES[name]
    src, tgt = make_fixture(case["source"]), make_fixture(case["target"])
    gold = GOLD[name]
    assert digest(src) == gold[0]["digest"] and digest(tgt) == gold[0]["target"]
    dev, target = DeviceLevelSet(src), DeviceLevelSet(tgt)
    dev.set_precision(mode)
    mask = DeviceLevelSet(make_fixture(case["mask"])) if "mask" in case else None
    sp, tp, tsp, ttp, nc = case["schemes"]
    m = LevelSetMorphing(dev, target)
    m.setSpatialScheme(sp)
    m.setTemporalScheme(tp)
    m.setTrackerSpatialScheme(tsp)
    m.setTrackerTemporalScheme(ttp)
    m.setNormCount(nc)
    out = []
    for op in case["ops"]:
        if len(op) > 3:
            m.setAlphaMask(mask)
            m.setMaskRange(*op[3])
            m.invertMask(op[4])
        n = m.advect(op[1], op[2])
        out.append((n, dev.to_host()))
    return gold, out


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MORPH_CASES))
def test_morph_parity(name):
    gold, out = _run(name, PARITY)
    for k, (n, g) in enumerate(out):
        rec = gold[k + 1]
        assert n == rec["count"], (name, k, n, rec["count"])
        assert digest(g) == rec["digest"], (name, k, rec["summary"], compare(g, g))


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MORPH_CASES))
def test_morph_fast_close(name):
    _, ref = _run(name, PARITY)
    _, fast = _run(name, FAST)
    for (n0, a), (n1, b) in zip(ref, fast):
        assert n0 == n1 and topology_equal(a, b), name
        d = np.abs(a.active_values().astype(np.float64) - b.active_values().astype(np.float64)).max()
        print("%s: FAST vs PARITY max |diff| %.3g of the band width" % (name, d / a.background))
        assert d <= 1e-3 * a.background, (name, d)
