"""Bit-exact parity of the device path (PARITY mode) with the reference.

The reference digests in tests/golden/parity_cases.json were produced by
tests/golden/make_golden.py from the reference's own LevelSetAdvection /
LevelSetTracker compiled from source.  Every operation of every case must
reproduce the reference grid exactly: leaf set, masks, values, node tiles.
On a mismatch the device grid is written to $GBLS_DUMP_DIR for diagnosis.
"""
import json
import os

import numpy as np
import pytest

from cases import CASES, box_mask, make_field, make_fixture
from openvdb_gb300 import PARITY, DeviceLevelSet, LevelSetAdvection, LevelSetTracker, digest, summary

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "parity_cases.json")))


def _dump(name, step, g):
    d = os.environ.get("GBLS_DUMP_DIR")
    if not d:
        return
    os.makedirs(d, exist_ok=True)
    np.savez_compressed(os.path.join(d, "%s_%02d.npz" % (name, step)),
                        **{k: getattr(g, k) for k in ("leaf_origins", "leaf_masks", "leaf_values",
                                                       "lower_origins", "lower_tiles", "upper_origins",
                                                       "upper_tiles", "root_tile_origins",
                                                       "root_tile_values")})


def run_case(name, mode=PARITY, check=True):
    case, gold = CASES[name], GOLD[name]
    host = make_fixture(case["fixture"])
    assert digest(host) == gold[0]["digest"], "input fixture differs from the reference input"
    dev = DeviceLevelSet(host)
    dev.set_precision(mode)
    sp, tp, tsp, ttp, nc = case["schemes"]
    adv = LevelSetAdvection(dev, make_field(case["field"]))
    adv.setSpatialScheme(sp)
    adv.setTemporalScheme(tp)
    adv.setTrackerSpatialScheme(tsp)
    adv.setTrackerTemporalScheme(ttp)
    adv.setNormCount(nc)
    adv.cfl = case.get("cfl", 0.0)
    tr = adv.tracker
    results = []
    for step, (op, rec) in enumerate(zip(case["ops"], gold[1:]), start=1):
        if op[0] == "state":
            s = op[1]
            if "norm_count" in s:
                tr.setNormCount(s["norm_count"])
            if "tr_temporal" in s:
                tr.setTemporalScheme(s["tr_temporal"])
            if "trim" in s:
                tr.setTrimming(s["trim"])
            continue
        count = None
        if op[0] == "advect":
            count = adv.advect(op[1], op[2])
        elif op[0] == "track":
            tr.track()
        elif op[0] == "normalize":
            tr.normalize()
        elif op[0] == "normalize_masked":
            tr.normalize(box_mask(dev.to_host(), op[1], op[2]))
        elif op[0] == "prune":
            tr.prune()
        elif op[0] == "dilate":
            tr.dilate(op[1])
        g = dev.to_host()
        results.append((op, count, g))
        if check:
            if count is not None:
                assert count == rec["count"], (name, step, op, count, rec["count"])
            if digest(g) != rec["digest"]:
                _dump(name, step, g)
                pytest.fail("%s op %d %s: device %s != reference %s" % (name, step, op, summary(g),
                                                                        rec["summary"]))
    return results


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_parity_bit_exact(name):
    run_case(name)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["sphere20_deformation", "tracker_ops", "union8_deformation"])
def test_parity_with_device_wide_candidate_sort(name, monkeypatch):
    """The dilation's fallback for more candidates than one CTA sorts (the
    device-wide sort, then new leaves and merge on host counts), forced for
    every dilation of handles created while GBLS_SMALL_SORT_LIMIT is 0: the
    same grids, bit for bit."""
    monkeypatch.setenv("GBLS_SMALL_SORT_LIMIT", "0")
    run_case(name)


@pytest.mark.gpu
@pytest.mark.parametrize("key", ["__batch__", "__batch_cfl05__"])
def test_batch_bit_exact_per_instance(key):
    """Batched advection: every instance equals its own reference advect call
    (independent CFL substep sequences in shared launches), at the reference
    CFL number and under the imposed CFL 0.5."""
    from cases import BATCH, BATCH_CFL, make_batch
    from openvdb_gb300 import DeviceBatch
    spec = BATCH_CFL if key == "__batch_cfl05__" else BATCH
    gold = GOLD[key]
    grids, fields = make_batch()
    for g, rec in zip(grids, gold):
        assert digest(g) == rec[0]["digest"]
    b = DeviceBatch(grids)
    b.set_precision(PARITY)
    sp, tp, tsp, ttp, nc = spec["schemes"]
    b.set_tracker(tsp, ttp, nc)
    for step, (t0, t1) in enumerate(spec["ops"], start=1):
        counts = b.advect(fields, t0, t1, spatial=sp, temporal=tp, cfl=spec.get("cfl", 0.0))
        for i, rec in enumerate(gold):
            assert counts[i] == rec[step]["count"], (i, step, counts[i], rec[step]["count"])
            h = b.to_host(i)
            if digest(h) != rec[step]["digest"]:
                _dump("batch%d" % i, step, h)
                pytest.fail("instance %d op %d: device %s != reference %s" % (i, step, summary(h),
                                                                             rec[step]["summary"]))
