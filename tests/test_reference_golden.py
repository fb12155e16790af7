"""The committed golden digests reproduced by the reference itself.

Where the reference oracle library is built (the machine that holds the
reference checkout), the LevelSetFilter cases (with and without alpha masks)
and the masked-normalize tracker case are run again through the reference and
must give the digests stored in tests/golden/parity_cases.json.  Skipped
elsewhere (the GPU machines have only the committed digests).
"""
import json
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))


def _reference():
    refpy = pytest.importorskip("oracle.refpy")
    if not refpy.available():
        pytest.skip("reference oracle library not built on this host")
    import make_golden
    return make_golden


GOLD = json.load(open(os.path.join(HERE, "golden", "parity_cases.json")))


@pytest.mark.parametrize("name", ["filter_masked", "filter_curvature_median", "filter_sphere_ops"])
def test_filter_golden_from_reference(name):
    mg = _reference()
    from cases import FILTER_CASES
    out = mg.run_filter(FILTER_CASES[name], 1)
    assert [r["digest"] for r in out] == [r["digest"] for r in GOLD["__filter__"][name]]


def test_masked_normalize_golden_from_reference():
    mg = _reference()
    from cases import CASES
    out = mg.run_reference("tracker_masked_normalize", CASES["tracker_masked_normalize"], 1)
    assert [r.get("digest") for r in out] == [r.get("digest") for r in GOLD["tracker_masked_normalize"]]
