"""Host fixtures against the reference (CPU)."""
import json
import os

import pytest

from cases import CASES, make_fixture
from openvdb_gb300 import bitwise_equal, digest
from openvdb_gb300 import fixtures

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "parity_cases.json")))


@pytest.mark.parametrize("name", list(CASES))
def test_fixture_matches_reference_input(name):
    """The input of every parity case equals the one the reference ran on."""
    assert digest(make_fixture(CASES[name]["fixture"])) == GOLD[name][0]["digest"]


def test_sphere_against_compiled_reference():
    refpy = pytest.importorskip("oracle.refpy")
    if not refpy.available():
        pytest.skip("reference oracle library not built on this host")
    for (r, c, dx, w) in [(64.0, (0, 0, 0), 1.0, 3.0), (20.0, (3.3, -7.1, 12.9), 1.0, 3.0),
                          (7.5, (0.5, 0.25, 0.125), 0.5, 3.0), (40.0, (100, -50, 2000), 1.0, 4.0),
                          (1.2, (0, 0, 0), 1.0, 3.0)]:
        mine = fixtures.sphere(r, c, dx, w)
        ref = refpy.RefGrid.sphere(r, c, dx, w).to_host()
        assert bitwise_equal(mine, ref), (r, c, dx, w)


def test_sphere_argument_errors():
    from openvdb_gb300._lib import GblsError
    with pytest.raises(GblsError):
        fixtures.sphere(-1.0)
    with pytest.raises(GblsError):
        fixtures.sphere(5.0, half_width=1.0)
