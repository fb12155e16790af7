"""Error of the FP32 path against an FP64 run of the same scheme (CPU).

The oracle's restatement compiled for double (same constants and
operations) serves as the FP64 reference; the FP32 restatement is
bit-identical to the reference, so this states the reference's own FP32
error on each configuration.
"""
import numpy as np
import pytest

from cases import CASES, make_field, make_fixture

port = pytest.importorskip("oracle.port")
if not port.available():
    pytest.skip("oracle port not built", allow_module_level=True)


@pytest.mark.parametrize("name", ["cfg1_sphere64", "sphere20_deformation", "union8_deformation",
                                  "sphere12_dense_noise", "sphere16_rotation_backward"])
def test_fp32_error_against_fp64(name):
    case = CASES[name]
    host = make_fixture(case["fixture"])
    field = make_field(case["field"])
    sp, tp, tsp, ttp, nc = case["schemes"]
    a = port.PortGrid(host, precision=32)
    b = port.PortGrid(host, precision=64)
    for op in case["ops"]:
        kw = dict(spatial=sp, temporal=tp, tracker_spatial=tsp, tracker_temporal=ttp, norm_count=nc)
        assert a.advect(field, op[1], op[2], **kw) == b.advect(field, op[1], op[2], **kw)
    ha, hb = a.to_host(), b.to_host()
    assert np.array_equal(ha.leaf_origins, hb.leaf_origins) and np.array_equal(ha.leaf_masks, hb.leaf_masks)
    err = float(np.abs(a.active_values() - b.active_values()).max())
    band = 2.0 * ha.background
    print("%s: max |phi_fp32 - phi_fp64| = %.3g (%.3g of the band width)" % (name, err, err / band))
    assert err / band < 1e-5
