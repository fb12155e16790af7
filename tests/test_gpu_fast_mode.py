"""FAST (FP32) mode against PARITY mode (bit-identical to the reference).

The FAST kernels evaluate the WENO5 weights in FP32 with contracted
arithmetic, so values differ from the reference in the last bits and a voxel
within a few ulps of the trim threshold may change its active state.  The
tolerance is stated relative to the band width 2*gamma.
"""
import numpy as np
import pytest

from cases import CASES, make_field, make_fixture
from openvdb_gb300 import FAST, PARITY, DeviceLevelSet, LevelSetAdvection


def _run(name, mode, steps):
    case = CASES[name]
    dev = DeviceLevelSet(make_fixture(case["fixture"]))
    dev.set_precision(mode)
    sp, tp, tsp, ttp, nc = case["schemes"]
    adv = LevelSetAdvection(dev, make_field(case["field"]))
    adv.setSpatialScheme(sp)
    adv.setTemporalScheme(tp)
    adv.setTrackerSpatialScheme(tsp)
    adv.setTrackerTemporalScheme(ttp)
    adv.setNormCount(nc)
    out = []
    for op in case["ops"][:steps]:
        adv.advect(op[1], op[2])
        out.append(dev.to_host())
    return out


def compare(a, b):
    ka = {tuple(o): i for i, o in enumerate(a.leaf_origins.tolist())}
    common = [(ka[tuple(o)], j) for j, o in enumerate(b.leaf_origins.tolist()) if tuple(o) in ka]
    ia = np.array([c[0] for c in common], dtype=np.int64)
    ib = np.array([c[1] for c in common], dtype=np.int64)
    ma, mb = a.active_mask_bool()[ia], b.active_mask_bool()[ib]
    both = ma & mb
    diff = np.abs(a.leaf_values[ia][both].astype(np.float64) - b.leaf_values[ib][both])
    flips = int((ma ^ mb).sum()) + int(a.active_voxel_count() - ma.sum()) + int(b.active_voxel_count() - mb.sum())
    return float(diff.max()) if diff.size else 0.0, flips, int(both.sum())


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cfg1_sphere64", "sphere20_deformation", "union8_deformation"])
def test_fast_mode_close_to_parity(name):
    steps = len(CASES[name]["ops"])
    par = _run(name, PARITY, steps)
    fast = _run(name, FAST, steps)
    band = 2.0 * float(par[0].background)
    worst = 0.0
    for k, (p, f) in enumerate(zip(par, fast)):
        dmax, flips, n = compare(p, f)
        worst = max(worst, dmax / band)
        print("%s step %d: max|dphi| = %.3g (%.3g of band width), active-state flips %d of %d"
              % (name, k + 1, dmax, dmax / band, flips, n))
        assert flips == 0, (name, k, flips)
    assert worst <= 1e-5, worst
