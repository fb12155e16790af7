"""The FP64 instance on the device (GBLS_MODE_FP64) against the oracle's FP64
instance.

Both run the FloatGrid scheme of LevelSetAdvection / LevelSetTracker with
the level set's values in double: WENO5, the RK stages, the Eikonal update
and the trim thresholds in double, the scheme's constants as floats,
velocities sampled as Vec3f, substep lengths and time in double.  Every
double operation rounds once on both sides, so the device's band (leaf
origins and active masks) and its active values must equal the oracle's bit
for bit, after every call: RK1/RK2/RK3 advection, the normaliser's RK1/RK2
stages, the imposed CFL 0.5 and the reference CFL, backward time, constant,
deformation, rotation and dense velocity fields.  The last test states the
FP32 (PARITY) run's error against the device FP64 run.
"""
import numpy as np
import pytest

from openvdb_gb300 import FP64, PARITY, DeviceLevelSet, Field, LevelSetAdvection, fixtures
from openvdb_gb300.grid import topology_equal
from openvdb_gb300.levelset import TVD_RK1, TVD_RK2, TVD_RK3

port = pytest.importorskip("oracle.port")


def _dense_field(n=48, seed=3):
    rng = np.random.Generator(np.random.PCG64(seed))
    v = (0.6 * rng.standard_normal((n, n, n, 3))).astype(np.float32)
    return Field.dense(v, origin=(-n // 2, -n // 2, -n // 2), background=(0.1, -0.2, 0.3))


CASES = {
    # name: (grid, field, spatial-temporal schemes, calls (t0, t1), cfl)
    "sphere_const_rk3": (lambda: fixtures.sphere(12.0, (3.5, -7.25, 1.0)), lambda: Field.constant_field((1.0, 0.5, 0.25)),
                         (TVD_RK3, TVD_RK1, 1), [(0.0, 1.0), (1.0, 2.0), (2.0, 3.0)], 0.0),
    "union_deform_cfl05": (lambda: fixtures.union_of_spheres(*fixtures.sixty_four_spheres(seed=5, n=6, domain=128.0,
                                                                                          rmin=8.0, rmax=20.0)),
                           lambda: Field.deformation(domain=128.0, period=20.0, scale=1.0),
                           (TVD_RK3, TVD_RK1, 1), [(0.0, 1.0), (1.0, 2.0)], 0.5),
    "sphere_rot_rk2_norm2": (lambda: fixtures.sphere(10.0, (2.0, 1.0, -3.0)),
                             lambda: Field.rotation((0.1, 0.0, -0.1), (0.02, -0.01, 0.03), (1.0, 0.0, -2.0)),
                             (TVD_RK2, TVD_RK2, 2), [(0.0, 2.0)], 0.0),
    "torus_backward_rk1": (lambda: fixtures.torus(14.0, 4.0, (1.0, 2.0, -1.0)),
                           lambda: Field.constant_field((-0.7, 0.3, 0.9)),
                           (TVD_RK1, TVD_RK1, 1), [(2.0, 0.5)], 0.5),
    "sphere_dense": (lambda: fixtures.sphere(9.0, (0.5, -0.5, 1.5)), _dense_field, (TVD_RK3, TVD_RK3, 1),
                     [(0.0, 1.5)], 0.5),
}


def _port_and_device(case):
    make_grid, make_field, (temporal, tr_temporal, norm_count), calls, cfl = CASES[case]
    g = make_grid()
    field = make_field()
    p = port.PortGrid(g, precision=64)
    d = DeviceLevelSet(g)
    d.set_precision(FP64)
    adv = LevelSetAdvection(d, field)
    adv.setTemporalScheme(temporal)
    adv.setTrackerTemporalScheme(tr_temporal)
    adv.setNormCount(norm_count)
    adv.cfl = cfl
    return p, d, adv, field, calls, (temporal, tr_temporal, norm_count, cfl)


@pytest.mark.gpu
@pytest.mark.parametrize("case", list(CASES))
def test_fp64_instance_matches_oracle_fp64(case):
    p, d, adv, field, calls, (temporal, tr_temporal, norm_count, cfl) = _port_and_device(case)
    for t0, t1 in calls:
        n_port = p.advect(field.desc(), t0, t1, spatial=port.HJWENO5_BIAS, temporal=temporal,
                          tracker_spatial=port.HJWENO5_BIAS, tracker_temporal=tr_temporal, norm_count=norm_count,
                          cfl=cfl)
        n_dev = adv.advect(t0, t1)
        assert n_dev == n_port, (t0, t1, n_dev, n_port)
        hp, hd = p.to_host(), d.to_host()
        assert topology_equal(hd, hp), (t0, t1)
        vp, vd = p.active_values(), d.active_values_f64()
        assert vp.shape == vd.shape
        bad = np.flatnonzero(vp.view(np.uint64) != vd.view(np.uint64))
        assert bad.size == 0, (t0, t1, bad[:5], vp[bad[:5]], vd[bad[:5]])
        # the FP32 download rounds the doubles
        assert np.array_equal(hd.active_values(), vd.astype(np.float32))
    d.close()


@pytest.mark.gpu
def test_fp64_mode_round_trip_and_refusals():
    """Widening is exact and narrowing rounds; FP32-only operations refuse
    an FP64 level set."""
    from openvdb_gb300._lib import GblsError
    from openvdb_gb300.nanovdb import export_device
    g = fixtures.sphere(12.0, (3.5, -7.25, 1.0))
    d = DeviceLevelSet(g)
    v32 = d.active_values_f64()
    d.set_precision(FP64)
    assert np.array_equal(d.active_values_f64(), v32)
    d.set_precision(PARITY)
    assert np.array_equal(d.active_values_f64(), v32)
    d.set_precision(FP64)
    with pytest.raises(GblsError):
        export_device(d, "x")
    adv = LevelSetAdvection(d, Field.constant_field((1.0, 0.0, 0.0)))
    adv.setSpatialScheme(0)  # FIRST_BIAS
    with pytest.raises(Exception):
        adv.advect(0.0, 1.0)
    d.close()


@pytest.mark.gpu
def test_fp32_error_against_device_fp64():
    """The FP32 PARITY run against the device FP64 run on the 6-sphere
    deformation case: the error statement's form, small and with the same
    substeps."""
    make_grid, make_field, _, calls, cfl = CASES["union_deform_cfl05"]
    g = make_grid()
    runs = []
    for mode in (PARITY, FP64):
        d = DeviceLevelSet(g)
        d.set_precision(mode)
        adv = LevelSetAdvection(d, make_field())
        adv.setTemporalScheme(TVD_RK3)
        adv.setTrackerTemporalScheme(TVD_RK1)
        adv.setNormCount(1)
        adv.cfl = cfl
        n = [adv.advect(t0, t1) for t0, t1 in calls]
        runs.append((n, d.to_host(), d.active_values_f64()))
        d.close()
    (n32, h32, v32), (n64, h64, v64) = runs
    assert n32 == n64
    if topology_equal(h32, h64):
        err = np.abs(v32 - v64).max() / g.background
        print("max |phi32 - phi64| / gamma = %.3g" % err)
        assert err < 1e-4


@pytest.mark.gpu
def test_fp64_upload_and_empty_grid():
    """A new level set uploaded into an FP64 handle is widened; an empty
    level set advects to nothing; gbls_get_counts and downloads work."""
    from openvdb_gb300 import HostGrid
    g1 = fixtures.sphere(12.0, (3.5, -7.25, 1.0))
    g2 = fixtures.torus(14.0, 4.0, (1.0, 2.0, -1.0))
    d = DeviceLevelSet(g1)
    d.set_precision(FP64)
    d.upload(g2)
    assert np.array_equal(d.active_values_f64(), g2.active_values().astype(np.float64))
    p = port.PortGrid(g2, precision=64)
    field = Field.constant_field((0.4, -0.8, 0.3))
    adv = LevelSetAdvection(d, field)
    adv.setTemporalScheme(TVD_RK3)
    adv.setTrackerTemporalScheme(TVD_RK1)
    adv.setNormCount(1)
    adv.cfl = 0.5
    assert adv.advect(0.0, 1.0) == p.advect(field.desc(), 0.0, 1.0, spatial=port.HJWENO5_BIAS, temporal=TVD_RK3,
                                             tracker_spatial=port.HJWENO5_BIAS, tracker_temporal=TVD_RK1,
                                             norm_count=1, cfl=0.5)
    assert np.array_equal(d.active_values_f64(), p.active_values())
    d.close()
    e = DeviceLevelSet(HostGrid(voxel_size=1.0, background=3.0))
    e.set_precision(FP64)
    assert LevelSetAdvection(e, field).advect(0.0, 1.0) == 0
    assert e.active_voxel_count() == 0 and e.active_values_f64().size == 0
    e.close()
