"""VolumeAdvection (tools/VolumeAdvect.h) on the device against digests made
by the reference's own VolumeAdvection<Vec3fGrid>::advect<FloatGrid,
BoxSampler> (tests/golden/parity_cases.json, "__volume__"): every
integrator (SEMI, MID, RK3, RK4, MacCormack, BFECC), every limiter, substeps,
a velocity grid with its own transform, a constant velocity and a half-voxel
volume."""
import json
import os

import pytest

from cases import VOLUME_CASES, make_field, make_volume

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "parity_cases.json")))["__volume__"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(VOLUME_CASES))
def test_volume_advection_bit_exact(name):
    from openvdb_gb300 import DeviceVolume, VolumeAdvection, digest, summary
    case, gold = VOLUME_CASES[name], GOLD[name]
    host = make_volume(case["volume"])
    assert digest(host) == gold[0]["digest"]
    dev = DeviceVolume(host)
    adv = VolumeAdvection(make_field(case["field"]))
    for op, want in zip(case["ops"], gold[1:]):
        _, integ, lim, sub, dt = op
        adv.setIntegrator(integ)
        adv.setLimiter(lim)
        adv.setSubSteps(sub)
        adv.advect(dev, dt)
        assert adv.getMaxVelocity() == want["max_velocity"], op
        got = dev.to_host()
        assert summary(got) == want["summary"], (op, summary(got), want["summary"])
        assert digest(got) == want["digest"], op


@pytest.mark.gpu
def test_volume_handles_refuse_level_set_operations():
    from openvdb_gb300 import DeviceVolume, LevelSetTracker
    dev = DeviceVolume(make_volume(("fog_shell", 6.0, (0.0, 0.0, 0.0), 1.0)))
    with pytest.raises(Exception):
        LevelSetTracker(dev).normalize()
