"""HOST_SAMPLED velocity fields: any functor, sampled on the host per substep.

The library hands the sampler the active voxels' index coordinates in the
reference's velocity order (tools/LevelSetAdvect.h:426-493) and reads the
velocities back per voxel.  A sampler that returns the values of an aligned
dense field, or a constant, must give exactly the grid that the device-side
DENSE / CONSTANT kinds give, forward and backward in time; the reference's
own default field (EnrightField) is pinned against the compiled reference in
test_gpu_parity.py (case enright_sphere_default_field).
"""
import numpy as np
import pytest

from openvdb_gb300 import PARITY, DeviceLevelSet, Field, LevelSetAdvection, digest, fixtures

LO, N = -26, 53  # dense box [LO, LO + N) on every axis


def _noise():
    rng = np.random.Generator(np.random.PCG64(5))
    return (0.6 * rng.standard_normal((N, N, N, 3))).astype(np.float32)


def _run(field, steps):
    dev = DeviceLevelSet(fixtures.sphere(16.0, (0.5, -1.0, 1.5), 1.0, 3.0))
    dev.set_precision(PARITY)
    adv = LevelSetAdvection(dev, field)
    adv.setTemporalScheme(2)  # TVD_RK3
    adv.setNormCount(1)
    out = []
    for t0, t1 in steps:
        n = adv.advect(t0, t1)
        out.append((n, digest(dev.to_host())))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("steps", [[(0.0, 1.0), (1.0, 2.0)], [(2.0, 1.0), (1.0, 0.5)]], ids=["forward", "backward"])
def test_host_sampled_equals_dense(steps):
    vel = _noise()

    def sample(ijk, t):
        q = ijk - LO
        inside = np.all((q >= 0) & (q < N), axis=1)
        v = np.zeros((len(ijk), 3), np.float32)
        v[inside] = vel[q[inside, 0], q[inside, 1], q[inside, 2]]
        return v

    host = _run(Field.host_sampled(sample), steps)
    dense = _run(Field.dense(vel, origin=(LO, LO, LO), background=(0.0, 0.0, 0.0)), steps)
    assert host == dense


@pytest.mark.gpu
def test_host_sampled_constant_equals_constant():
    c = np.array([1.0, 0.5, 0.25], np.float32)
    host = _run(Field.host_sampled(lambda ijk, t: np.broadcast_to(c, (len(ijk), 3))), [(0.0, 1.0), (1.0, 3.0)])
    const = _run(Field.constant_field(tuple(c)), [(0.0, 1.0), (1.0, 3.0)])
    assert host == const
