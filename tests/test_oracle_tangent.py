"""The oracle's tangent-linear instance: FP32 values bit-identical to the
FP32 instance, and FP64 directional derivatives that agree with central
differences of the FP64 instance run on the tangent run's band (the
references the adjoint tests use).  CPU only."""
import numpy as np
import pytest

from cases import smoothed_noise
from gradient_ref import Problem, relative_errors, unit_rows, velocity_probe

port = pytest.importorskip("oracle.port")


def _problem(cfl):
    from openvdb_gb300 import fixtures
    center = np.array([16.0, 16.0, 16.0])
    template = fixtures.sphere(9.0, tuple(center))
    vel = smoothed_noise(32, 3.0, 0.8, seed=5)

    def target(c):
        return np.sqrt(((c.astype(np.float64) - center) ** 2).sum(1)) - 10.0

    # unit intervals: CFL-limited substeps and the short last substep of each
    return Problem(template, vel, [0.0, 1.0, 2.0, 3.0], target, cfl=cfl, threads=4)


@pytest.mark.parametrize("cfl", [0.0, 0.3])
def test_tangent_matches_fp64_differences(cfl):
    assert port.available()
    pb = _problem(cfl)
    phi0 = pb.template.active_values().astype(np.float64)
    rng = np.random.Generator(np.random.PCG64(11))
    k = port.tangent_lanes()
    dphi = unit_rows(rng.standard_normal((k, phi0.size)))
    tl_phi = pb.tangents(phi0, dphi=dphi)
    # the values of the tangent run are the FP32 instance's, bit for bit
    g32, n32 = pb.run(32, phi0)
    assert n32 == pb.substeps and np.array_equal(g32.active_values(), pb.source.active_values())
    assert pb.substeps > len(pb.times) - 1  # CFL-limited substeps happen
    h = 1e-3
    vps, vms, dv = zip(*(velocity_probe(pb.vel, d, h)
                         for d in unit_rows(rng.standard_normal((k,) + pb.vel.shape))))
    tl_vel = pb.tangents(phi0, dv=np.stack(dv))
    fd_phi = np.array([pb.difference(phi0, 1e-4, dphi=d) for d in dphi])
    fd_vel = np.array([pb.difference(phi0, h, vp=vp, vm=vm) for vp, vm in zip(vps, vms)])
    e_phi = relative_errors(fd_phi, tl_phi, np.abs(tl_phi).max() * np.sqrt(phi0.size), phi0.size)
    e_vel = relative_errors(fd_vel, tl_vel, np.abs(tl_vel).max() * np.sqrt(pb.vel.size), pb.vel.size)
    print("cfl %g: phi rel err max %.2e, velocity rel err max %.2e" % (cfl, e_phi.max(), e_vel.max()))
    assert e_phi.max() < 1e-3 and e_vel.max() < 1e-3


def test_tangent_time_step_derivative():
    """A velocity direction along the velocity of the voxel that holds max
    |v| over the initial band: it changes the CFL-limited time steps (and
    the short last substep of each interval), which only carried time-step
    derivatives get right."""
    pb = _problem(0.0)
    phi0 = pb.template.active_values().astype(np.float64)
    c = pb.template.active_coords()
    v = pb.vel[c[:, 0], c[:, 1], c[:, 2]].astype(np.float64)
    i = int(np.argmax((v * v).sum(1)))
    d = np.zeros((1,) + pb.vel.shape)
    d[0, c[i, 0], c[i, 1], c[i, 2]] = v[i]
    d = unit_rows(d)
    # a step that keeps every substep's maximum at its voxel (at 1e-3 a
    # later substep's maximum switches voxels and the quotient is 1% off)
    h = 1e-4
    vp, vm, dv = velocity_probe(pb.vel, d[0], h)
    tl = pb.tangents(phi0, dv=dv[None])[0]
    fd = pb.difference(phi0, h, vp=vp, vm=vm)
    print("max-|v| direction: tangent %.9e difference %.9e" % (tl, fd))
    assert abs(tl) > 0 and abs(fd - tl) <= 1e-3 * abs(tl), (tl, fd)
