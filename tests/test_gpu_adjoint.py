"""Adjoint of advection + tracking against central finite differences.

Loss L = sum over the final band of (phi_T - phi_target)^2.  The intervals
are shorter than the CFL limit, so every substep takes dt = the interval and
dt does not depend on the velocity; directions whose perturbed forward runs
change the topology (a voxel crossing the trim threshold) are rejected, since
the adjoint holds the recorded topology fixed.
"""
import numpy as np
import pytest

from cases import smoothed_noise


def _target(grid, radius, center):
    c = grid.active_coords().astype(np.float64)
    return (np.sqrt(((c - np.asarray(center)) ** 2).sum(1)) - radius).astype(np.float64)


def _loss(phi, grid, radius, center):
    d = phi.astype(np.float64) - _target(grid, radius, center)
    return float((d * d).sum()), 2.0 * d


@pytest.mark.gpu
def test_adjoint_matches_finite_differences():
    from openvdb_gb300 import PARITY, digest, fixtures
    from openvdb_gb300.adjoint import AdvectionTape

    center, r0, rt = (16.0, 16.0, 16.0), 9.0, 10.0
    template = fixtures.sphere(r0, center)
    vel = smoothed_noise(32, 3.0, 0.8, seed=5)
    times = [0.0, 0.3, 0.6, 0.9, 1.2]
    tape = AdvectionTape(template, vel, mode=PARITY)
    phi0 = template.active_values().copy()
    phiT, gT = tape.forward(phi0, times)
    assert all(n == 1 for n in tape.substeps)
    L0, dL = _loss(phiT, gT, rt, center)
    g_phi, g_vel = tape.backward(dL.astype(np.float32))
    assert np.isfinite(g_phi).all() and np.isfinite(g_vel).all()
    assert np.abs(g_phi).max() > 0 and np.abs(g_vel).max() > 0

    rng = np.random.Generator(np.random.PCG64(1234))
    h = 1e-4
    ref_digest = None
    checked, worst = 0, 0.0
    for trial in range(24):
        dphi = rng.standard_normal(phi0.size).astype(np.float32)
        dv = rng.standard_normal(vel.shape).astype(np.float32) * (trial % 2)
        vals = []
        topo = []
        for sgn in (1.0, -1.0):
            tape.set_velocity(vel + sgn * h * dv)
            p, g = tape.forward(phi0 + sgn * h * dphi, times, record=False)
            topo.append((g.leaf_origins.tobytes(), g.leaf_masks.tobytes(), tuple(tape.substeps)))
            vals.append((p, g))
        tape.set_velocity(vel)
        base = (gT.leaf_origins.tobytes(), gT.leaf_masks.tobytes(), tuple([1] * 4))
        if topo[0] != base or topo[1] != base:
            continue
        Lp = _loss(vals[0][0], vals[0][1], rt, center)[0]
        Lm = _loss(vals[1][0], vals[1][1], rt, center)[0]
        fd = (Lp - Lm) / (2 * h)
        ad = float(np.dot(g_phi.astype(np.float64), dphi) + np.dot(g_vel.reshape(-1).astype(np.float64),
                                                                   dv.reshape(-1)))
        rel = abs(fd - ad) / max(abs(fd), abs(ad), 1e-12)
        print("direction %d (velocity %s): fd %.6g adjoint %.6g rel %.2e" % (trial, bool(trial % 2), fd, ad, rel))
        worst = max(worst, rel)
        checked += 1
        if checked >= 8:
            break
    assert checked >= 4, checked
    assert worst < 2e-2, worst
