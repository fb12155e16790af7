"""Adjoint of advection + tracking against central finite differences.

Loss L = sum over the final band of (phi_T - phi_target)^2.  The adjoint holds
the recorded topology, upwind directions, Godunov branches, trimming and CFL
time steps fixed, so each probe direction perturbs a few seeded voxels of
phi_0 (or a few cells of the velocity grid): a dense perturbation moves some
voxel across the trim threshold and changes the topology, which the
finite difference would see as a jump.  Probes whose perturbed runs change
the topology are rejected.
"""
import time

import numpy as np
import pytest

from cases import smoothed_noise


def _sdf_sphere(grid, radius, center):
    c = grid.active_coords().astype(np.float64)
    return np.sqrt(((c - np.asarray(center)) ** 2).sum(1)) - radius


def _loss(phi, target):
    d = phi.astype(np.float64) - target
    return float((d * d).sum()), 2.0 * d


def _same_topology(a, b):
    return np.array_equal(a.leaf_origins, b.leaf_origins) and np.array_equal(a.leaf_masks, b.leaf_masks)


def _probe(tape, phi0, vel, times, gT, target_fn, g_phi, g_vel, rng, kind, h, nsel=8):
    dphi = np.zeros_like(phi0)
    dv = np.zeros_like(vel)
    if kind == "phi":
        idx = rng.choice(phi0.size, nsel, replace=False)
        dphi[idx] = rng.standard_normal(nsel).astype(np.float32)
    else:
        flat = dv.reshape(-1)
        idx = rng.choice(flat.size, nsel, replace=False)
        flat[idx] = rng.standard_normal(nsel).astype(np.float32)
    vals = []
    for sgn in (1.0, -1.0):
        tape.set_velocity(vel + sgn * h * dv)
        p, g = tape.forward(phi0 + sgn * h * dphi, times, record=False)
        if not _same_topology(g, gT):
            tape.set_velocity(vel)
            return None
        vals.append(_loss(p, target_fn(g))[0])
    tape.set_velocity(vel)
    fd = (vals[0] - vals[1]) / (2 * h)
    ad = float(np.dot(g_phi.astype(np.float64), dphi) + np.dot(g_vel.reshape(-1).astype(np.float64), dv.reshape(-1)))
    return fd, ad


@pytest.mark.gpu
def test_adjoint_matches_finite_differences():
    from openvdb_gb300 import PARITY, fixtures
    from openvdb_gb300.adjoint import AdvectionTape

    center, r0, rt = (16.0, 16.0, 16.0), 9.0, 10.0
    template = fixtures.sphere(r0, center)
    vel = smoothed_noise(32, 3.0, 0.8, seed=5)
    times = [0.0, 0.3, 0.6, 0.9, 1.2]  # below the CFL limit: dt independent of v
    tape = AdvectionTape(template, vel, mode=PARITY)
    phi0 = template.active_values().copy()
    phiT, gT = tape.forward(phi0, times)
    assert tape.substeps == [1, 1, 1, 1]
    target = lambda g: _sdf_sphere(g, rt, center)
    _, dL = _loss(phiT, target(gT))
    g_phi, g_vel = tape.backward(dL.astype(np.float32))
    assert np.isfinite(g_phi).all() and np.isfinite(g_vel).all()
    rng = np.random.Generator(np.random.PCG64(1234))
    checked = {"phi": 0, "vel": 0}
    for trial in range(40):
        kind = "phi" if trial % 2 == 0 else "vel"
        r = _probe(tape, phi0, vel, times, gT, target, g_phi, g_vel, rng, kind, 1e-3)
        if r is None:
            continue
        fd, ad = r
        scale = max(abs(fd), abs(ad), 1e-3)
        tol = 1e-2 if kind == "phi" else 5e-2  # velocity probes cross upwind switches at v = 0
        print("%s probe %d: fd %+.6e adjoint %+.6e rel %.2e" % (kind, trial, fd, ad, abs(fd - ad) / scale))
        assert abs(fd - ad) <= tol * scale + 1e-3, (kind, trial, fd, ad)
        checked[kind] += 1
        if min(checked.values()) >= 8:
            break
    assert min(checked.values()) >= 6, checked


@pytest.mark.gpu
def test_adjoint_inverse_problem_scale_and_cost():
    """The 128^3 adjoint configuration: phi_0 a radius-40 sphere, the target
    a seeded 5%-perturbed radius-44 sphere, a seeded smoothed-noise velocity
    grid (sigma 4 voxels, amplitude 1), 20 unit steps; probes of dL/dphi_0 and
    the cost of forward + adjoint against the plain forward pass."""
    import torch
    from openvdb_gb300 import FAST, fixtures
    from openvdb_gb300.adjoint import AdvectionTape

    center = np.array([64.0, 64.0, 64.0])
    rng = np.random.Generator(np.random.PCG64(44))
    axes = rng.standard_normal((4, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    amps = rng.uniform(-1.0, 1.0, 4)
    amps /= np.abs(amps).sum()

    def target(g):
        c = g.active_coords().astype(np.float64) - center
        r = np.linalg.norm(c, axis=1)
        n = c / np.maximum(r, 1e-9)[:, None]
        return r - 44.0 * (1.0 + 0.05 * (n @ axes.T) @ amps)

    template = fixtures.sphere(40.0, tuple(center))
    vel = smoothed_noise(128, 4.0, 1.0, seed=9)
    times = [float(t) for t in range(21)]
    tape = AdvectionTape(template, vel, mode=FAST)
    phi0 = template.active_values().copy()
    # plain forward, then forward with the tape, then the adjoint
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tape.forward(phi0, times, record=False)
    t_plain = time.perf_counter() - t0
    t0 = time.perf_counter()
    phiT, gT = tape.forward(phi0, times, record=True)
    t_rec = time.perf_counter() - t0
    L, dL = _loss(phiT, target(gT))
    t0 = time.perf_counter()
    g_phi, g_vel = tape.backward(dL.astype(np.float32))
    t_adj = time.perf_counter() - t0
    print("adjoint 128^3: %d substeps, %d -> %d active voxels, L = %.6g" % (sum(tape.substeps), phi0.size,
                                                                            phiT.size, L))
    print("wall time: forward %.3f s, recorded forward %.3f s, adjoint %.3f s, (fwd+adj)/fwd = %.2f"
          % (t_plain, t_rec, t_adj, (t_rec + t_adj) / t_plain))
    assert np.isfinite(g_phi).all() and np.isfinite(g_vel).all()
    assert np.abs(g_vel).max() > 0
    checked = 0
    for trial in range(12):
        r = _probe(tape, phi0, vel, times, gT, target, g_phi, g_vel, rng, "phi", 1e-3)
        if r is None:
            continue
        fd, ad = r
        scale = max(abs(fd), abs(ad), 1e-3)
        print("phi probe %d: fd %+.6e adjoint %+.6e rel %.2e" % (trial, fd, ad, abs(fd - ad) / scale))
        assert abs(fd - ad) <= 2e-2 * scale + 1e-3, (trial, fd, ad)
        checked += 1
        if checked >= 4:
            break
    assert checked >= 3
