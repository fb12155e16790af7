"""Adjoint of advection + tracking against an FP64 reference gradient.

Loss L = sum over the final band of (phi_T - phi_target)^2.  The reference
gradient comes from central differences of the FP64 run of the same scheme
(the oracle's restatement compiled for double: same constants, same
operations) with h = 1e-6 along seeded dense directions in phi_0 and h = 1e-4
along seeded sparse directions in the velocity grid; in FP64 the
difference is neither limited by rounding nor, at that step, by the strong
nonlinearity of the WENO5 weights.  The adjoint under test is the GPU
reverse sweep of the FP32 forward pass.  It holds the recorded topology,
upwind directions, Godunov branches, trimming and CFL time steps fixed;
probes whose perturbed FP64 runs change the topology after any interval are
rejected, and
velocity probes use intervals below the CFL limit so that dt does not depend
on the velocity, and perturb only components away from zero, where the
upwind side (fixed in the adjoint) cannot switch.
"""
import time

import numpy as np
import pytest

from cases import smoothed_noise


def _sdf_sphere(coords, radius, center):
    return np.sqrt(((coords.astype(np.float64) - np.asarray(center)) ** 2).sum(1)) - radius


def _fp64_loss(template, phi0, field, times, target_fn):
    from oracle import port
    g = port.PortGrid(template, precision=64)
    g.set_active_values(phi0)
    # substep counts and the topology after every interval: a voxel trimmed
    # in one interval and re-activated in a later one leaves the final
    # topology unchanged but makes L jump
    trail = []
    for k in range(len(times) - 1):
        n = g.advect(field, times[k], times[k + 1], temporal=2, tracker_temporal=0, norm_count=1)
        host = g.to_host()
        trail.append((n, host.leaf_origins.tobytes(), host.leaf_masks.tobytes()))
    d = g.active_values() - target_fn(host.active_coords())
    return float((d * d).sum()), host, trail


def _same_topology(a, b):
    return np.array_equal(a.leaf_origins, b.leaf_origins) and np.array_equal(a.leaf_masks, b.leaf_masks)


def _check_case(template, vel, times, target_fn, nprobe, vel_probes, tol_median, tol_max, seed):
    from openvdb_gb300 import PARITY, Field
    from openvdb_gb300.adjoint import AdvectionTape
    port = pytest.importorskip("oracle.port")
    assert port.available()

    tape = AdvectionTape(template, vel, mode=PARITY)
    phi0 = template.active_values().copy()
    phiT, gT = tape.forward(phi0, times)
    d = phiT.astype(np.float64) - target_fn(gT.active_coords())
    g_phi, g_vel = tape.backward((2.0 * d).astype(np.float32))
    assert np.isfinite(g_phi).all() and np.isfinite(g_vel).all()

    base_field = Field.dense(vel)
    _, host0, counts0 = _fp64_loss(template, phi0.astype(np.float64), base_field, times, target_fn)
    assert _same_topology(host0, gT), "FP64 run and FP32 run differ in topology"
    rng = np.random.Generator(np.random.PCG64(seed))
    c = template.active_coords()
    inside = ((c >= 0) & (c < np.array(vel.shape[:3]))).all(1)
    vox = np.ravel_multi_index(c[inside].T, vel.shape[:3])
    comp = (vox[:, None] * 3 + np.arange(3)).reshape(-1)
    cand = comp[np.abs(vel.reshape(-1)[comp]) > 0.05]
    errs, kinds = [], []
    for k in range(nprobe):
        is_vel = vel_probes and k % 2 == 1
        if is_vel:
            h = 1e-4
            # sparse: 32 components at voxels of the initial band, away from
            # v = 0 (where the upwind side, fixed in the adjoint, switches); a
            # dense direction moves every voxel and crosses Godunov/upwind
            # kinks, which leaves its difference quotient uncertain at 1e-2
            dv = np.zeros(vel.shape, np.float32)
            pick = rng.choice(cand, 32, replace=False)
            dv.reshape(-1)[pick] = rng.standard_normal(32)
            vp = (vel + h * dv).astype(np.float32)
            vm = (vel - h * dv).astype(np.float32)
            Lp, hp, cp = _fp64_loss(template, phi0.astype(np.float64), Field.dense(vp), times, target_fn)
            Lm, hm, cm = _fp64_loss(template, phi0.astype(np.float64), Field.dense(vm), times, target_fn)
            ad = float(np.dot(g_vel.reshape(-1).astype(np.float64),
                              (vp.astype(np.float64) - vm.astype(np.float64)).reshape(-1))) / (2 * h)
            gnorm = float(np.linalg.norm(g_vel.reshape(-1)[pick].astype(np.float64)))
        else:
            h = 1e-6
            dphi = rng.standard_normal(phi0.size)
            Lp, hp, cp = _fp64_loss(template, phi0 + h * dphi, base_field, times, target_fn)
            Lm, hm, cm = _fp64_loss(template, phi0 - h * dphi, base_field, times, target_fn)
            ad = float(np.dot(g_phi.astype(np.float64), dphi))
            gnorm = float(np.linalg.norm(g_phi.astype(np.float64)))
        if not (cp == counts0 and cm == counts0):
            continue
        fd = (Lp - Lm) / (2 * h)
        # g.d of a standard normal direction d has the scale |g| on the
        # direction's support; a direction nearly orthogonal to g is measured
        # against a tenth of that scale, not against its own tiny |fd|
        rel = abs(fd - ad) / max(abs(fd), 0.1 * gnorm, 1e-12)
        errs.append(rel)
        kinds.append(is_vel)
        print("%s probe %d: fp64 fd %+.9e adjoint %+.9e rel %.2e" % ("vel" if is_vel else "phi", k, fd, ad, rel))
    assert len(errs) >= nprobe * 3 // 4, len(errs)
    errs, kinds = np.array(errs), np.array(kinds)
    for name, sel in (("phi", ~kinds), ("velocity", kinds)):
        if sel.any():
            print("%s probes: relative error median %.2e max %.2e over %d probes"
                  % (name, np.median(errs[sel]), errs[sel].max(), sel.sum()))
    assert np.median(errs) < tol_median and errs.max() < tol_max
    return tape


@pytest.mark.gpu
def test_adjoint_matches_fp64_reference_gradient():
    from openvdb_gb300 import fixtures
    center, r0, rt = (16.0, 16.0, 16.0), 9.0, 10.0
    template = fixtures.sphere(r0, center)
    vel = smoothed_noise(32, 3.0, 0.8, seed=5)
    times = [0.0, 0.3, 0.6, 0.9, 1.2]  # below the CFL limit: dt = 0.3 independent of v
    _check_case(template, vel, times, lambda c: _sdf_sphere(c, rt, center), nprobe=64, vel_probes=True,
                tol_median=1e-3, tol_max=1e-2, seed=1234)


@pytest.mark.gpu
def test_adjoint_inverse_problem_128():
    """The 128^3 adjoint configuration: phi_0 a radius-40 sphere, the target a
    seeded 5%-perturbed radius-44 sphere, a seeded smoothed-noise velocity
    grid (sigma 4 voxels, amplitude 1 voxel per time unit), 20 unit steps of
    RK3-HJWENO5; dL/dphi_0 against the FP64 reference on seeded probes, and
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

    def target(coords):
        c = coords.astype(np.float64) - center
        r = np.linalg.norm(c, axis=1)
        n = c / np.maximum(r, 1e-9)[:, None]
        return r - 44.0 * (1.0 + 0.05 * (n @ axes.T) @ amps)

    template = fixtures.sphere(40.0, tuple(center))
    vel = smoothed_noise(128, 4.0, 1.0, seed=9)
    times = [float(t) for t in range(21)]
    tape = AdvectionTape(template, vel, mode=FAST)
    phi0 = template.active_values().copy()
    tape.forward(phi0, times, record=False)  # warm-up
    torch.cuda.synchronize()
    # best of three of each (wall times of about 10 ms)
    t_plain = t_rec = t_adj = float("inf")
    for _ in range(3):
        t0 = time.perf_counter()
        tape.forward(phi0, times, record=False)
        t_plain = min(t_plain, time.perf_counter() - t0)
    for _ in range(3):
        t0 = time.perf_counter()
        phiT, gT = tape.forward(phi0, times, record=True)
        t_rec = min(t_rec, time.perf_counter() - t0)
        d = phiT.astype(np.float64) - target(gT.active_coords())
        t0 = time.perf_counter()
        g_phi, g_vel = tape.backward((2.0 * d).astype(np.float32))
        t_adj = min(t_adj, time.perf_counter() - t0)
    print("adjoint 128^3: %d substeps, %d -> %d active voxels, L = %.6g" % (sum(tape.substeps), phi0.size,
                                                                            phiT.size, float((d * d).sum())))
    print("wall time: forward %.3f s, recorded forward %.3f s, adjoint %.3f s, (fwd+adj)/fwd = %.2f"
          % (t_plain, t_rec, t_adj, (t_rec + t_adj) / t_plain))
    assert (t_rec + t_adj) / t_plain < 3.5
    assert np.isfinite(g_phi).all() and np.isfinite(g_vel).all() and np.abs(g_vel).max() > 0
    # dL/dphi_0 against the FP64 reference (the PARITY forward matches the FP64 topology)
    _check_case(template, vel, times, target, nprobe=8, vel_probes=False, tol_median=1e-2, tol_max=5e-2,
                seed=77)


@pytest.mark.gpu
def test_checkpointed_matches_single_tape():
    """Segments of 2 intervals with recompute give the gradients of one tape
    over the whole horizon (dL/dv accumulated on the device; float atomics
    make the sums order-dependent, hence a relative tolerance)."""
    import torch
    from openvdb_gb300 import FAST, fixtures
    from openvdb_gb300.adjoint import AdvectionTape, CheckpointedAdvection
    center = (16.0, 16.0, 16.0)
    template = fixtures.sphere(9.0, center)
    vel = smoothed_noise(32, 3.0, 0.8, seed=5)
    times = [0.0, 0.5, 1.0, 1.5, 2.0, 2.5, 3.0]
    phi0 = template.active_values().copy()
    tape = AdvectionTape(template, vel, mode=FAST, cfl=0.5)
    phiT, gT = tape.forward(phi0, times)
    d = phiT.astype(np.float64) - _sdf_sphere(gT.active_coords(), 10.0, center)
    g_phi, g_vel = tape.backward((2.0 * d).astype(np.float32))

    ck = CheckpointedAdvection(template, vel, every=2, mode=FAST, cfl=0.5)
    phiT2, gT2 = ck.forward(phi0, times)
    assert np.array_equal(phiT2, phiT) and ck.substeps == sum(tape.substeps)
    g_phi2, dvel, recorded = ck.backward((2.0 * d).astype(np.float32))
    g_vel2 = dvel.cpu().numpy()
    assert recorded == ck.substeps and len(ck.segments) == 3
    assert np.abs(g_phi2 - g_phi).max() <= 1e-5 * np.abs(g_phi).max()
    assert np.abs(g_vel2 - g_vel).max() <= 1e-5 * np.abs(g_vel).max()
    torch.cuda.synchronize()
