"""Adjoint of advection + tracking against the FP64 reference gradient.

Loss L = sum over the final band of (phi_T - phi_target)^2.  The adjoint
under test is the GPU reverse sweep (FP32) of the PARITY forward pass, whose
values are bit-identical to the reference's.  It holds the recorded
topology, upwind directions, Godunov branches and trims fixed and carries
the time steps' dependence on the velocity (CFL-limited substeps through
max |v|^2, the last substep of an interval through the ones before it).

References (tests/golden/gradient_ref.py): the oracle's tangent runs, FP64
directional derivatives of the same FP32 map along every probe direction,
and central differences of the oracle's FP64 run on the tangent run's band.
Probe directions are seeded unit vectors: half in phi_0, half in the
velocity grid.
"""
import time

import numpy as np
import pytest

from cases import smoothed_noise
from gradient_ref import Problem, relative_errors, unit_rows, velocity_probe

H = 1e-3  # central-difference step along a unit direction


def _sdf_sphere(coords, radius, center):
    return np.sqrt(((coords.astype(np.float64) - np.asarray(center)) ** 2).sum(1)) - radius


def small_problem(cfl):
    from openvdb_gb300 import fixtures
    center = (16.0, 16.0, 16.0)
    template = fixtures.sphere(9.0, center)
    vel = smoothed_noise(32, 3.0, 0.8, seed=5)
    # unit intervals: CFL-limited substeps and the short last substep of each
    return Problem(template, vel, [0.0, 1.0, 2.0, 3.0], lambda c: _sdf_sphere(c, 10.0, center), cfl=cfl)


def config4_problem():
    """phi_0 a radius-40 sphere, the target a seeded 5%-perturbed radius-44
    sphere on a 128^3 domain, a seeded smoothed-noise velocity grid (sigma 4
    voxels, amplitude 1 voxel per time unit), 20 unit steps of RK3-HJWENO5
    (openvdb_gb300.fixtures.adjoint_128)."""
    from openvdb_gb300 import fixtures
    template, vel, target, times = fixtures.adjoint_128()
    return Problem(template, vel, times, target)


def probes(pb, n_phi, n_vel, seed):
    """Seeded unit directions: rows of dphi, and velocity (v+, v-, realised
    direction) triples for steps of H."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n0 = pb.template.active_values().size
    dphi = unit_rows(rng.standard_normal((n_phi, n0)))
    vel = [velocity_probe(pb.vel, d, H) for d in unit_rows(rng.standard_normal((n_vel,) + pb.vel.shape))]
    return dphi, vel


def references(pb, dphi, vel, with_differences=True):
    """Tangent derivatives and (optionally) central differences per probe."""
    phi0 = pb.template.active_values().astype(np.float64)
    dv = np.stack([p[2] for p in vel])
    tl_phi = pb.tangents(phi0, dphi=dphi)
    tl_vel = pb.tangents(phi0, dv=dv)
    fd_phi = fd_vel = None
    if with_differences:
        fd_phi = np.array([pb.difference(phi0, H, dphi=d) for d in dphi], dtype=object)
        fd_vel = np.array([pb.difference(phi0, H, vp=vp, vm=vm) for vp, vm, _ in vel], dtype=object)
    return tl_phi, tl_vel, fd_phi, fd_vel


def gpu_gradients(pb, mode, cfl):
    from openvdb_gb300.adjoint import AdvectionTape
    tape = AdvectionTape(pb.template, pb.vel, mode=mode, cfl=cfl)
    phi0 = pb.template.active_values().copy()
    phiT, gT = tape.forward(phi0, pb.times)
    r = phiT.astype(np.float64) - pb.target_fn(gT.active_coords())
    g_phi, g_vel = tape.backward((2.0 * r).astype(np.float32))
    assert np.isfinite(g_phi).all() and np.isfinite(g_vel).all()
    return tape, phiT, g_phi.astype(np.float64), g_vel.astype(np.float64)


def check(pb, mode, cfl, n_phi, n_vel, seed, tol_tangent, tol_diff):
    from openvdb_gb300 import PARITY
    tape, phiT, g_phi, g_vel = gpu_gradients(pb, mode, cfl)
    dphi, vel = probes(pb, n_phi, n_vel, seed)
    tl_phi, tl_vel, fd_phi, fd_vel = references(pb, dphi, vel)
    # the PARITY forward is the oracle's FP32 map: same substeps, same values
    assert sum(tape.substeps) == pb.substeps
    if mode == PARITY:
        assert np.array_equal(phiT.astype(np.float64), pb.source.active_values())
    ad_phi = dphi @ g_phi
    ad_vel = np.array([np.dot(g_vel.reshape(-1), p[2].reshape(-1)) for p in vel])
    e_phi = relative_errors(ad_phi, tl_phi, np.linalg.norm(g_phi), g_phi.size)
    e_vel = relative_errors(ad_vel, tl_vel, np.linalg.norm(g_vel), g_vel.size)
    ok_p = np.array([f is not None for f in fd_phi])
    ok_v = np.array([f is not None for f in fd_vel])
    f_phi = relative_errors(fd_phi[ok_p].astype(np.float64), tl_phi[ok_p], np.linalg.norm(g_phi), g_phi.size)
    f_vel = relative_errors(fd_vel[ok_v].astype(np.float64), tl_vel[ok_v], np.linalg.norm(g_vel), g_vel.size)
    a_phi = relative_errors(ad_phi[ok_p], fd_phi[ok_p].astype(np.float64), np.linalg.norm(g_phi), g_phi.size)
    a_vel = relative_errors(ad_vel[ok_v], fd_vel[ok_v].astype(np.float64), np.linalg.norm(g_vel), g_vel.size)
    for name, e in (("adjoint vs FP64 tangent, dL/dphi0", e_phi), ("adjoint vs FP64 tangent, dL/dv", e_vel),
                    ("FP64 difference vs tangent, dL/dphi0", f_phi), ("FP64 difference vs tangent, dL/dv", f_vel),
                    ("adjoint vs FP64 difference, dL/dphi0", a_phi), ("adjoint vs FP64 difference, dL/dv", a_vel)):
        print("%-40s rel err median %.2e max %.2e over %d probes" % (name, np.median(e), e.max(), e.size))
    # a difference may run other substep counts (a step at a kink of max |v|)
    assert ok_p.sum() >= 3 * n_phi // 4 and ok_v.sum() >= 3 * n_vel // 4
    assert e_phi.max() < tol_tangent and e_vel.max() < tol_tangent
    assert f_phi.max() < tol_diff and f_vel.max() < tol_diff
    assert a_phi.max() < tol_diff and a_vel.max() < tol_diff
    return tape


@pytest.mark.gpu
@pytest.mark.parametrize("cfl", [0.0, 0.3])
def test_adjoint_matches_fp64_reference_gradient(cfl):
    from openvdb_gb300 import PARITY
    check(small_problem(cfl), PARITY, cfl, n_phi=32, n_vel=32, seed=1234, tol_tangent=1e-4, tol_diff=5e-3)


@pytest.mark.gpu
def test_adjoint_config4_gradients():
    """dL/dv and dL/dphi_0 of the 128^3 configuration on 64 seeded probe
    directions: within 1e-4 of the FP64 reference gradient, and against
    central differences with h = 1e-3 (their own truncation error, up to a
    few 1e-4 along phi_0 directions where the WENO5 weights bend, is what the
    looser bound covers)."""
    from openvdb_gb300 import PARITY
    check(config4_problem(), PARITY, 0.0, n_phi=32, n_vel=32, seed=77, tol_tangent=1e-4, tol_diff=5e-3)


@pytest.mark.gpu
def test_adjoint_cost_128():
    """Forward + adjoint against the plain forward pass on the 128^3
    configuration (FAST arithmetic, wall time of the whole calls)."""
    import torch
    from openvdb_gb300 import FAST
    from openvdb_gb300.adjoint import AdvectionTape
    pb = config4_problem()
    tape = AdvectionTape(pb.template, pb.vel, mode=FAST)
    phi0 = pb.template.active_values().copy()
    tape.forward(phi0, pb.times, record=False)  # warm-up
    torch.cuda.synchronize()
    t_plain = t_rec = t_adj = float("inf")
    for _ in range(3):
        t0 = time.perf_counter()
        tape.forward(phi0, pb.times, record=False)
        t_plain = min(t_plain, time.perf_counter() - t0)
    for _ in range(3):
        t0 = time.perf_counter()
        phiT, gT = tape.forward(phi0, pb.times, record=True)
        t_rec = min(t_rec, time.perf_counter() - t0)
        r = phiT.astype(np.float64) - pb.target_fn(gT.active_coords())
        t0 = time.perf_counter()
        g_phi, g_vel = tape.backward((2.0 * r).astype(np.float32))
        t_adj = min(t_adj, time.perf_counter() - t0)
    print("adjoint 128^3: %d substeps, %d -> %d active voxels, L = %.6g" % (sum(tape.substeps), phi0.size,
                                                                            phiT.size, float((r * r).sum())))
    print("wall time: forward %.3f s, recorded forward %.3f s, adjoint %.3f s, (fwd+adj)/fwd = %.2f"
          % (t_plain, t_rec, t_adj, (t_rec + t_adj) / t_plain))
    assert (t_rec + t_adj) / t_plain < 3.5
    assert np.isfinite(g_phi).all() and np.isfinite(g_vel).all() and np.abs(g_vel).max() > 0


@pytest.mark.gpu
def test_checkpointed_matches_single_tape():
    """Segments of 2 intervals with recompute give the gradients of one tape
    over the whole horizon, dL/dv accumulated on the device.  Every
    accumulation runs in a fixed order, so the two agree bit for bit."""
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


@pytest.mark.gpu
def test_checkpointed_descent_uses_the_new_velocity():
    """After set_velocity the checkpointed forward is the forward of the new
    velocity (its shared tape follows the field), and a normalised descent
    step along -dL/dv lowers the loss."""
    from openvdb_gb300 import FAST, fixtures
    from openvdb_gb300.adjoint import AdvectionTape, CheckpointedAdvection
    center = (16.0, 16.0, 16.0)
    template = fixtures.sphere(9.0, center)
    vel = smoothed_noise(32, 3.0, 0.8, seed=5)
    times = [0.0, 0.5, 1.0, 1.5, 2.0]
    phi0 = template.active_values().copy()

    def loss(phi, g):
        d = phi.astype(np.float64) - _sdf_sphere(g.active_coords(), 10.0, center)
        return float((d * d).sum()), (2.0 * d).astype(np.float32)

    ck = CheckpointedAdvection(template, vel, every=2, mode=FAST, cfl=0.5)
    L0, lam = loss(*ck.forward(phi0, times))
    _, dvel, _ = ck.backward(lam)
    g = dvel.cpu().numpy()
    vel2 = (vel - (0.05 / np.abs(g).max()) * g).astype(np.float32)
    ck.set_velocity(vel2)
    phi2, g2 = ck.forward(phi0, times)
    ref_phi, _ = AdvectionTape(template, vel2, mode=FAST, cfl=0.5).forward(phi0, times, record=False)
    assert np.array_equal(phi2, ref_phi)
    L1, _ = loss(phi2, g2)
    assert L1 < L0, (L0, L1)


@pytest.mark.gpu
def test_adjoint_is_deterministic():
    """Two backward sweeps of one tape give the same bits."""
    from openvdb_gb300 import FAST
    pb = small_problem(0.0)
    from openvdb_gb300.adjoint import AdvectionTape
    tape = AdvectionTape(pb.template, pb.vel, mode=FAST)
    phiT, gT = tape.forward(pb.template.active_values().copy(), pb.times)
    lam = (2.0 * (phiT.astype(np.float64) - pb.target_fn(gT.active_coords()))).astype(np.float32)
    a = tape.backward(lam)
    b = tape.backward(lam)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.gpu
def test_autograd_function_device_resident():
    """torch.autograd.Function over DeviceTape: phi0 and the velocity grid
    are CUDA tensors, the loss is formed in torch, and loss.backward() fills
    both gradients on the device.  They equal the host tape's bit for bit
    (same kernels, fixed summation order)."""
    import torch
    from openvdb_gb300 import FAST
    from openvdb_gb300.adjoint import AdvectionTape, DeviceTape, make_autograd_function
    pb = small_problem(0.0)
    phi0_h = pb.template.active_values().copy()
    tape_h = AdvectionTape(pb.template, pb.vel, mode=FAST)
    phiT_h, gT = tape_h.forward(phi0_h, pb.times)
    target = pb.target_fn(gT.active_coords()).astype(np.float32)
    g_phi_h, g_vel_h = tape_h.backward((2.0 * (phiT_h - target)).astype(np.float32))

    dev = torch.device("cuda", 0)
    phi0 = torch.tensor(phi0_h, device=dev, requires_grad=True)
    vel = torch.tensor(pb.vel, device=dev, requires_grad=True)
    tape = DeviceTape(pb.template, pb.vel.shape, mode=FAST)
    F = make_autograd_function()
    phiT = F.apply(phi0, vel, tape, pb.times)
    assert phiT.is_cuda and sum(tape.substeps) == sum(tape_h.substeps)
    assert np.array_equal(phiT.detach().cpu().numpy(), phiT_h)
    loss = ((phiT - torch.tensor(target, device=dev)) ** 2).sum()
    loss.backward()
    assert phi0.grad.is_cuda and vel.grad.is_cuda
    assert np.array_equal(phi0.grad.cpu().numpy(), g_phi_h)
    assert np.array_equal(vel.grad.cpu().numpy(), g_vel_h)
