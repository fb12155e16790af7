"""Parity cases shared by the golden-vector generator and the GPU tests.

Each case builds an input level set, then applies a list of operations:
  ("advect", t0, t1)            LevelSetAdvection::advect with the case schemes
  ("track",) ("normalize",) ("prune",) ("dilate", n)
                                LevelSetTracker operations
  ("normalize_masked", lo, hi)  LevelSetTracker::normalize(&mask) with the mask of
                                box_mask(grid, lo, hi)
  ("state", {...})              change tracker state (norm_count, tr_temporal, trim)
A case with "cfl" > 0 advects under that imposed CFL number: the reference's
advect(tau, tau') over greedy intervals of cfl*dx/max|v| (the interval driver
of oracle/ref/ref_harness.cc), the device through gbls_advect(..., cfl).
The golden file records, after every operation, the SHA-256 digest of the
grid's canonical arrays (openvdb_gb300.grid.digest) and the substep count.
"""
import numpy as np

from openvdb_gb300 import _abi
from openvdb_gb300.fields import Field

HJ = _abi.HJWENO5_BIAS
RK1, RK2, RK3 = _abi.TVD_RK1, _abi.TVD_RK2, _abi.TVD_RK3


def box_mask(grid, lo, hi):
    """Leaf origins and active masks of the active voxels of `grid` whose index
    lies in the box [lo, hi] (inclusive), plus one full leaf at (800, 800, 800)
    where the test level sets have none."""
    origins, masks = [], []
    yz = np.arange(64)
    for o, m in zip(grid.leaf_origins, grid.leaf_masks):
        gy, gz = o[1] + (yz >> 3), o[2] + (yz & 7)
        inside_yz = (gy >= lo[1]) & (gy <= hi[1]) & (gz >= lo[2]) & (gz <= hi[2])
        pattern = np.uint64(0)
        for b in np.nonzero(inside_yz)[0]:
            pattern |= np.uint64(1) << np.uint64(b)
        words = np.zeros(8, np.uint64)
        for x in range(8):
            if lo[0] <= o[0] + x <= hi[0]:
                words[x] = m[x] & pattern
        if words.any():
            origins.append(o)
            masks.append(words)
    origins.append(np.array([800, 800, 800], np.int32))
    masks.append(np.full(8, np.iinfo(np.uint64).max, np.uint64))
    return np.array(origins, np.int32), np.array(masks, np.uint64)


def smoothed_noise(n, sigma, amplitude, seed):
    """Seeded Gaussian-smoothed noise velocity on an n^3 grid, shape (n,n,n,3)."""
    from openvdb_gb300.fixtures import smoothed_noise as f
    return f(n, sigma, amplitude, seed)


def union8():
    rng = np.random.Generator(np.random.PCG64(7))
    c = (16 + rng.random((8, 3)) * 96).astype(np.float32)
    r = (8 + rng.random(8) * 12).astype(np.float32)
    return c, r


CASES = {
    # configuration 1 at the reference CFL: sphere r=64, constant velocity,
    # HJWENO5 + TVD_RK3, tracker HJWENO5 + TVD_RK1 with one renormalisation
    "cfg1_sphere64": dict(
        fixture=("sphere", 64.0, (0.0, 0.0, 0.0), 1.0, 3.0),
        field=("constant", (1.0, 0.5, 0.25)),
        schemes=(HJ, RK3, HJ, RK1, 1),
        ops=[("advect", float(t), float(t + 1)) for t in range(10)],
    ),
    # configuration 1 as specified: CFL 0.5 imposed by the interval driver
    "cfg1_sphere64_cfl05": dict(
        fixture=("sphere", 64.0, (0.0, 0.0, 0.0), 1.0, 3.0),
        field=("constant", (1.0, 0.5, 0.25)),
        schemes=(HJ, RK3, HJ, RK1, 1),
        cfl=0.5,
        ops=[("advect", float(t), float(t + 1)) for t in range(10)],
    ),
    "union8_deformation_cfl05": dict(
        fixture=("union8",),
        field=("deformation", 128.0, 10.0, 1.0),
        schemes=(HJ, RK3, HJ, RK1, 1),
        cfl=0.5,
        ops=[("advect", float(t), float(t + 1)) for t in range(3)],
    ),
    # the benchmark workload: 64 seeded spheres (csgUnion of createLevelSetSphere
    # in the reference), LeVeque deformation on 1024^3 x cos(pi t/100), CFL 0.5,
    # its first 25 unit steps (the benchmark's warm-up and timed window)
    "bench64_cfl05": dict(
        fixture=("sixty_four", 2024),
        field=("deformation", 1024.0, 100.0, 1.0),
        schemes=(HJ, RK3, HJ, RK1, 1),
        cfl=0.5,
        large=True,
        ops=[("advect", float(t), float(t + 1)) for t in range(25)],
    ),
    # the reference's default FieldT, tools::EnrightField<float>, with the
    # default schemes (HJWENO5 + TVD_RK2, tracker TVD_RK1, normCount 3): the
    # classic Enright sphere in the unit box, sampled on the host
    "enright_sphere_default_field": dict(
        port=False,  # the oracle's C++ restatement takes device-style fields only
        fixture=("sphere", 0.15, (0.35, 0.35, 0.35), 0.01, 3.0),
        field=("enright", 0.01),
        schemes=(HJ, RK2, HJ, RK1, 3),
        ops=[("advect", 0.0, 0.02), ("advect", 0.02, 0.05)],
    ),
    "sphere20_deformation": dict(
        fixture=("sphere", 20.0, (32.0, 30.0, 34.0), 1.0, 3.0),
        field=("deformation", 64.0, 8.0, 1.0),
        schemes=(HJ, RK3, HJ, RK1, 1),
        ops=[("advect", float(t), float(t + 1)) for t in range(4)],
    ),
    "sphere16_rotation_backward": dict(
        fixture=("sphere", 16.0, (5.5, -3.25, 2.0), 1.0, 3.0),
        field=("rotation", (0.3, -0.2, 0.1), (0.02, -0.03, 0.05), (5.0, -3.0, 2.0)),
        schemes=(HJ, RK3, HJ, RK1, 1),
        ops=[("advect", 3.0, 2.0), ("advect", 2.0, 1.0)],
    ),
    "sphere12_rk1_default_tracker": dict(
        fixture=("sphere", 12.0, (0.0, 1.0, 2.0), 1.0, 3.0),
        field=("constant", (-0.7, 0.4, 1.1)),
        schemes=(HJ, RK1, HJ, RK1, 3),
        ops=[("advect", 0.0, 1.0), ("advect", 1.0, 2.5)],
    ),
    "sphere12_rk2": dict(
        fixture=("sphere", 12.0, (0.0, 1.0, 2.0), 1.0, 3.0),
        field=("constant", (-0.7, 0.4, 1.1)),
        schemes=(HJ, RK2, HJ, RK1, 3),
        ops=[("advect", 0.0, 1.0), ("advect", 1.0, 2.5)],
    ),
    "sphere24_tracker_rk3_rk2": dict(
        fixture=("sphere", 24.0, (-10.0, 4.0, 9.0), 1.0, 3.0),
        field=("constant", (0.6, -0.9, 0.2)),
        schemes=(HJ, RK3, HJ, RK3, 2),
        ops=[("advect", 0.0, 1.0), ("state", {"tr_temporal": RK2}), ("advect", 1.0, 2.0)],
    ),
    "tracker_ops": dict(
        fixture=("sphere", 20.0, (1.0, 2.0, 3.0), 1.0, 3.0),
        field=("constant", (0.0, 0.0, 0.0)),
        schemes=(HJ, RK1, HJ, RK1, 3),
        ops=[("normalize",), ("dilate", 2), ("normalize",), ("prune",), ("track",),
             ("state", {"trim": _abi.TRIM_INTERIOR}), ("dilate", 1), ("track",),
             ("state", {"trim": _abi.TRIM_EXTERIOR}), ("track",),
             ("state", {"trim": _abi.TRIM_NONE}), ("track",),
             ("state", {"trim": _abi.TRIM_ALL, "norm_count": 0}), ("track",)],
    ),
    # normalize(mask): the renormalisation restricted to the active voxels in
    # an index box (the mask also holds a leaf the level set does not have)
    "tracker_masked_normalize": dict(
        port=False,  # the oracle's C++ restatement has no masked normalize
        fixture=("sphere", 18.0, (0.5, 1.0, -2.0), 1.0, 3.0),
        field=("constant", (0.0, 0.0, 0.0)),
        schemes=(HJ, RK1, HJ, RK1, 3),
        ops=[("normalize_masked", (-20, -20, -20), (4, 30, 30)), ("state", {"tr_temporal": RK2, "norm_count": 2}),
             ("normalize_masked", (-6, -30, -5), (30, 9, 30)), ("track",)],
    ),
    "union8_deformation": dict(
        fixture=("union8",),
        field=("deformation", 128.0, 10.0, 1.0),
        schemes=(HJ, RK3, HJ, RK1, 1),
        ops=[("advect", float(t), float(t + 1)) for t in range(3)],
    ),
    "sphere12_dense_noise": dict(
        fixture=("sphere", 12.0, (16.0, 16.0, 16.0), 1.0, 3.0),
        field=("dense", 32, 4.0, 1.0, 11),
        schemes=(HJ, RK3, HJ, RK1, 1),
        ops=[("advect", float(t), float(t + 1)) for t in range(3)],
    ),
    # non-aligned DiscreteField: the velocity grid has its own voxel size and
    # translation, sampled trilinearly at every voxel's world position
    "sphere12_dense_xform": dict(
        fixture=("sphere", 12.0, (16.0, 16.0, 16.0), 1.0, 3.0),
        field=("dense_xform", 24, 3.0, 1.0, 13, 1.5, (0.3, -0.2, 0.1), (0, 0, 0)),
        schemes=(HJ, RK3, HJ, RK1, 1),
        ops=[("advect", float(t), float(t + 1)) for t in range(3)],
    ),
    "half_voxel_dense_xform": dict(
        fixture=("sphere", 6.0, (0.25, -0.5, 1.0), 0.5, 3.0),
        field=("dense_xform", 32, 4.0, 0.5, 17, 1.0, (0.0, 0.0, 0.0), (-10, -10, -10)),
        schemes=(HJ, RK2, HJ, RK1, 3),
        ops=[("advect", 0.0, 1.0), ("advect", 1.0, 2.0)],
    ),
    # the other biased schemes for advection and tracker (the oracle's C++
    # restatement implements HJWENO5 only: port=False)
    "sphere12_first_bias": dict(
        fixture=("sphere", 12.0, (0.0, 1.0, 2.0), 1.0, 3.0),
        field=("constant", (-0.7, 0.4, 1.1)),
        schemes=(0, RK1, 0, RK1, 3),
        ops=[("advect", 0.0, 1.0), ("advect", 1.0, 2.0)],
        port=False,
    ),
    "sphere12_second_bias": dict(
        fixture=("sphere", 12.0, (0.0, 1.0, 2.0), 1.0, 3.0),
        field=("rotation", (0.3, -0.2, 0.1), (0.02, -0.03, 0.05), (0.0, 1.0, 2.0)),
        schemes=(1, RK2, 1, RK1, 2),
        ops=[("advect", 0.0, 1.0), ("advect", 1.0, 2.0)],
        port=False,
    ),
    "sphere12_third_bias": dict(
        fixture=("sphere", 12.0, (0.0, 1.0, 2.0), 1.0, 3.0),
        field=("constant", (0.6, -0.9, 0.2)),
        schemes=(2, RK3, 2, RK2, 1),
        ops=[("advect", 0.0, 1.0), ("advect", 1.0, 2.0)],
        port=False,
    ),
    "sphere12_weno5_bias": dict(
        fixture=("sphere", 12.0, (0.0, 1.0, 2.0), 1.0, 3.0),
        field=("dense", 32, 4.0, 1.0, 11),
        schemes=(3, RK3, 3, RK3, 1),
        ops=[("advect", 0.0, 1.0), ("advect", 1.0, 2.0)],
        port=False,
    ),
    "sphere_half_voxel": dict(
        fixture=("sphere", 6.0, (0.25, -0.5, 1.0), 0.5, 3.0),
        field=("constant", (0.5, 0.25, -0.3)),
        schemes=(HJ, RK3, HJ, RK1, 1),
        ops=[("advect", 0.0, 1.0), ("advect", 1.0, 2.0)],
    ),
}


def make_field(spec):
    kind = spec[0]
    if kind == "constant":
        return Field.constant_field(spec[1])
    if kind == "deformation":
        return Field.deformation(domain=spec[1], period=spec[2], scale=spec[3])
    if kind == "rotation":
        return Field.rotation(spec[1], spec[2], spec[3])
    if kind == "dense":
        n, sigma, amp, seed = spec[1:]
        return Field.dense(smoothed_noise(n, sigma, amp, seed), origin=(0, 0, 0),
                           background=(0.0, 0.0, 0.0))
    if kind == "enright":
        # the grid's map holds the float voxel size the sphere was made with
        # (createLinearTransform(double(voxelSize))), and the field is
        # evaluated at index * that double
        return Field.enright(voxel_size=float(np.float32(spec[1])))
    if kind == "dense_xform":
        n, sigma, amp, seed, voxel, translation, origin = spec[1:]
        return Field.dense_xform(smoothed_noise(n, sigma, amp, seed), voxel, translation, origin=origin,
                                 background=(0.0, 0.0, 0.0))
    raise ValueError(kind)


def make_fixture(spec):
    from openvdb_gb300 import fixtures
    if spec[0] == "sphere":
        return fixtures.sphere(spec[1], spec[2], spec[3], spec[4])
    if spec[0] == "union8":
        c, r = union8()
        return fixtures.union_of_spheres(c, r)
    if spec[0] == "sixty_four":
        c, r = fixtures.sixty_four_spheres(seed=spec[1])
        return fixtures.union_of_spheres(c, r, 1.0, 3.0)
    if spec[0] == "torus":
        return fixtures.torus(spec[1], spec[2], spec[3])
    raise ValueError(spec[0])


# LevelSetMorphing (tools/LevelSetMorph.h): source fixture morphed towards a
# target fixture, optionally with an alpha mask (a level set), through the
# listed advect(t0, t1) calls.  Fixture specs as for make_fixture, plus
# ("torus", R, r, center).
MORPH_CASES = {
    "morph_sphere_to_sphere_rk2": dict(
        source=("sphere", 12.0, (0.0, 0.0, 0.0), 1.0, 3.0),
        target=("sphere", 15.0, (2.0, 1.0, -1.0), 1.0, 3.0),
        schemes=(HJ, RK2, HJ, RK1, 3),
        ops=[("morph", 0.0, 1.0), ("morph", 1.0, 2.0), ("morph", 2.0, 4.0)],
    ),
    "morph_sphere_to_torus_rk3": dict(
        source=("sphere", 16.0, (0.0, 0.0, 0.0), 1.0, 3.0),
        target=("torus", 14.0, 5.0, (0.5, -0.5, 0.0)),
        schemes=(HJ, RK3, HJ, RK1, 1),
        ops=[("morph", 0.0, 1.0), ("morph", 1.0, 2.0), ("morph", 2.0, 3.0)],
    ),
    "morph_first_bias_rk3": dict(
        source=("sphere", 11.0, (0.0, 0.0, 0.0), 1.0, 3.0),
        target=("sphere", 13.0, (1.0, -1.0, 0.5), 1.0, 3.0),
        schemes=(0, RK3, 0, RK1, 2),
        ops=[("morph", 0.0, 1.0), ("morph", 1.0, 2.0)],
    ),
    "morph_masked_rk1": dict(
        source=("sphere", 14.0, (0.0, 0.0, 0.0), 1.0, 3.0),
        target=("sphere", 10.0, (3.0, 0.0, 0.0), 1.0, 3.0),
        mask=("sphere", 9.0, (8.0, 4.0, 0.0), 1.0, 3.0),
        schemes=(HJ, RK1, HJ, RK1, 2),
        ops=[("morph", 0.0, 1.0, (-2.0, 2.0), False), ("morph", 1.0, 2.0, (-1.0, 3.0), True)],
    ),
}


# LevelSetFilter (tools/LevelSetFilter.h): filters applied in sequence to one
# fixture; each op is (filter, width, value) with filter 0 laplacian, 1 mean,
# 2 gaussian, 3 offset, 4 meanCurvature, 5 fillet, 6 median, or
# (filter, width, value, (mask min, mask max), invert) with the case's alpha
# mask level set; tracker schemes as (spatial, temporal, normCount).
FILTER_CASES = {
    "filter_sphere_ops": dict(
        fixture=("sphere", 14.0, (0.5, -1.0, 2.0), 1.0, 3.0),
        tracker=(HJ, RK1, 3),
        ops=[(0, 1, 0.0), (1, 1, 0.0), (3, 1, 1.3), (2, 2, 0.0), (3, 1, -0.7), (1, 3, 0.0)],
    ),
    "filter_torus_rk2_tracker": dict(
        fixture=("torus", 14.0, 4.0, (0.0, 0.0, 0.0)),
        tracker=(HJ, RK2, 1),
        ops=[(0, 1, 0.0), (0, 1, 0.0), (2, 1, 0.0), (3, 1, 0.4)],
    ),
    # 4 meanCurvature, 5 fillet, 6 median(width): stencils with edge and
    # corner neighbours
    "filter_curvature_median": dict(
        fixture=("sphere", 12.0, (1.5, -2.0, 0.5), 1.0, 3.0),
        tracker=(HJ, RK1, 3),
        ops=[(4, 1, 0.0), (6, 1, 0.0), (4, 1, 0.0), (5, 1, 0.0), (6, 2, 0.0), (6, 3, 0.0)],
    ),
    "filter_torus_fillet": dict(
        fixture=("torus", 14.0, 4.5, (0.5, 0.0, -0.5)),
        tracker=(HJ, RK1, 1),
        ops=[(5, 1, 0.0), (5, 1, 0.0), (4, 1, 0.0), (6, 1, 0.0), (5, 1, 0.0)],
    ),
    # every filter with an alpha mask (a sphere level set overlapping part of
    # the fixture: voxels with alpha 0, fractional and 1), both polarities
    "filter_masked": dict(
        fixture=("sphere", 14.0, (0.5, -1.0, 2.0), 1.0, 3.0),
        mask=("sphere", 9.0, (7.0, 3.0, 1.0), 1.0, 3.0),
        tracker=(HJ, RK1, 3),
        ops=[(0, 1, 0.0, (-2.0, 2.0), False), (1, 1, 0.0, (-1.0, 3.0), True), (3, 1, 1.1, (-2.0, 2.0), False),
             (2, 1, 0.0, (-2.0, 2.0), True), (4, 1, 0.0, (-2.5, 1.5), False), (5, 1, 0.0, (-3.0, 1.0), False),
             (6, 1, 0.0, (-2.0, 2.0), True), (3, 1, -0.6, (-1.0, 1.0), True), (5, 1, 0.0, (-2.0, 2.0), True)],
    ),
}


# Batched advection: each instance must equal its own reference advect call.
BATCH = dict(n=6, seed=11, rmin=6.0, rmax=20.0, schemes=(HJ, RK3, HJ, RK1, 1),
             ops=[(0.0, 1.0), (1.0, 2.0)])


# The batched configuration's per-instance imposed CFL number.
BATCH_CFL = dict(BATCH, cfl=0.5)


def make_batch():
    from openvdb_gb300 import fixtures
    specs, fields = fixtures.batch_instances(BATCH["n"], BATCH["seed"], BATCH["rmin"], BATCH["rmax"])
    return [fixtures.build_instance(s) for s in specs], fields


# VolumeAdvection (tools/VolumeAdvect.h): a FloatGrid volume advected by
# tools::VolumeAdvection<Vec3fGrid>::advect<FloatGrid, BoxSampler> through the
# listed ("volume", integrator, limiter, substeps, time_step) calls.
# integrator: 0 SEMI, 1 MID, 2 RK3, 3 RK4, 4 MAC, 5 BFECC; limiter: 0 none,
# 1 CLAMP, 2 REVERT.  Volumes: ("fog_shell", radius, center, voxel_size) is
# the level-set sphere's narrow band turned into a density 0.5 - phi/6 (zero
# outside the band, zero background and tiles); ("fog_ball", radius, center,
# voxel_size) a sphere whose band reaches the centre, density -phi/radius
# clamped to [0, 1].
VOLUME_CASES = {
    "vol_shell_noise_all_schemes": dict(
        volume=("fog_shell", 12.0, (16.0, 16.0, 16.0), 1.0),
        field=("dense", 32, 3.0, 1.5, 3),
        ops=[("volume", 0, 1, 1, 1.0), ("volume", 1, 1, 1, 1.0), ("volume", 2, 1, 1, 1.0),
             ("volume", 3, 1, 1, 1.0), ("volume", 4, 0, 1, 1.0), ("volume", 4, 1, 1, 1.0),
             ("volume", 4, 2, 1, 1.0), ("volume", 5, 0, 1, 1.0), ("volume", 5, 1, 1, 1.0),
             ("volume", 5, 2, 1, 1.0)],
    ),
    "vol_ball_xform_substeps": dict(
        volume=("fog_ball", 8.0, (2.0, -1.0, 0.5), 1.0),
        field=("dense_xform", 24, 2.0, 1.2, 11, 1.5, (0.25, -0.5, 0.75), (-10, -10, -10)),
        ops=[("volume", 4, 1, 2, 1.5), ("volume", 2, 1, 3, -1.0), ("volume", 5, 2, 2, 0.75)],
    ),
    "vol_half_voxel_constant": dict(
        volume=("fog_ball", 4.0, (0.3, 0.2, -0.1), 0.5),
        field=("constant", (1.25, -0.6, 0.35)),
        ops=[("volume", 3, 1, 1, 2.0), ("volume", 0, 1, 3, 1.0), ("volume", 5, 1, 1, 0.5)],
    ),
}


def make_volume(spec):
    """A FloatGrid volume from the level-set sphere fixture (see VOLUME_CASES)."""
    from openvdb_gb300 import fixtures
    kind, radius, center, dx = spec
    if kind == "fog_shell":
        g = fixtures.sphere(radius, center, dx, 3.0)
        m = g.active_mask_bool()
        g.leaf_values = np.where(m, np.float32(0.5) - g.leaf_values / np.float32(6.0),
                                 np.float32(0.0)).astype(np.float32)
    elif kind == "fog_ball":
        g = fixtures.sphere(radius, center, dx, radius / dx + 2.0)
        m = g.active_mask_bool()
        d = np.clip(-g.leaf_values / np.float32(radius), np.float32(0.0), np.float32(1.0)).astype(np.float32)
        g.leaf_values = np.where(m, d, np.float32(0.0)).astype(np.float32)
    else:
        raise ValueError(kind)
    g.background = 0.0
    g.lower_tiles[:] = 0.0
    g.upper_tiles[:] = 0.0
    g.root_tile_values[:] = 0.0
    return g
