"""Level-set fixtures built by the native host code (gbls_host_*).

sphere() equals tools::createLevelSetSphere (tools/LevelSetSphere.h:219-230)
voxel for voxel; union_of_spheres() rasterises a union of spheres directly.
The workload generators below produce the seeded inputs of the benchmark
configurations.
"""
import ctypes as C

import numpy as np

from . import _abi
from ._lib import check, lib
from .grid import HostGrid


def _from_native(handle):
    d = _abi.GridDesc()
    L = lib()
    try:
        check(L.gbls_host_grid_view(handle, C.byref(d)), host=True)

        def arr(ptr, n, shape, dtype):
            if n == 0:
                return np.zeros((0,) + shape, dtype)
            ct = np.ctypeslib.as_array(ptr, shape=(n * int(np.prod(shape)),))
            return np.array(ct, dtype=dtype).reshape((n,) + shape)

        g = HostGrid(
            voxel_size=d.voxel_size, background=d.background, map_type=d.map_type,
            translation=tuple(d.translation),
            leaf_origins=arr(d.leaf_origins, d.leaf_count, (3,), np.int32),
            leaf_masks=arr(d.leaf_masks, d.leaf_count, (8,), np.uint64),
            leaf_values=arr(d.leaf_values, d.leaf_count, (512,), np.float32),
            lower_origins=arr(d.lower_origins, d.lower_count, (3,), np.int32),
            lower_tiles=arr(d.lower_tiles, d.lower_count, (4096,), np.float32),
            upper_origins=arr(d.upper_origins, d.upper_count, (3,), np.int32),
            upper_tiles=arr(d.upper_tiles, d.upper_count, (32768,), np.float32),
            root_tile_origins=arr(d.root_tile_origins, d.root_tile_count, (3,), np.int32),
            root_tile_values=arr(d.root_tile_values, d.root_tile_count, (), np.float32),
        )
    finally:
        L.gbls_host_grid_free(handle)
    return g


def sphere(radius, center=(0.0, 0.0, 0.0), voxel_size=1.0, half_width=3.0):
    """createLevelSetSphere<FloatGrid>(radius, center, voxel_size, half_width)."""
    h = C.c_void_p()
    c = (C.c_float * 3)(*center)
    check(lib().gbls_host_sphere(radius, c, voxel_size, half_width, C.byref(h)), host=True)
    return _from_native(h)


def torus(major_radius, minor_radius, center=(0.0, 0.0, 0.0), voxel_size=1.0, half_width=3.0):
    """Narrow-band torus around the y axis (batch fixtures)."""
    h = C.c_void_p()
    c = (C.c_float * 3)(*center)
    check(lib().gbls_host_torus(major_radius, minor_radius, c, voxel_size, half_width, C.byref(h)),
          host=True)
    return _from_native(h)


def union_of_spheres(centers, radii, voxel_size=1.0, half_width=3.0):
    c = np.ascontiguousarray(centers, np.float32).reshape(-1)
    r = np.ascontiguousarray(radii, np.float32).reshape(-1)
    h = C.c_void_p()
    check(lib().gbls_host_union_of_spheres(len(r), c.ctypes.data_as(C.POINTER(C.c_float)),
                                           r.ctypes.data_as(C.POINTER(C.c_float)), voxel_size,
                                           half_width, C.byref(h)), host=True)
    return _from_native(h)


def sixty_four_spheres(seed=2024, n=64, domain=1024.0, rmin=20.0, rmax=80.0):
    """Seeded centres U[0,domain]^3 and radii U[rmin,rmax] (cx, cy, cz, r per sphere)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    vals = rng.random((n, 4))
    centers = (vals[:, :3] * domain).astype(np.float32)
    radii = (rmin + vals[:, 3] * (rmax - rmin)).astype(np.float32)
    return centers, radii


def batch_instances(n=512, seed=7, rmin=8.0, rmax=128.0):
    """Seeded batch: 50/50 spheres and tori, radius log-uniform in [rmin, rmax],
    torus tube ratio U[0.2, 0.4]; each with a constant-plus-rotation velocity
    (constant U[-1,1]^3, angular velocity U[-0.01,0.01]^3 rad per time unit
    about the shape's centre).  Returns (list of shape specs, list of Fields)."""
    from .fields import Field
    rng = np.random.Generator(np.random.PCG64(seed))
    specs, fields = [], []
    for i in range(n):
        kind = "sphere" if rng.random() < 0.5 else "torus"
        R = float(np.float32(np.exp(np.log(rmin) + rng.random() * (np.log(rmax) - np.log(rmin)))))
        ratio = float(np.float32(0.2 + 0.2 * rng.random()))
        center = tuple(float(np.float32(x)) for x in rng.random(3) * 16.0)
        c = tuple(float(np.float32(x)) for x in rng.uniform(-1.0, 1.0, 3))
        om = tuple(float(np.float32(x)) for x in rng.uniform(-0.01, 0.01, 3))
        specs.append((kind, R, ratio, center))
        fields.append(Field.rotation(c, om, center))
    return specs, fields


def build_instance(spec):
    kind, R, ratio, center = spec
    if kind == "sphere":
        return sphere(R, center)
    return torus(R, max(1.6, R * ratio), center)


def smoothed_noise(n, sigma, amplitude, seed):
    """Seeded Gaussian-smoothed noise velocity on an n^3 grid, shape
    (n, n, n, 3), float32: standard normal components convolved per axis
    with a periodic Gaussian of width sigma voxels (truncated at 3 sigma),
    scaled so that the largest component magnitude is `amplitude`."""
    rng = np.random.Generator(np.random.PCG64(seed))
    v = rng.standard_normal((n, n, n, 3))
    r = int(3 * sigma)
    x = np.arange(-r, r + 1)
    k = np.exp(-0.5 * (x / sigma) ** 2)
    k /= k.sum()
    for ax in range(3):
        v = np.apply_along_axis(lambda a: np.convolve(np.pad(a, r, mode="wrap"), k, "valid"), ax, v)
    v *= amplitude / np.abs(v).max()
    return v.astype(np.float32)


def adjoint_128():
    """The 128^3 adjoint configuration: phi_0 a radius-40 sphere centred in
    the domain, a seeded 5%-perturbed radius-44 sphere as the target
    (returned as a function of index coordinates), a smoothed-noise velocity
    grid (sigma 4 voxels, amplitude 1 voxel per time unit, seed 9) and 20
    unit steps."""
    center = np.array([64.0, 64.0, 64.0])
    rng = np.random.Generator(np.random.PCG64(44))
    axes = rng.standard_normal((4, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    amps = rng.uniform(-1.0, 1.0, 4)
    amps /= np.abs(amps).sum()

    def target(coords):
        c = coords.astype(np.float64) - center
        r = np.linalg.norm(c, axis=1)
        nrm = c / np.maximum(r, 1e-9)[:, None]
        return r - 44.0 * (1.0 + 0.05 * (nrm @ axes.T) @ amps)

    template = sphere(40.0, tuple(center))
    vel = smoothed_noise(128, 4.0, 1.0, seed=9)
    return template, vel, target, [float(t) for t in range(21)]
