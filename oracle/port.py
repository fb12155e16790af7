"""ctypes wrapper of the oracle's C++ restatement (oracle/_build/liboracle_port.so).

Test infrastructure: the parity oracle on hosts without the compiled
reference, and the timed CPU baseline / reference arm of bench.py.  Pinned
against the compiled reference through tests/golden/parity_cases.json
(tests/test_oracle_port.py).

The module imports nothing from the product package: the reference arm of
bench.py builds its 64-sphere input with the oracle's own rasteriser
(oport_create_spheres) and passes its own mirror of gbls_field_desc, so its
process loads no product library.  Grids given by the tests (HostGrid) and
their fields are passed by address.
"""
import ctypes as C
import os
import time

import numpy as np

# gbls.h constants the arm uses (values of the reference enums)
HJWENO5_BIAS = 4
TVD_RK1, TVD_RK2, TVD_RK3 = 0, 1, 2
TRIM_ALL = 3
FIELD_DEFORMATION = 2


class GridCounts(C.Structure):
    """gbls_grid_counts (include/gbls.h)."""
    _fields_ = [("leaf_count", C.c_int64), ("lower_count", C.c_int64), ("upper_count", C.c_int64),
                ("root_tile_count", C.c_int64), ("active_voxel_count", C.c_int64), ("background", C.c_float)]


class FieldDesc(C.Structure):
    """gbls_field_desc (include/gbls.h)."""
    _fields_ = [("kind", C.c_int32), ("constant", C.c_float * 3), ("dense_origin", C.c_int32 * 3),
                ("dense_dims", C.c_int32 * 3), ("dense_values", C.POINTER(C.c_float)),
                ("dense_background", C.c_float * 3), ("domain", C.c_float), ("period", C.c_float),
                ("scale", C.c_float), ("omega", C.c_float * 3), ("center", C.c_float * 3),
                ("dense_map_type", C.c_int32), ("dense_voxel_size", C.c_double),
                ("dense_translation", C.c_double * 3), ("host_sample", C.c_void_p), ("host_user", C.c_void_p)]


def deformation(domain=1024.0, period=100.0, scale=1.0):
    """The LeVeque deformation field descriptor (gbls_fields.h)."""
    f = FieldDesc()
    f.kind = FIELD_DEFORMATION
    f.domain, f.period, f.scale = domain, period, scale
    return f


def sixty_four_spheres(seed=2024, n=64, domain=1024.0, rmin=20.0, rmax=80.0):
    """Seeded centres U[0,domain]^3 and radii U[rmin,rmax] (cx, cy, cz, r per
    sphere, numpy PCG64): the benchmark's sphere set."""
    rng = np.random.Generator(np.random.PCG64(seed))
    vals = rng.random((n, 4))
    return (vals[:, :3] * domain).astype(np.float32), (rmin + vals[:, 3] * (rmax - rmin)).astype(np.float32)


_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liboracle_port.so")
_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.oport_last_error.restype = C.c_char_p
        L.oport_create.argtypes = [vp, C.c_int]
        L.oport_create.restype = vp
        L.oport_create_prec.argtypes = [vp, C.c_int, C.c_int]
        L.oport_create_prec.restype = vp
        L.oport_create_spheres.argtypes = [C.c_int64, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float,
                                           C.c_float, C.c_int, C.c_int]
        L.oport_create_spheres.restype = vp
        L.oport_active_values.argtypes = [vp, C.POINTER(C.c_double)]
        L.oport_set_active_values.argtypes = [vp, C.POINTER(C.c_double)]
        L.oport_free.argtypes = [vp]
        L.oport_free.restype = None
        L.oport_set_threads.argtypes = [vp, C.c_int]
        L.oport_set_threads.restype = None
        L.oport_counts.argtypes = [vp, C.POINTER(GridCounts)]
        L.oport_weno5.argtypes = [C.c_int64, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.oport_weno5.restype = None
        L.oport_export.argtypes = [vp, vp]
        L.oport_tracker_op.argtypes = [vp] + [C.c_int] * 6 + [C.POINTER(C.c_int)]
        L.oport_advect.argtypes = [vp, vp] + [C.c_int] * 5 + \
            [C.c_float, C.c_float, C.c_float, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.oport_tangent_lanes.restype = C.c_int
        L.oport_topology.argtypes = [vp, C.c_int, vp]
        L.oport_topology_count.argtypes = [vp]
        L.oport_topology_count.restype = C.c_int64
        L.oport_set_tangents.argtypes = [vp, C.POINTER(C.c_double)]
        L.oport_active_tangents.argtypes = [vp, C.POINTER(C.c_double)]
        L.oport_set_velocity_tangent.argtypes = [vp, C.POINTER(C.c_double), C.c_int64]
        _lib = L
    return _lib


def available():
    try:
        lib()
        return True
    except OSError:
        return False


def _check(rc):
    if rc != 0:
        raise RuntimeError("oracle port error %d: %s" % (rc, lib().oport_last_error().decode()))


TANGENT = 1  # PortGrid precision: FP32 values with FP64 tangents


def tangent_lanes():
    """Directions one TANGENT run carries."""
    return int(lib().oport_tangent_lanes())


class PortGrid:
    """A level set held by the C++ restatement."""

    def __init__(self, host, threads=0, precision=32):
        """precision 32: bit-identical to the reference; 64: the same scheme
        (same constants, same operations) evaluated in FP64; 1 (TANGENT):
        the FP32 computation with an FP64 directional derivative carried
        beside every value (tangent-linear mode).  `host` is a HostGrid
        (its gbls_grid_desc is passed by address)."""
        self.updates = 0
        if host is None:
            self.h = None
            return
        d = host.desc()
        self.h = C.c_void_p(lib().oport_create_prec(C.addressof(d), int(threads), int(precision)))

    @classmethod
    def spheres(cls, centers, radii, voxel_size=1.0, half_width=3.0, threads=0, precision=32):
        """The union of narrow-band spheres rasterised by the oracle itself."""
        c = np.ascontiguousarray(centers, np.float32).reshape(-1)
        r = np.ascontiguousarray(radii, np.float32).reshape(-1)
        g = cls(None)
        g.h = C.c_void_p(lib().oport_create_spheres(r.size, c.ctypes.data_as(C.POINTER(C.c_float)),
                                                    r.ctypes.data_as(C.POINTER(C.c_float)), voxel_size,
                                                    half_width, int(threads), int(precision)))
        return g

    def active_values(self):
        out = np.zeros(self.counts().active_voxel_count, np.float64)
        _check(lib().oport_active_values(self.h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def set_active_values(self, values):
        v = np.ascontiguousarray(values, np.float64)
        assert v.size == self.counts().active_voxel_count
        _check(lib().oport_set_active_values(self.h, v.ctypes.data_as(C.POINTER(C.c_double))))

    def set_tangents(self, d):
        """TANGENT grids: the derivatives of the active values along the
        probe directions, d[lane, active] (canonical active order; fewer
        than tangent_lanes() rows leave the others at zero)."""
        n = self.counts().active_voxel_count
        v = np.zeros((tangent_lanes(), n), np.float64)
        d = np.asarray(d, np.float64).reshape(-1, n)
        v[:d.shape[0]] = d
        _check(lib().oport_set_tangents(self.h, v.ctypes.data_as(C.POINTER(C.c_double))))

    def active_tangents(self):
        """TANGENT grids: (tangent_lanes(), active) derivatives."""
        out = np.zeros((tangent_lanes(), self.counts().active_voxel_count), np.float64)
        _check(lib().oport_active_tangents(self.h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def set_velocity_tangent(self, dv):
        """TANGENT grids: the derivatives of a dense field's values along
        the probe directions, dv[lane, nx, ny, nz, 3] (None: zero)."""
        if dv is None:
            self._vel_tangent = None
            _check(lib().oport_set_velocity_tangent(self.h, None, 0))
            return
        dv = np.asarray(dv, np.float64)
        v = np.zeros((tangent_lanes(),) + dv.shape[1:], np.float64)
        v[:dv.shape[0]] = dv
        self._vel_tangent = v
        _check(lib().oport_set_velocity_tangent(self.h, v.ctypes.data_as(C.POINTER(C.c_double)), v.size))

    def record_topology(self):
        """Record the band after every trim from now on."""
        _check(lib().oport_topology(self.h, 1, None))

    def replay_topology(self, source=None):
        """Impose the band recorded by `source` (a PortGrid; None: this
        grid's own record) on every trim from now on, in order."""
        _check(lib().oport_topology(self.h, 2, source.h if source is not None else None))

    def topology_count(self):
        return int(lib().oport_topology_count(self.h))

    def __del__(self):
        if getattr(self, "h", None) and self.h.value and _lib is not None:
            _lib.oport_free(self.h)

    def set_threads(self, n):
        lib().oport_set_threads(self.h, int(n))

    def counts(self):
        c = GridCounts()
        _check(lib().oport_counts(self.h, C.byref(c)))
        return c

    def to_host(self):
        """The grid as a HostGrid (tests; imports the product's host types)."""
        from openvdb_gb300.grid import HostGrid
        c = self.counts()
        g = HostGrid.allocate(c)
        d = g.desc()
        _check(lib().oport_export(self.h, C.addressof(d)))
        g.copy_scalars_from(d)
        return g

    def advect(self, field, t0, t1, spatial=HJWENO5_BIAS, temporal=TVD_RK2,
               tracker_spatial=HJWENO5_BIAS, tracker_temporal=TVD_RK1, norm_count=3,
               cfl=0.0):
        n, u = C.c_uint64(), C.c_uint64()
        fd = field.desc() if hasattr(field, "desc") else field
        _check(lib().oport_advect(self.h, C.addressof(fd), spatial, temporal, tracker_spatial,
                                  tracker_temporal, norm_count, t0, t1, cfl, C.byref(n),
                                  C.byref(u)))
        self.updates += u.value
        return n.value

    def tracker_op(self, op, arg=0, spatial=HJWENO5_BIAS, temporal=TVD_RK1,
                   norm_count=3, trim=TRIM_ALL):
        r = C.c_int()
        _check(lib().oport_tracker_op(self.h, op, arg, spatial, temporal, norm_count, trim,
                                      C.byref(r)))
        return r.value

    def track(self, **kw):
        self.tracker_op(0, **kw)

    def normalize(self, **kw):
        self.tracker_op(1, **kw)

    def prune(self, **kw):
        self.tracker_op(2, **kw)

    def dilate(self, n=1, **kw):
        self.tracker_op(3, n, **kw)

    def erode(self, n=1, **kw):
        self.tracker_op(4, n, **kw)

    def resize(self, half_width=3, **kw):
        return bool(self.tracker_op(5, half_width, **kw))


def weno5(v):
    """math::WENO5<float> (math/FiniteDifference.h:301-321) of each row of
    the float32 array v of shape (n, 5)."""
    v = np.ascontiguousarray(v, np.float32)
    out = np.empty(v.shape[0], np.float32)
    lib().oport_weno5(v.shape[0], v.ctypes.data_as(C.POINTER(C.c_float)), out.ctypes.data_as(C.POINTER(C.c_float)))
    return out


def _workload(threads=0):
    """The 64-sphere benchmark input (oracle rasteriser) and its field."""
    c, r = sixty_four_spheres(seed=2024)
    return PortGrid.spheres(c, r, 1.0, 3.0, threads), deformation(1024.0, 100.0, 1.0)


def _unit_step(grid, field, t):
    return grid.advect(field, t, t + 1.0, temporal=TVD_RK3, norm_count=1, cfl=0.5, tracker_temporal=TVD_RK1)


def bench_sample(seconds=15.0, threads=0):
    """CPU baseline on a bounded sample of the 64-sphere workload: whole unit
    steps from t = 0 until `seconds` of CPU time are spent."""
    g, field = _workload(threads)
    nthreads = threads if threads > 0 else (os.cpu_count() or 1)
    t, steps, el = 0.0, 0, 0.0
    while el < seconds:
        t0 = time.perf_counter()
        _unit_step(g, field, t)
        el += time.perf_counter() - t0
        t += 1.0
        steps += 1
    return {"value": g.updates / el, "unit": "voxel-updates/s", "cores": nthreads, "kind": "port",
            "sample": "64-sphere workload from t=0, %d whole time steps (%.1f s), all host threads"
                      % (steps, el)}


def bench_reference(steps=10, warmup=3, threads=0):
    """Reference arm: the restatement on all host threads over the same unit
    steps the GPU arm times: `warmup` untimed steps from t = 0, then `steps`
    timed steps, each advect(t, t+1) at CFL 0.5."""
    g, field = _workload(threads)
    nthreads = threads if threads > 0 else (os.cpu_count() or 1)
    t = 0.0
    for _ in range(warmup):
        _unit_step(g, field, t)
        t += 1.0
    g.updates = 0
    substeps = 0
    t_start = t
    t0 = time.perf_counter()
    for _ in range(steps):
        substeps += _unit_step(g, field, t)
        t += 1.0
    el = time.perf_counter() - t0
    value = g.updates / el
    return {"value": value, "ms_per_step": 1e3 * el / max(1, steps), "substeps": substeps,
            "t_start": t_start,
            "cpu_baseline": {"value": value, "unit": "voxel-updates/s", "cores": nthreads, "kind": "port",
                             "sample": "the timed unit steps t = %g .. %g of the 64-sphere workload "
                                       "(%.1f s), all host threads" % (t_start, t, el)}}


def bench_batch_sample(seconds=15.0, threads=0):
    """CPU baseline of the batched configuration: the restatement advances the
    seeded instances in order, one time unit each (RK3, tracker RK1, one
    renormalisation, CFL 0.5), until `seconds` of CPU time are spent."""
    from openvdb_gb300 import fixtures  # the batched line's CPU leg runs in the GPU arm's process
    specs, fields = fixtures.batch_instances(n=512, seed=7)
    nthreads = threads if threads > 0 else (os.cpu_count() or 1)
    updates, el, done = 0, 0.0, 0
    for spec, field in zip(specs, fields):
        g = PortGrid(fixtures.build_instance(spec), threads)
        t0 = time.perf_counter()
        g.advect(field, 0.0, 1.0, temporal=TVD_RK3, norm_count=1, cfl=0.5, tracker_temporal=TVD_RK1)
        el += time.perf_counter() - t0
        updates += g.updates
        done += 1
        if el >= seconds:
            break
    return {"value": updates / el, "unit": "voxel-updates/s", "cores": nthreads, "kind": "port",
            "sample": "batched configuration: the first %d of 512 instances, one time unit each (%.1f s), "
                      "all host threads" % (done, el)}

