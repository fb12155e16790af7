"""ctypes wrapper of the oracle's C++ restatement (oracle/_build/liboracle_port.so).

Test infrastructure: the parity oracle on hosts without the compiled
reference, and the timed CPU baseline / reference arm of bench.py.  Pinned
against the compiled reference through tests/golden/parity_cases.json
(tests/test_oracle_port.py).
"""
import ctypes as C
import os
import time

import numpy as np

from openvdb_gb300 import _abi
from openvdb_gb300.grid import HostGrid

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liboracle_port.so")
_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.oport_last_error.restype = C.c_char_p
        L.oport_create.argtypes = [C.POINTER(_abi.GridDesc), C.c_int]
        L.oport_create.restype = vp
        L.oport_create_prec.argtypes = [C.POINTER(_abi.GridDesc), C.c_int, C.c_int]
        L.oport_create_prec.restype = vp
        L.oport_active_values.argtypes = [vp, C.POINTER(C.c_double)]
        L.oport_set_active_values.argtypes = [vp, C.POINTER(C.c_double)]
        L.oport_free.argtypes = [vp]
        L.oport_free.restype = None
        L.oport_set_threads.argtypes = [vp, C.c_int]
        L.oport_set_threads.restype = None
        L.oport_counts.argtypes = [vp, C.POINTER(_abi.GridCounts)]
        L.oport_export.argtypes = [vp, C.POINTER(_abi.GridDesc)]
        L.oport_tracker_op.argtypes = [vp] + [C.c_int] * 6 + [C.POINTER(C.c_int)]
        L.oport_advect.argtypes = [vp, C.POINTER(_abi.FieldDesc)] + [C.c_int] * 5 + \
            [C.c_float, C.c_float, C.c_float, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
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


class PortGrid:
    """A level set held by the C++ restatement."""

    def __init__(self, host, threads=0, precision=32):
        """precision 32: bit-identical to the reference; 64: the same scheme
        (same constants, same operations) evaluated in FP64."""
        d = host.desc()
        self.h = C.c_void_p(lib().oport_create_prec(C.byref(d), int(threads), int(precision)))
        self.updates = 0

    def active_values(self):
        out = np.zeros(self.counts().active_voxel_count, np.float64)
        _check(lib().oport_active_values(self.h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def set_active_values(self, values):
        v = np.ascontiguousarray(values, np.float64)
        assert v.size == self.counts().active_voxel_count
        _check(lib().oport_set_active_values(self.h, v.ctypes.data_as(C.POINTER(C.c_double))))

    def __del__(self):
        if getattr(self, "h", None) and self.h.value and _lib is not None:
            _lib.oport_free(self.h)

    def set_threads(self, n):
        lib().oport_set_threads(self.h, int(n))

    def counts(self):
        c = _abi.GridCounts()
        _check(lib().oport_counts(self.h, C.byref(c)))
        return c

    def to_host(self):
        g = HostGrid.allocate(self.counts())
        d = g.desc()
        _check(lib().oport_export(self.h, C.byref(d)))
        g.copy_scalars_from(d)
        return g

    def advect(self, field, t0, t1, spatial=_abi.HJWENO5_BIAS, temporal=_abi.TVD_RK2,
               tracker_spatial=_abi.HJWENO5_BIAS, tracker_temporal=_abi.TVD_RK1, norm_count=3,
               cfl=0.0):
        n, u = C.c_uint64(), C.c_uint64()
        fd = field.desc() if hasattr(field, "desc") else field
        _check(lib().oport_advect(self.h, C.byref(fd), spatial, temporal, tracker_spatial,
                                  tracker_temporal, norm_count, t0, t1, cfl, C.byref(n),
                                  C.byref(u)))
        self.updates += u.value
        return n.value

    def tracker_op(self, op, arg=0, spatial=_abi.HJWENO5_BIAS, temporal=_abi.TVD_RK1,
                   norm_count=3, trim=_abi.TRIM_ALL):
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


def _workload():
    from openvdb_gb300 import Field, fixtures
    centers, radii = fixtures.sixty_four_spheres(seed=2024)
    host = fixtures.union_of_spheres(centers, radii, 1.0, 3.0)
    return host, Field.deformation(domain=1024.0, period=100.0, scale=1.0)


def _advect_for(grid, field, t, seconds):
    """Advect unit time steps from t until `seconds` of CPU time are spent."""
    t0 = time.perf_counter()
    steps = 0
    while True:
        grid.advect(field, t, t + 1.0, temporal=_abi.TVD_RK3, norm_count=1, cfl=0.5,
                    tracker_temporal=_abi.TVD_RK1)
        t += 1.0
        steps += 1
        if time.perf_counter() - t0 >= seconds:
            break
    return steps, time.perf_counter() - t0, t


def bench_sample(seconds=15.0, threads=0):
    """CPU baseline on a bounded sample of the 64-sphere workload."""
    host, field = _workload()
    g = PortGrid(host, threads)
    nthreads = threads if threads > 0 else (os.cpu_count() or 1)
    steps, el, _ = _advect_for(g, field, 0.0, seconds)
    return {"value": g.updates / el, "unit": "voxel-updates/s", "cores": nthreads, "kind": "port",
            "sample": "64-sphere workload from t=0, %d whole time steps (%.1f s), all host threads"
                      % (steps, el)}


def bench_reference(steps=10, warmup=3, seconds=15.0, threads=0):
    """Reference arm: the restatement on all host threads; each step is a
    bounded sample (whole time units until seconds/steps of CPU time)."""
    host, field = _workload()
    g = PortGrid(host, threads)
    nthreads = threads if threads > 0 else (os.cpu_count() or 1)
    t = 0.0
    per = max(0.5, seconds / max(1, steps))
    for _ in range(min(warmup, 1)):
        g.advect(field, t, t + 1.0, temporal=_abi.TVD_RK3, norm_count=1, cfl=0.5)
        t += 1.0
    g.updates = 0
    tot = 0.0
    nsteps = 0
    for _ in range(steps):
        n, el, t = _advect_for(g, field, t, per)
        tot += el
        nsteps += n
    value = g.updates / tot
    return {"value": value, "ms_per_step": 1e3 * tot / max(1, nsteps),
            "cpu_baseline": {"value": value, "unit": "voxel-updates/s", "cores": nthreads,
                             "kind": "port",
                             "sample": "64-sphere workload, %d time steps in %.1f s" % (nsteps, tot)}}


def bench_batch_sample(seconds=15.0, threads=0):
    """CPU baseline of the batched configuration: the restatement advances the
    seeded instances in order, one time unit each (RK3, tracker RK1, one
    renormalisation, CFL 0.5), until `seconds` of CPU time are spent."""
    from openvdb_gb300 import fixtures
    specs, fields = fixtures.batch_instances(n=512, seed=7)
    nthreads = threads if threads > 0 else (os.cpu_count() or 1)
    updates, el, done = 0, 0.0, 0
    for spec, field in zip(specs, fields):
        g = PortGrid(fixtures.build_instance(spec), threads)
        t0 = time.perf_counter()
        g.advect(field, 0.0, 1.0, temporal=_abi.TVD_RK3, norm_count=1, cfl=0.5, tracker_temporal=_abi.TVD_RK1)
        el += time.perf_counter() - t0
        updates += g.updates
        done += 1
        if el >= seconds:
            break
    return {"value": updates / el, "unit": "voxel-updates/s", "cores": nthreads, "kind": "port",
            "sample": "batched configuration: the first %d of 512 instances, one time unit each (%.1f s), "
                      "all host threads" % (done, el)}

