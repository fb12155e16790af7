"""ctypes wrapper of oracle/_ref/libvdbref.so: the UNMODIFIED reference
(OpenVDB tools::LevelSetAdvection / LevelSetTracker, compiled from source by
oracle/ref/build_ref.py).  Test infrastructure only.

The library exists only where the reference checkout was present at build
time (the development container); `available()` reports whether it loaded.
"""
import ctypes as C
import os

import numpy as np

from openvdb_gb300 import _abi
from openvdb_gb300.grid import HostGrid

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libvdbref.so")
_lib = None


def available():
    try:
        lib()
        return True
    except OSError:
        return False


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(LIB_PATH)
        L.vdbref_last_error.restype = C.c_char_p
        L.vdbref_sphere.argtypes = [C.c_float] * 6 + [C.POINTER(C.c_void_p)]
        L.vdbref_union_spheres.argtypes = [C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                           C.c_float, C.c_float, C.POINTER(C.c_void_p)]
        L.vdbref_counts.argtypes = [C.c_void_p, C.POINTER(_abi.GridCounts)]
        L.vdbref_export.argtypes = [C.c_void_p, C.POINTER(_abi.GridDesc)]
        L.vdbref_from_desc.argtypes = [C.POINTER(_abi.GridDesc), C.POINTER(C.c_void_p)]
        L.vdbref_free.argtypes = [C.c_void_p]
        L.vdbref_free.restype = None
        L.vdbref_advect.argtypes = [C.c_void_p, C.POINTER(_abi.FieldDesc)] + [C.c_int] * 5 + \
            [C.c_float, C.c_float, C.POINTER(C.c_uint64)]
        L.vdbref_advect_cfl.argtypes = [C.c_void_p, C.POINTER(_abi.FieldDesc)] + [C.c_int] * 5 + \
            [C.c_float] * 3 + [C.POINTER(C.c_uint64)]
        L.vdbref_advect_enright.argtypes = [C.c_void_p] + [C.c_int] * 5 + [C.c_float] * 3 + [C.POINTER(C.c_uint64)]
        L.vdbref_tracker_op.argtypes = [C.c_void_p] + [C.c_int] * 6 + [C.POINTER(C.c_int)]
        L.vdbref_volume_advect.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double,
                                           C.POINTER(C.c_double)]
        L.vdbref_set_threads.argtypes = [C.c_int]
        L.vdbref_filter.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float] + [C.c_int] * 4
        L.vdbref_normalize_masked.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p] + [C.c_int] * 4
        L.vdbref_filter_masked.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_float] + [C.c_int] * 4 + \
            [C.c_float, C.c_float, C.c_int]
        L.vdbref_morph.argtypes = [C.c_void_p] * 3 + [C.c_int] * 5 + [C.c_float] * 4 + [C.c_int,
                                                                                    C.POINTER(C.c_uint64)]
        L.vdbref_write_vdb.argtypes = [C.c_void_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_int]
        L.vdbref_read_vdb.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_void_p)]
        L.vdbref_nano_float.argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.c_int, C.c_void_p, C.c_int64,
                                        C.POINTER(C.c_int64)]
        L.vdbref_nano_last_error.restype = C.c_char_p
        L.vdbref_nano_onindex.argtypes = [C.c_void_p, C.c_char_p] + [C.c_int] * 4 + [C.c_void_p, C.c_int64,
                                                                              C.POINTER(C.c_int64)]
        L.vdbref_nano_probe.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                        C.c_void_p]
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise RuntimeError("reference oracle error %d: %s" % (rc, lib().vdbref_last_error().decode()))


def set_threads(n):
    lib().vdbref_set_threads(int(n))


def threads():
    return lib().vdbref_threads()


class RefGrid:
    """A reference openvdb::FloatGrid held by the harness."""

    def __init__(self, handle):
        self.h = C.c_void_p(handle)

    def __del__(self):
        if getattr(self, "h", None) and self.h.value and _lib is not None:
            _lib.vdbref_free(self.h)
            self.h = None

    @classmethod
    def sphere(cls, radius, center=(0.0, 0.0, 0.0), voxel_size=1.0, half_width=3.0):
        h = C.c_void_p()
        _check(lib().vdbref_sphere(radius, center[0], center[1], center[2], voxel_size,
                                   half_width, C.byref(h)))
        return cls(h.value)

    @classmethod
    def union_of_spheres(cls, centers, radii, voxel_size=1.0, half_width=3.0):
        import numpy as np
        c = np.ascontiguousarray(centers, np.float32).reshape(-1)
        r = np.ascontiguousarray(radii, np.float32).reshape(-1)
        h = C.c_void_p()
        _check(lib().vdbref_union_spheres(len(r), c.ctypes.data_as(C.POINTER(C.c_float)),
                                          r.ctypes.data_as(C.POINTER(C.c_float)), voxel_size,
                                          half_width, C.byref(h)))
        return cls(h.value)

    @classmethod
    def from_host(cls, grid):
        d = grid.desc()
        h = C.c_void_p()
        _check(lib().vdbref_from_desc(C.byref(d), C.byref(h)))
        return cls(h.value)

    @classmethod
    def read_vdb(cls, path, name):
        """The grid `name` of a .vdb file, read by the reference's own
        GridDescriptor / MetaMap / Transform / tree deserialisers."""
        h = C.c_void_p()
        _check(lib().vdbref_read_vdb(os.fsencode(path), name.encode(), C.byref(h)))
        return cls(h.value)

    def write_vdb(self, path, name, uuid="0" * 36, half=False):
        """A one-grid .vdb file written by the reference's own serialisers
        (class, name and statistics metadata; active-mask compression)."""
        _check(lib().vdbref_write_vdb(self.h, name.encode(), os.fsencode(path), uuid.encode(), int(half)))

    def nanovdb(self, name, stats=3, checksum=1):
        """nanovdb::tools::createNanoGrid(grid, StatsMode(stats), CheckMode(checksum))
        of the reference, as a uint8 array."""
        n = C.c_int64()
        L = lib()
        if L.vdbref_nano_float(self.h, name.encode(), stats, checksum, None, 0, C.byref(n)):
            raise RuntimeError(L.vdbref_nano_last_error().decode())
        buf = np.zeros(n.value, np.uint8)
        if L.vdbref_nano_float(self.h, name.encode(), stats, checksum, buf.ctypes.data, n.value, C.byref(n)):
            raise RuntimeError(L.vdbref_nano_last_error().decode())
        return buf

    def nanovdb_index(self, name, channels=1, stats=True, tiles=True, checksum=1):
        """createNanoGrid<FloatGrid, ValueOnIndex>(grid, channels, stats, tiles) of the reference."""
        n = C.c_int64()
        L = lib()
        args = (self.h, name.encode(), channels, int(stats), int(tiles), checksum)
        if L.vdbref_nano_onindex(*args, None, 0, C.byref(n)):
            raise RuntimeError(L.vdbref_nano_last_error().decode())
        buf = np.zeros(n.value, np.uint8)
        if L.vdbref_nano_onindex(*args, buf.ctypes.data, n.value, C.byref(n)):
            raise RuntimeError(L.vdbref_nano_last_error().decode())
        return buf

    def counts(self):
        c = _abi.GridCounts()
        _check(lib().vdbref_counts(self.h, C.byref(c)))
        return c

    def to_host(self):
        g = HostGrid.allocate(self.counts())
        d = g.desc()
        _check(lib().vdbref_export(self.h, C.byref(d)))
        g.copy_scalars_from(d)
        return g

    def advect(self, field, t0, t1, spatial=_abi.HJWENO5_BIAS, temporal=_abi.TVD_RK2,
               tracker_spatial=_abi.HJWENO5_BIAS, tracker_temporal=_abi.TVD_RK1, norm_count=3, cfl=0.0):
        """advect(t0, t1); with cfl > 0 the reference's advect over greedy
        intervals of cfl*dx/max|v| (the imposed-CFL driver of ref_harness.cc)."""
        n = C.c_uint64()
        fd = field.desc() if hasattr(field, "desc") else field
        _check(lib().vdbref_advect_cfl(self.h, C.byref(fd), spatial, temporal, tracker_spatial,
                                       tracker_temporal, norm_count, t0, t1, cfl, C.byref(n)))
        return n.value

    def advect_enright(self, t0, t1, spatial=_abi.HJWENO5_BIAS, temporal=_abi.TVD_RK2,
                       tracker_spatial=_abi.HJWENO5_BIAS, tracker_temporal=_abi.TVD_RK1, norm_count=3, cfl=0.0):
        """LevelSetAdvection<FloatGrid>::advect with its default field,
        tools::EnrightField<float>."""
        n = C.c_uint64()
        _check(lib().vdbref_advect_enright(self.h, spatial, temporal, tracker_spatial, tracker_temporal, norm_count,
                                           t0, t1, cfl, C.byref(n)))
        return n.value

    def volume_advect(self, field, time_step, integrator=0, limiter=1, substeps=1):
        """tools::VolumeAdvection<Vec3fGrid>::advect<FloatGrid, BoxSampler>
        (tools/VolumeAdvect.h:205-222) in the dense velocity `field`; the grid
        becomes the advected copy.  Returns getMaxVelocity()."""
        fd = field.desc() if hasattr(field, "desc") else field
        m = C.c_double()
        _check(lib().vdbref_volume_advect(self.h, C.addressof(fd), integrator, limiter, substeps, time_step,
                                          C.byref(m)))
        return m.value

    def morph(self, target, t0, t1, mask=None, mask_range=(0.0, 1.0), invert=False,
              spatial=_abi.HJWENO5_BIAS, temporal=_abi.TVD_RK2, tracker_spatial=_abi.HJWENO5_BIAS,
              tracker_temporal=_abi.TVD_RK1, norm_count=3):
        """tools::LevelSetMorphing::advect(t0, t1) towards the RefGrid `target`."""
        n = C.c_uint64()
        _check(lib().vdbref_morph(self.h, target.h, mask.h if mask is not None else None, spatial, temporal,
                                  tracker_spatial, tracker_temporal, norm_count, t0, t1, mask_range[0],
                                  mask_range[1], 1 if invert else 0, C.byref(n)))
        return n.value

    def filter(self, op, width=1, value=0.0, spatial=_abi.HJWENO5_BIAS, temporal=_abi.TVD_RK1, norm_count=3,
               trim=_abi.TRIM_ALL, mask=None, mask_range=(0.0, 1.0), invert=False):
        """tools::LevelSetFilter: op 0 laplacian, 1 mean, 2 gaussian, 3 offset, 4 meanCurvature,
        5 fillet, 6 median; `mask` (a RefGrid) is the filter's alpha mask."""
        if mask is None:
            _check(lib().vdbref_filter(self.h, op, width, value, spatial, temporal, norm_count, trim))
        else:
            _check(lib().vdbref_filter_masked(self.h, mask.h, op, width, value, spatial, temporal, norm_count,
                                              trim, mask_range[0], mask_range[1], 1 if invert else 0))

    def tracker_op(self, op, arg=0, spatial=_abi.HJWENO5_BIAS, temporal=_abi.TVD_RK1,
                   norm_count=3, trim=_abi.TRIM_ALL):
        r = C.c_int()
        _check(lib().vdbref_tracker_op(self.h, op, arg, spatial, temporal, norm_count, trim,
                                       C.byref(r)))
        return r.value

    def track(self, **kw):
        self.tracker_op(0, **kw)

    def normalize(self, **kw):
        self.tracker_op(1, **kw)

    def normalize_masked(self, origins, masks, spatial=_abi.HJWENO5_BIAS, temporal=_abi.TVD_RK1, norm_count=3,
                         trim=_abi.TRIM_ALL):
        """LevelSetTracker::normalize(&mask), the mask a MaskTree of the given leaves."""
        o = np.ascontiguousarray(origins, dtype=np.int32)
        m = np.ascontiguousarray(masks, dtype=np.uint64)
        _check(lib().vdbref_normalize_masked(self.h, len(o), o.ctypes.data, m.ctypes.data, spatial, temporal,
                                             norm_count, trim))

    def prune(self, **kw):
        self.tracker_op(2, **kw)

    def dilate(self, n=1, **kw):
        self.tracker_op(3, n, **kw)

    def erode(self, n=1, **kw):
        self.tracker_op(4, n, **kw)

    def resize(self, half_width=3, **kw):
        return bool(self.tracker_op(5, half_width, **kw))


def nano_probe(buf, ijk):
    """The reference's ReadAccessor on a NanoVDB buffer: (float values or
    uint64 indices, active flags) at the index coordinates ijk (n x 3)."""
    L = lib()
    b = np.ascontiguousarray(buf, np.uint8)
    c = np.ascontiguousarray(ijk, np.int32)
    n = c.shape[0]
    fv = np.zeros(n, np.float32)
    iv = np.zeros(n, np.uint64)
    act = np.zeros(n, np.uint8)
    if L.vdbref_nano_probe(b.ctypes.data, b.size, c.ctypes.data, n, fv.ctypes.data, iv.ctypes.data, act.ctypes.data):
        raise RuntimeError(L.vdbref_nano_last_error().decode())
    is_float = int(np.frombuffer(b[636:640].tobytes(), np.uint32)[0]) == 1
    return (fv if is_float else iv), act

