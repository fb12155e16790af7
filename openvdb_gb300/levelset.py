"""Python mirror of OpenVDB's LevelSetTracker / LevelSetAdvection call surface
over the C ABI (include/gbls.h).

Reference interfaces:
  tools/LevelSetTracker.h:56-256  LevelSetTracker (ctor :258-277, setters
                                  :137-173, track :302-315, normalize :394-446,
                                  prune :279-300, dilate :317-337)
  tools/LevelSetAdvect.h:71-213   LevelSetAdvection (ctor defaults :86-89,
                                  advect :216-289)

The level set lives on the GPU in a DeviceLevelSet; the reference mutates its
FloatGrid in place, here the DeviceLevelSet is mutated in place and
to_host() returns the grid in the reference's canonical layout.
"""
import ctypes as C

import numpy as np

from . import _abi
from ._lib import GblsError, check, lib
from .grid import HostGrid

HJWENO5_BIAS = _abi.HJWENO5_BIAS
TVD_RK1, TVD_RK2, TVD_RK3 = _abi.TVD_RK1, _abi.TVD_RK2, _abi.TVD_RK3
PARITY, FAST, FP64 = _abi.MODE_PARITY, _abi.MODE_FAST, _abi.MODE_FP64


class ValueError_(ValueError):
    """openvdb::ValueError (unsupported scheme or map)."""


class RuntimeError_(RuntimeError):
    """openvdb::RuntimeError (not a level set / non-uniform voxels)."""


def _raise(e):
    if e.code == _abi.ERR_VALUE:
        raise ValueError_(str(e)) from None
    if e.code == _abi.ERR_RUNTIME:
        raise RuntimeError_(str(e)) from None
    raise e


def _call(rc):
    try:
        return check(rc)
    except GblsError as e:
        _raise(e)


class DeviceLevelSet:
    """A narrow-band FP32 level set resident on the GPU (one gbls_handle)."""

    def __init__(self, grid, device=0):
        L = lib()
        _call(L.gbls_set_device(int(device)))
        self._h = C.c_void_p()
        self._keep = grid  # the descriptor points into grid's arrays during create
        d = grid.desc()
        _call(L.gbls_create(C.byref(d), C.byref(self._h)))
        self._keep = None
        self.voxel_size = grid.voxel_size
        self.background = grid.background
        self.device = int(device)

    @classmethod
    def _adopt(cls, handle, voxel_size, background, device):
        """A DeviceLevelSet owning an already created gbls_handle."""
        obj = cls.__new__(cls)
        obj._h = handle
        obj._keep = None
        obj.voxel_size = voxel_size
        obj.background = background
        obj.device = int(device)
        return obj

    @property
    def handle(self):
        return self._h

    def upload(self, grid):
        """Replace the level set with `grid`, keeping this handle's device
        allocations and settings (gbls_upload)."""
        self._keep = grid
        d = grid.desc()
        try:
            _call(lib().gbls_upload(self._h, C.byref(d)))
        finally:
            self._keep = None
        self.voxel_size = grid.voxel_size
        self.background = grid.background

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().gbls_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def counts(self):
        c = _abi.GridCounts()
        _call(lib().gbls_get_counts(self._h, C.byref(c)))
        return c

    def active_voxel_count(self):
        return self.counts().active_voxel_count

    def leaf_count(self):
        return self.counts().leaf_count

    def to_host(self, arena=None):
        """Download into a new HostGrid (arrays from `arena` when given)."""
        g = HostGrid.allocate(self.counts(), arena)
        d = g.desc()
        _call(lib().gbls_download(self._h, C.byref(d)))
        g.copy_scalars_from(d)
        return g

    def set_precision(self, mode):
        """PARITY, FAST, or FP64 (the values widened to double: the FP64
        instance of the scheme, the error oracle of the FP32 run)."""
        _call(lib().gbls_set_precision(self._h, int(mode)))

    def active_values_f64(self):
        """Active values in canonical order as float64 (FP64 instance: its
        doubles; FP32 level sets: widened)."""
        out = np.zeros(self.active_voxel_count(), np.float64)
        _call(lib().gbls_get_active_values_f64(self._h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def set_stream(self, stream_ptr):
        _call(lib().gbls_set_stream(self._h, C.c_void_p(stream_ptr)))

    def stats(self):
        st = _abi.Stats()
        _call(lib().gbls_get_stats(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in _abi.Stats._fields_}

    def reset_stats(self):
        _call(lib().gbls_reset_stats(self._h))

    def set_profiling(self, enable=True):
        _call(lib().gbls_set_profiling(self._h, 1 if enable else 0))


class DeviceVolume(DeviceLevelSet):
    """A FloatGrid volume (e.g. a fog density) resident on the GPU
    (gbls_create_volume): any background; volume operations only."""

    def __init__(self, grid, device=0):
        L = lib()
        _call(L.gbls_set_device(int(device)))
        self._h = C.c_void_p()
        self._keep = grid
        d = grid.desc()
        _call(L.gbls_create_volume(C.byref(d), C.byref(self._h)))
        self._keep = None
        self.voxel_size = grid.voxel_size
        self.background = grid.background
        self.device = int(device)


class VolumeAdvection:
    """tools::VolumeAdvection<Vec3fGrid> (tools/VolumeAdvect.h:76-262) with the
    reference's method names, advecting FloatGrid volumes (fog densities)
    held by a DeviceVolume through gbls_volume_advect.  advect(grid, dt)
    replaces the grid's contents with the advected copy (the reference returns
    a new grid and leaves its input unchanged)."""

    SEMI, MID, RK3, RK4, MAC, BFECC = range(6)
    NO_LIMITER, CLAMP, REVERT = range(3)

    def __init__(self, velocity):
        """`velocity`: a Field (DENSE or CONSTANT) or a DeviceField."""
        self._field = velocity if isinstance(velocity, DeviceField) else DeviceField(velocity)
        self._integrator = self.SEMI
        self._limiter = self.CLAMP
        self._substeps = 1
        self._max_velocity = None

    def spatialOrder(self):
        return 2 if self._integrator in (self.MAC, self.BFECC) else 1

    def temporalOrder(self):
        return {self.SEMI: 1, self.MID: 2, self.RK3: 3, self.RK4: 4, self.BFECC: 2, self.MAC: 2}[self._integrator]

    def setIntegrator(self, integrator):
        self._integrator = int(integrator)

    def getIntegrator(self):
        return self._integrator

    def setLimiter(self, limiter):
        self._limiter = int(limiter)

    def getLimiter(self):
        return self._limiter

    def isLimiterOn(self):
        return self.spatialOrder() > 1 and self._limiter != self.NO_LIMITER

    def setSubSteps(self, substeps):
        self._substeps = max(1, int(substeps))

    def getSubSteps(self):
        return self._substeps

    def getMaxVelocity(self):
        """max |v| over the velocity grid's values and background (known after
        the first advect call)."""
        return self._max_velocity

    def advect(self, grid, time_step):
        m = C.c_double()
        _call(lib().gbls_volume_advect(grid.handle, self._field._h, self._integrator, self._limiter,
                                       self._substeps, float(time_step), C.byref(m)))
        self._max_velocity = m.value
        return grid


class DeviceField:
    """A velocity field uploaded to the GPU (gbls_field)."""

    def __init__(self, field):
        self._h = C.c_void_p()
        self._field = field
        d = field.desc()
        _call(lib().gbls_field_create(C.byref(d), C.byref(self._h)))

    def __del__(self):
        try:
            if self._h.value:
                lib().gbls_field_destroy(self._h)
        except Exception:
            pass


class LevelSetTracker:
    """tools::LevelSetTracker<FloatGrid> over a DeviceLevelSet."""

    def __init__(self, grid, interrupter=None):
        self._grid = grid
        self._intr_keep = None
        if interrupter is not None:
            self.setInterrupter(interrupter)

    # ---- state (tools/LevelSetTracker.h:74-83, :137-173) ----
    def _state(self):
        s, t, n, g = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _call(lib().gbls_get_tracker_state(self._grid.handle, C.byref(s), C.byref(t), C.byref(n),
                                           C.byref(g)))
        return [s.value, t.value, n.value, g.value]

    def _set(self, i, v):
        st = self._state()
        st[i] = int(v)
        _call(lib().gbls_set_tracker_state(self._grid.handle, *st))

    def getSpatialScheme(self):
        return self._state()[0]

    def setSpatialScheme(self, s):
        self._set(0, s)

    def getTemporalScheme(self):
        return self._state()[1]

    def setTemporalScheme(self, t):
        self._set(1, t)

    def getNormCount(self):
        return self._state()[2]

    def setNormCount(self, n):
        self._set(2, n)

    def getGrainSize(self):
        return self._state()[3]

    def setGrainSize(self, g):
        self._set(3, g)

    def setTrimming(self, mode):
        _call(lib().gbls_set_trimming(self._grid.handle, int(mode)))

    def voxelSize(self):
        return np.float32(self._grid.voxel_size)

    def getHalfWidth(self):
        # background / dx in float, with the device's current background
        return float(np.float32(self._grid.counts().background) / np.float32(self._grid.voxel_size))

    def grid(self):
        return self._grid

    def setInterrupter(self, obj):
        """obj has start(name), end(), wasInterrupted(percent) (util/NullInterrupter.h:29-49)."""
        start = _abi.INTERRUPT_START(lambda u, name: obj.start(name.decode() if name else ""))
        end = _abi.INTERRUPT_END(lambda u: obj.end())
        chk = _abi.INTERRUPT_CHECK(lambda u, p: 1 if obj.wasInterrupted(p) else 0)
        it = _abi.Interrupter(start, end, chk, None)
        self._intr_keep = (start, end, chk, it)
        _call(lib().gbls_set_interrupter(self._grid.handle, C.byref(it)))

    # ---- operations ----
    def track(self):
        _call(lib().gbls_track(self._grid.handle))

    def normalize(self, mask=None):
        """normalize() or normalize(&mask): `mask` is (leaf origins [n, 3],
        active masks [n, 8] uint64) of the mask tree's leaves; only their
        active voxels in leaves of the level set are renormalised."""
        if mask is None:
            _call(lib().gbls_normalize(self._grid.handle))
            return
        o = np.ascontiguousarray(mask[0], dtype=np.int32).reshape(-1, 3)
        m = np.ascontiguousarray(mask[1], dtype=np.uint64).reshape(-1, 8)
        if len(o) != len(m):
            raise ValueError("mask origins and masks differ in length")
        _call(lib().gbls_normalize_masked(self._grid.handle, len(o), o.ctypes.data, m.ctypes.data))

    def prune(self):
        _call(lib().gbls_prune(self._grid.handle))

    def dilate(self, iterations=1):
        _call(lib().gbls_dilate(self._grid.handle, int(iterations)))

    def erode(self, iterations=1):
        _call(lib().gbls_erode(self._grid.handle, int(iterations)))

    def resize(self, half_width=3):
        ch = C.c_int()
        _call(lib().gbls_resize(self._grid.handle, int(half_width), C.byref(ch)))
        return bool(ch.value)


class LevelSetAdvection:
    """tools::LevelSetAdvection<FloatGrid, FieldT> over a DeviceLevelSet.

    Defaults follow the reference constructor (tools/LevelSetAdvect.h:86-89):
    HJWENO5 + TVD_RK2 for advection, and the tracker's HJWENO5 + TVD_RK1 with
    normCount 3.  `cfl` <= 0 keeps the reference CFL number; `precision`
    selects PARITY (bit-identical to the reference) or FAST (FP32) kernels.
    """

    def __init__(self, grid, field, interrupter=None):
        self._grid = grid
        self._field = field if isinstance(field, DeviceField) else DeviceField(field)
        self.tracker = LevelSetTracker(grid, interrupter)
        self._spatial = HJWENO5_BIAS
        self._temporal = TVD_RK2
        self.cfl = 0.0

    def getSpatialScheme(self):
        return self._spatial

    def setSpatialScheme(self, s):
        self._spatial = int(s)

    def getTemporalScheme(self):
        return self._temporal

    def setTemporalScheme(self, t):
        self._temporal = int(t)

    def getTrackerSpatialScheme(self):
        return self.tracker.getSpatialScheme()

    def setTrackerSpatialScheme(self, s):
        self.tracker.setSpatialScheme(s)

    def getTrackerTemporalScheme(self):
        return self.tracker.getTemporalScheme()

    def setTrackerTemporalScheme(self, t):
        self.tracker.setTemporalScheme(t)

    def getNormCount(self):
        return self.tracker.getNormCount()

    def setNormCount(self, n):
        self.tracker.setNormCount(n)

    def getGrainSize(self):
        return self.tracker.getGrainSize()

    def setGrainSize(self, g):
        self.tracker.setGrainSize(g)

    def setPrecision(self, mode):
        self._grid.set_precision(mode)

    def advect(self, t0, t1):
        """Advect from t0 to t1; returns the number of CFL substeps."""
        n = C.c_uint64()
        rc = lib().gbls_advect(self._grid.handle, self._field._h, self._spatial, self._temporal,
                               np.float32(t0), np.float32(t1), np.float32(self.cfl), C.byref(n))
        if rc == _abi.ERR_INTERRUPTED:
            return n.value
        _call(rc)
        return n.value


class LevelSetFilter(LevelSetTracker):
    """tools::LevelSetFilter<FloatGrid, FloatGrid> (tools/LevelSetFilter.h:47-160):
    filters on a DeviceLevelSet, each followed by track() with this tracker's
    state.  The optional alpha mask of every filter is a DeviceLevelSet on the
    same device with the same transform (setMaskRange, invertMask as the
    reference); widths above 3 are refused (GBLS status)."""

    def __init__(self, grid, interrupter=None):
        super().__init__(grid, interrupter)
        self._min_mask, self._max_mask, self._invert = 0.0, 1.0, False

    def minMask(self):
        return self._min_mask

    def maxMask(self):
        return self._max_mask

    def setMaskRange(self, lo, hi):
        if not lo < hi:
            raise ValueError("Invalid mask range (expects min < max)")
        self._min_mask, self._max_mask = float(lo), float(hi)

    def isMaskInverted(self):
        return self._invert

    def invertMask(self, invert=True):
        self._invert = bool(invert)

    def _filter(self, op, width=1, value=0.0, mask=None):
        if mask is None:
            rc = lib().gbls_filter(self._grid.handle, int(op), int(width), np.float32(value))
        else:
            rc = lib().gbls_filter_masked(self._grid.handle, int(op), int(width), np.float32(value), mask.handle,
                                          np.float32(self._min_mask), np.float32(self._max_mask),
                                          1 if self._invert else 0)
        if rc == _abi.ERR_INTERRUPTED:
            return
        _call(rc)

    def laplacian(self, mask=None):
        self._filter(0, mask=mask)

    def mean(self, width=1, mask=None):
        self._filter(1, width, mask=mask)

    def gaussian(self, width=1, mask=None):
        self._filter(2, width, mask=mask)

    def offset(self, value, mask=None):
        self._filter(3, 1, value, mask=mask)

    def meanCurvature(self, mask=None):
        self._filter(4, mask=mask)

    def fillet(self, mask=None):
        self._filter(5, mask=mask)

    def median(self, width=1, mask=None):
        self._filter(6, width, mask=mask)


class LevelSetMorphing:
    """tools::LevelSetMorphing<FloatGrid> over DeviceLevelSets
    (tools/LevelSetMorph.h:47-141): `source` moves towards `target`.

    Defaults follow the reference constructor: HJWENO5 + TVD_RK2, the
    tracker's HJWENO5 + TVD_RK1 with normCount 3, mask range [0, 1], mask not
    inverted.  The target and the alpha mask are level sets on the source's
    device with the same transform.
    """

    def __init__(self, source, target, interrupter=None):
        self._grid = source
        self._target = target
        self._mask = None
        self.tracker = LevelSetTracker(source, interrupter)
        self._spatial = HJWENO5_BIAS
        self._temporal = TVD_RK2
        self._min_mask, self._max_mask, self._invert = 0.0, 1.0, False

    def setTarget(self, target):
        self._target = target

    def setAlphaMask(self, mask):
        self._mask = mask

    def getSpatialScheme(self):
        return self._spatial

    def setSpatialScheme(self, s):
        self._spatial = int(s)

    def getTemporalScheme(self):
        return self._temporal

    def setTemporalScheme(self, t):
        self._temporal = int(t)

    def getTrackerSpatialScheme(self):
        return self.tracker.getSpatialScheme()

    def setTrackerSpatialScheme(self, s):
        self.tracker.setSpatialScheme(s)

    def getTrackerTemporalScheme(self):
        return self.tracker.getTemporalScheme()

    def setTrackerTemporalScheme(self, t):
        self.tracker.setTemporalScheme(t)

    def getNormCount(self):
        return self.tracker.getNormCount()

    def setNormCount(self, n):
        self.tracker.setNormCount(n)

    def getGrainSize(self):
        return self.tracker.getGrainSize()

    def setGrainSize(self, g):
        self.tracker.setGrainSize(g)

    def minMask(self):
        return self._min_mask

    def maxMask(self):
        # the reference returns mDeltaMask + mMinMask with mDeltaMask = max - min
        return float((np.float32(self._max_mask) - np.float32(self._min_mask)) + np.float32(self._min_mask))

    def setMaskRange(self, lo, hi):
        if not (np.float32(lo) < np.float32(hi)):
            raise ValueError("Invalid mask range (expects min < max)")
        # gbls_morph forms max - min itself, as setMaskRange does
        self._min_mask = float(np.float32(lo))
        self._max_mask = float(np.float32(hi))

    def isMaskInverted(self):
        return self._invert

    def invertMask(self, invert=True):
        self._invert = bool(invert)

    def advect(self, t0, t1):
        """Morph from t0 to t1; returns the number of CFL substeps."""
        n = C.c_uint64()
        lo, hi = np.float32(self._min_mask), np.float32(self._max_mask)
        rc = lib().gbls_morph(self._grid.handle, self._target.handle,
                              self._mask.handle if self._mask is not None else None, self._spatial,
                              self._temporal, np.float32(t0), np.float32(t1), lo, hi,
                              1 if self._invert else 0, C.byref(n))
        if rc == _abi.ERR_INTERRUPTED:
            return n.value
        _call(rc)
        return n.value


class DeviceBatch:
    """Many independent level sets on the GPU (gbls_batch_*): each instance is
    advanced exactly as its own LevelSetAdvection::advect call would."""

    def __init__(self, grids, device=0):
        L = lib()
        _call(L.gbls_set_device(int(device)))
        self._keep = list(grids)
        descs = (_abi.GridDesc * len(self._keep))(*[g.desc() for g in self._keep])
        self._h = C.c_void_p()
        _call(L.gbls_batch_create(len(self._keep), descs, C.byref(self._h)))
        self._keep = None
        self.n = len(descs)
        self.device = int(device)

    @property
    def handle(self):
        return self._h

    def __del__(self):
        try:
            if self._h.value:
                lib().gbls_destroy(self._h)
        except Exception:
            pass

    def set_precision(self, mode):
        _call(lib().gbls_set_precision(self._h, int(mode)))

    def set_tracker(self, spatial=HJWENO5_BIAS, temporal=TVD_RK1, norm_count=1, grain=1):
        _call(lib().gbls_set_tracker_state(self._h, int(spatial), int(temporal), int(norm_count),
                                           int(grain)))

    def counts(self, i):
        c = _abi.GridCounts()
        _call(lib().gbls_batch_get_counts(self._h, int(i), C.byref(c)))
        return c

    def to_host(self, i):
        g = HostGrid.allocate(self.counts(i))
        d = g.desc()
        _call(lib().gbls_batch_download(self._h, int(i), C.byref(d)))
        g.copy_scalars_from(d)
        return g

    def advect(self, fields, t0, t1, spatial=HJWENO5_BIAS, temporal=TVD_RK3, cfl=0.0):
        fd = (_abi.FieldDesc * self.n)(*[f.desc() for f in fields])
        counts = (C.c_uint64 * self.n)()
        _call(lib().gbls_batch_advect(self._h, fd, int(spatial), int(temporal), np.float32(t0),
                                      np.float32(t1), np.float32(cfl), counts))
        return list(counts)

    def stats(self):
        st = _abi.Stats()
        _call(lib().gbls_get_stats(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in _abi.Stats._fields_}

    def reset_stats(self):
        _call(lib().gbls_reset_stats(self._h))

    def set_profiling(self, enable=True):
        _call(lib().gbls_set_profiling(self._h, 1 if enable else 0))

    def set_stream(self, stream_ptr):
        _call(lib().gbls_set_stream(self._h, C.c_void_p(stream_ptr)))
