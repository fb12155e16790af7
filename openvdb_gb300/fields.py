"""Velocity-field descriptions (gbls_field_desc) for the advection entry point.

The reference advects in any functor with operator()(Coord, t)
(tools/LevelSetAdvect.h:32-52).  The kinds here cover the reference's
DiscreteField (tools/VelocityFields.h:42-94), aligned or with its own
transform (trilinear BoxSampler), two analytic fields whose arithmetic is
defined in include/gbls_fields.h, and any functor sampled on the host once
per substep (the reference's default EnrightField among them).
"""
import ctypes as C

import numpy as np

from . import _abi


class Field:
    def __init__(self, kind, **kw):
        self.kind = kind
        self.constant = tuple(kw.get("constant", (0.0, 0.0, 0.0)))
        self.dense_origin = tuple(kw.get("dense_origin", (0, 0, 0)))
        self.dense_values = kw.get("dense_values")
        self.dense_background = tuple(kw.get("dense_background", (0.0, 0.0, 0.0)))
        self.domain = float(kw.get("domain", 1.0))
        self.period = float(kw.get("period", 1.0))
        self.scale = float(kw.get("scale", 1.0))
        self.omega = tuple(kw.get("omega", (0.0, 0.0, 0.0)))
        self.center = tuple(kw.get("center", (0.0, 0.0, 0.0)))
        self.dense_map_type = int(kw.get("dense_map_type", 0))
        self.dense_voxel_size = float(kw.get("dense_voxel_size", 1.0))
        self.dense_translation = tuple(float(x) for x in kw.get("dense_translation", (0.0, 0.0, 0.0)))
        if self.dense_values is not None:
            self.dense_values = np.ascontiguousarray(self.dense_values, np.float32)
            assert self.dense_values.ndim == 4 and self.dense_values.shape[3] == 3

    @classmethod
    def constant_field(cls, v):
        """DiscreteField over an empty Vec3fGrid whose background is v."""
        return cls(_abi.FIELD_CONSTANT, constant=v)

    @classmethod
    def dense(cls, values, origin=(0, 0, 0), background=(0.0, 0.0, 0.0)):
        """Aligned DiscreteField over a dense Vec3f block values[nx,ny,nz,3]."""
        return cls(_abi.FIELD_DENSE, dense_values=values, dense_origin=origin,
                   dense_background=background)

    @classmethod
    def dense_xform(cls, values, voxel_size, translation=(0.0, 0.0, 0.0), origin=(0, 0, 0),
                    background=(0.0, 0.0, 0.0)):
        """DiscreteField over a dense Vec3f block values[nx,ny,nz,3] in a grid
        with its own transform (uniform scale `voxel_size`, world
        `translation`): sampled trilinearly at each voxel's world position."""
        mt = _abi.MAP_UNIFORM_SCALE_TRANSLATE if any(translation) else _abi.MAP_UNIFORM_SCALE
        return cls(_abi.FIELD_DENSE, dense_values=values, dense_origin=origin, dense_background=background,
                   dense_map_type=1 + mt, dense_voxel_size=voxel_size, dense_translation=translation)

    @classmethod
    def host_sampled(cls, fn):
        """Any velocity functor (the reference's FieldT), sampled on the host
        once per CFL substep: fn(ijk, t) receives the index coordinates of
        the active voxels, an (n, 3) int32 array in the reference's order,
        and returns their (n, 3) velocities in index space per time unit.
        An exception inside fn leaves the velocities of that substep at 0
        (ctypes reports it on stderr)."""
        f = cls(_abi.FIELD_HOST_SAMPLED)

        def sample(user, n, ijk, t, vel):
            if n <= 0:
                return
            a = np.ctypeslib.as_array(ijk, shape=(n, 3))
            out = np.ctypeslib.as_array(vel, shape=(n, 3))
            out[...] = np.asarray(fn(a, float(t)), np.float32).reshape(n, 3)

        f._sampler = _abi.HOST_SAMPLE(sample)
        f._sampler_ptr = C.cast(f._sampler, C.c_void_p).value
        return f

    @classmethod
    def enright(cls, voxel_size=1.0, translation=(0.0, 0.0, 0.0)):
        """The reference's default field, tools::EnrightField<float>
        (tools/VelocityFields.h:101-141), sampled on the host by the
        library's gbls_host_sample_enright at each voxel's world position
        (index * voxel_size + translation, in double).  voxel_size and
        translation must be the level set's map exactly: a grid made with a
        float voxel size (gbls_host_sphere, the reference's
        createLevelSetSphere) holds that float widened to double, so pass
        the grid's own voxel_size rather than a decimal literal."""
        from ._lib import lib
        f = cls(_abi.FIELD_HOST_SAMPLED)
        f._map = _abi.HostMap()
        f._map.scale = float(voxel_size)
        f._map.translation[:] = [float(x) for x in translation]
        f._sampler_ptr = C.cast(lib().gbls_host_sample_enright, C.c_void_p).value
        f._user_ptr = C.addressof(f._map)
        return f

    @classmethod
    def deformation(cls, domain=1024.0, period=100.0, scale=1.0):
        return cls(_abi.FIELD_DEFORMATION, domain=domain, period=period, scale=scale)

    @classmethod
    def rotation(cls, constant, omega, center):
        return cls(_abi.FIELD_ROTATION, constant=constant, omega=omega, center=center)

    def desc(self):
        d = _abi.FieldDesc()
        d.kind = self.kind
        d.constant[:] = self.constant
        d.dense_origin[:] = self.dense_origin
        if self.dense_values is not None:
            d.dense_dims[:] = self.dense_values.shape[:3]
            d.dense_values = self.dense_values.ctypes.data_as(C.POINTER(C.c_float))
        d.dense_background[:] = self.dense_background
        d.domain = self.domain
        d.period = self.period
        d.scale = self.scale
        d.omega[:] = self.omega
        d.center[:] = self.center
        d.dense_map_type = self.dense_map_type
        d.dense_voxel_size = self.dense_voxel_size
        d.dense_translation[:] = self.dense_translation
        d.host_sample = getattr(self, "_sampler_ptr", None)
        d.host_user = getattr(self, "_user_ptr", None)
        return d
