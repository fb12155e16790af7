"""Velocity-field descriptions (gbls_field_desc) for the advection entry point.

The reference advects in any functor with operator()(Coord, t)
(tools/LevelSetAdvect.h:32-52).  The kinds here cover the reference's
DiscreteField (tools/VelocityFields.h:42-94), aligned or with its own
transform (trilinear BoxSampler), plus two
analytic fields whose arithmetic is defined in include/gbls_fields.h.
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
        return d
