"""Reverse-mode derivatives of level-set advection (gbls_adjoint_*) and a
torch.autograd.Function around them.

The forward pass is LevelSetAdvection::advect (HJWENO5 + TVD-RK3, tracker
TVD-RK1 with one renormalisation) with recording enabled; the backward pass
runs the recorded substeps in reverse with the topology, upwind directions,
Godunov branches and trimming held at their forward values, and with the
CFL time steps' dependence on the velocity carried.
Inputs: the active values of the initial level set (canonical order) and a
dense velocity grid; output: the active values after advection.
"""
import ctypes as C

import numpy as np

from . import _abi
from ._lib import lib
from .fields import Field
from .levelset import PARITY, TVD_RK1, TVD_RK3, DeviceField, DeviceLevelSet, LevelSetAdvection, _call

_declared = False


def _declare():
    global _declared
    if _declared:
        return
    L = lib()
    vp = C.c_void_p
    L.gbls_adjoint_record.argtypes = [vp, C.c_int]
    L.gbls_adjoint_record.restype = C.c_int
    L.gbls_adjoint_sizes.argtypes = [vp] + [C.POINTER(C.c_int64)] * 3
    L.gbls_adjoint_sizes.restype = C.c_int
    P = C.POINTER(C.c_float)
    L.gbls_adjoint_backward.argtypes = [vp, vp, P, P, P]
    L.gbls_adjoint_backward.restype = C.c_int
    L.gbls_adjoint_backward_accumulate.argtypes = [vp, vp, P, P, vp]
    L.gbls_adjoint_backward_accumulate.restype = C.c_int
    L.gbls_adjoint_backward_device.argtypes = [vp, vp, vp, vp, vp]
    L.gbls_adjoint_backward_device.restype = C.c_int
    L.gbls_get_active_values_device.argtypes = [vp, vp]
    L.gbls_get_active_values_device.restype = C.c_int
    L.gbls_set_active_values_device.argtypes = [vp, vp]
    L.gbls_set_active_values_device.restype = C.c_int
    L.gbls_field_set_dense_device.argtypes = [vp, vp, vp]
    L.gbls_field_set_dense_device.restype = C.c_int
    L.gbls_set_stream.argtypes = [vp, vp]
    L.gbls_set_stream.restype = C.c_int
    _declared = True


def with_active_values(template, values):
    """Copy of a HostGrid whose active voxels (canonical order) take `values`."""
    g = template.copy()
    m = g.active_mask_bool()
    v = g.leaf_values.copy()
    v[m] = np.asarray(values, np.float32).reshape(-1)
    g.leaf_values = v
    return g


class AdvectionTape:
    """Advect a level set with recording; then pull gradients back."""

    def __init__(self, template, velocity, origin=(0, 0, 0), background=(0.0, 0.0, 0.0),
                 mode=PARITY, cfl=0.0, field=None):
        """`field`: an existing DeviceField of `velocity` to share (not re-uploaded)."""
        _declare()
        self.template = template
        self.origin = tuple(origin)
        self.background = tuple(background)
        self.mode = mode
        self.cfl = cfl
        if field is not None:
            self.velocity = velocity
            self.field = field
        else:
            self.set_velocity(velocity)
        self.dev = None

    def set_velocity(self, velocity):
        self.velocity = np.ascontiguousarray(velocity, np.float32)
        self.field = DeviceField(Field.dense(self.velocity, self.origin, self.background))

    def forward(self, phi0, times, record=True):
        """Advect the template with active values phi0 through consecutive
        intervals times[k] -> times[k+1]; returns (phi_final, final HostGrid)."""
        g = with_active_values(self.template, phi0)
        if self.dev is None:
            self.dev = DeviceLevelSet(g)
        else:
            self.dev.upload(g)  # keeps the handle's allocations and its tape's arrays
        self.dev.set_precision(self.mode)
        adv = LevelSetAdvection(self.dev, self.field)
        adv.setTemporalScheme(TVD_RK3)
        adv.setTrackerTemporalScheme(TVD_RK1)
        adv.setNormCount(1)
        adv.cfl = self.cfl
        _call(lib().gbls_adjoint_record(self.dev.handle, 1 if record else 0))
        self.substeps = [adv.advect(times[k], times[k + 1]) for k in range(len(times) - 1)]
        out = self.dev.to_host()
        return out.active_values().copy(), out

    def backward(self, dl_final):
        """dL/dphi_final -> (dL/dphi0, dL/dvelocity)."""
        n0, nf, ns = C.c_int64(), C.c_int64(), C.c_int64()
        _call(lib().gbls_adjoint_sizes(self.dev.handle, C.byref(n0), C.byref(nf), C.byref(ns)))
        dlf = np.ascontiguousarray(dl_final, np.float32).reshape(-1)
        assert dlf.size == nf.value, (dlf.size, nf.value)
        d0 = np.zeros(n0.value, np.float32)
        dv = np.zeros_like(self.velocity)
        P = C.POINTER(C.c_float)
        _call(lib().gbls_adjoint_backward(self.dev.handle, self.field._h, dlf.ctypes.data_as(P),
                                          d0.ctypes.data_as(P), dv.ctypes.data_as(P)))
        return d0, dv

    def backward_accumulate(self, dl_final, dvel):
        """dL/dphi_final -> dL/dphi0 (host); dL/dvelocity is added into `dvel`, a
        float32 CUDA tensor of the velocity grid's shape on the tape's device."""
        n0, nf, ns = C.c_int64(), C.c_int64(), C.c_int64()
        _call(lib().gbls_adjoint_sizes(self.dev.handle, C.byref(n0), C.byref(nf), C.byref(ns)))
        dlf = np.ascontiguousarray(dl_final, np.float32).reshape(-1)
        assert dlf.size == nf.value, (dlf.size, nf.value)
        assert dvel.is_cuda and dvel.dtype.is_floating_point and dvel.is_contiguous()
        d0 = np.zeros(n0.value, np.float32)
        P = C.POINTER(C.c_float)
        _call(lib().gbls_adjoint_backward_accumulate(self.dev.handle, self.field._h, dlf.ctypes.data_as(P),
                                                     d0.ctypes.data_as(P), C.c_void_p(dvel.data_ptr())))
        return d0


class DeviceTape:
    """AdvectionTape with every array on the device: the initial values,
    the velocity grid, the final values and both gradients are CUDA tensors,
    and the handle runs on torch's current stream.  The template's topology
    is uploaded once per forward (it is the advected object, not data)."""

    def __init__(self, template, shape, origin=(0, 0, 0), background=(0.0, 0.0, 0.0), mode=PARITY, cfl=0.0,
                 device=0):
        _declare()
        self.template = template
        self.mode = mode
        self.cfl = cfl
        self.device = device
        self.shape = tuple(shape)
        # the field object: a dense grid of this shape whose values the
        # forward pass replaces on the device
        self.field = DeviceField(Field.dense(np.zeros(self.shape, np.float32), origin, background))
        self.dev = DeviceLevelSet(template, device=device)
        self.dev.set_precision(mode)
        self.substeps = []

    def _stream(self):
        import torch
        return C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def forward(self, phi0, velocity, times, record=True):
        """phi0: float32 CUDA tensor of the template's active values;
        velocity: float32 CUDA tensor of `shape`.  Returns phi_T (CUDA)."""
        import torch
        assert phi0.is_cuda and phi0.dtype == torch.float32 and phi0.is_contiguous()
        assert velocity.is_cuda and velocity.dtype == torch.float32 and tuple(velocity.shape) == self.shape
        velocity = velocity.contiguous()
        s = self._stream()
        _call(lib().gbls_field_set_dense_device(self.field._h, C.c_void_p(velocity.data_ptr()), s))
        self.dev.upload(self.template)
        _call(lib().gbls_set_stream(self.dev.handle, s))
        _call(lib().gbls_set_active_values_device(self.dev.handle, C.c_void_p(phi0.data_ptr())))
        adv = LevelSetAdvection(self.dev, self.field)
        adv.setTemporalScheme(TVD_RK3)
        adv.setTrackerTemporalScheme(TVD_RK1)
        adv.setNormCount(1)
        adv.cfl = self.cfl
        _call(lib().gbls_adjoint_record(self.dev.handle, 1 if record else 0))
        self.substeps = [adv.advect(times[k], times[k + 1]) for k in range(len(times) - 1)]
        out = torch.empty(self.dev.active_voxel_count(), dtype=torch.float32, device=phi0.device)
        _call(lib().gbls_get_active_values_device(self.dev.handle, C.c_void_p(out.data_ptr())))
        return out

    def backward(self, dl_final):
        """dL/dphi_T (CUDA tensor) -> (dL/dphi0, dL/dvelocity), CUDA tensors."""
        import torch
        n0, nf, ns = C.c_int64(), C.c_int64(), C.c_int64()
        _call(lib().gbls_adjoint_sizes(self.dev.handle, C.byref(n0), C.byref(nf), C.byref(ns)))
        dlf = dl_final.detach().to(torch.float32).contiguous()
        assert dlf.is_cuda and dlf.numel() == nf.value, (dlf.numel(), nf.value)
        d0 = torch.empty(n0.value, dtype=torch.float32, device=dlf.device)
        dv = torch.zeros(self.shape, dtype=torch.float32, device=dlf.device)
        _call(lib().gbls_set_stream(self.dev.handle, self._stream()))
        _call(lib().gbls_adjoint_backward_device(self.dev.handle, self.field._h, C.c_void_p(dlf.data_ptr()),
                                                 C.c_void_p(d0.data_ptr()), C.c_void_p(dv.data_ptr())))
        return d0, dv


class CheckpointedAdvection:
    """Adjoint of a long advection with checkpoints: the forward pass keeps the
    level set only at the start of every segment of `every` intervals (host
    grids); the reverse sweep re-runs each segment with recording, from the
    last to the first, and pulls dL/dphi back through it while dL/dv
    accumulates on the device.  Memory: one segment's tape plus the
    checkpoints, instead of the tape of the whole horizon."""

    def __init__(self, template, velocity, every=10, origin=(0, 0, 0), background=(0.0, 0.0, 0.0),
                 mode=PARITY, cfl=0.0):
        _declare()
        self.template = template
        self.every = int(every)
        self.origin = tuple(origin)
        self.background = tuple(background)
        self.mode = mode
        self.cfl = cfl
        self.set_velocity(velocity)

    def set_velocity(self, velocity):
        self.velocity = np.ascontiguousarray(velocity, np.float32)
        self.field = DeviceField(Field.dense(self.velocity, self.origin, self.background))

    def _tape(self, grid):
        """One tape (one device handle) serves every segment in turn, always
        with the current velocity field."""
        if getattr(self, "_shared", None) is None:
            self._shared = AdvectionTape(grid, self.velocity, self.origin, self.background, self.mode, self.cfl,
                                         field=self.field)
        self._shared.template = grid
        self._shared.velocity = self.velocity
        self._shared.field = self.field
        return self._shared

    def forward(self, phi0, times):
        """Advect through times[0] -> times[-1]; returns (phi_final, final HostGrid)."""
        self.times = list(times)
        self.segments = []  # (start grid, its times)
        self.substeps = 0
        self.voxel_updates = 0
        g = with_active_values(self.template, phi0)
        for a in range(0, len(self.times) - 1, self.every):
            seg = self.times[a:a + self.every + 1]
            self.segments.append((g, seg))
            tape = self._tape(g)
            before = tape.dev.stats()["voxel_updates"] if tape.dev is not None else 0
            _, g = tape.forward(g.active_values(), seg, record=False)
            self.substeps += sum(tape.substeps)
            self.voxel_updates += tape.dev.stats()["voxel_updates"] - before
        return g.active_values().copy(), g

    def backward(self, dl_final, dvel=None):
        """dL/dphi_final -> (dL/dphi0, dL/dv as a CUDA tensor, recorded substeps)."""
        import torch
        if dvel is None:
            dvel = torch.zeros(self.velocity.shape, dtype=torch.float32, device="cuda")
        lam = np.asarray(dl_final, np.float32)
        recorded = 0
        self.recorded_voxel_updates = 0
        for g, seg in reversed(self.segments):
            tape = self._tape(g)
            before = tape.dev.stats()["voxel_updates"] if tape.dev is not None else 0
            tape.forward(g.active_values(), seg, record=True)
            recorded += sum(tape.substeps)
            self.recorded_voxel_updates += tape.dev.stats()["voxel_updates"] - before
            lam = tape.backward_accumulate(lam, dvel)
        return lam, dvel, recorded


def make_autograd_function():
    """torch.autograd.Function (phi0, velocity, tape, times) -> phi_T, with
    phi0 the template's active values and velocity the dense grid, both
    float32 CUDA tensors, and tape a DeviceTape: forward and backward stay on
    the device (gbls_set_active_values_device, gbls_adjoint_backward_device)."""
    import torch

    class LevelSetAdvect(torch.autograd.Function):
        @staticmethod
        def forward(ctx, phi0, velocity, tape, times):
            out = tape.forward(phi0.detach(), velocity.detach(), times, record=True)
            ctx.tape = tape
            return out

        @staticmethod
        def backward(ctx, grad_out):
            d0, dv = ctx.tape.backward(grad_out)
            return d0, dv, None, None

    return LevelSetAdvect
