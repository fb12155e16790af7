"""Reverse-mode derivatives of level-set advection (gbls_adjoint_*) and a
torch.autograd.Function around them.

The forward pass is LevelSetAdvection::advect (HJWENO5 + TVD-RK3, tracker
TVD-RK1 with one renormalisation) with recording enabled; the backward pass
runs the recorded substeps in reverse with the topology, upwind directions,
Godunov branches, trimming and CFL time steps held at their forward values.
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
        self.dev = DeviceLevelSet(g)
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
        return AdvectionTape(grid, self.velocity, self.origin, self.background, self.mode, self.cfl, field=self.field)

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
            _, g = tape.forward(g.active_values(), seg, record=False)
            self.substeps += sum(tape.substeps)
            self.voxel_updates += tape.dev.stats()["voxel_updates"]
            tape.dev.close()
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
            tape.forward(g.active_values(), seg, record=True)
            recorded += sum(tape.substeps)
            self.recorded_voxel_updates += tape.dev.stats()["voxel_updates"]
            lam = tape.backward_accumulate(lam, dvel)
            tape.dev.close()
        return lam, dvel, recorded


def make_autograd_function():
    """torch.autograd.Function: (phi0 active values, dense velocity) -> phi_final."""
    import torch

    class LevelSetAdvect(torch.autograd.Function):
        @staticmethod
        def forward(ctx, phi0, velocity, tape, times):
            tape.set_velocity(velocity.detach().cpu().numpy())
            out, _ = tape.forward(phi0.detach().cpu().numpy(), times)
            ctx.tape = tape
            return torch.from_numpy(out).to(phi0.device)

        @staticmethod
        def backward(ctx, grad_out):
            d0, dv = ctx.tape.backward(grad_out.detach().cpu().numpy())
            dev = grad_out.device
            return torch.from_numpy(d0).to(dev), torch.from_numpy(dv).to(dev), None, None

    return LevelSetAdvect
