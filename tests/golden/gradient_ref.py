"""FP64 reference gradients of an advection loss, for the adjoint tests.

The loss is L(phi0, v) = sum over the final band of (phi_T - target)^2,
phi_T the level set after HJWENO5 + TVD-RK3 advection (tracker TVD-RK1, one
renormalisation) of phi0 through consecutive intervals in a dense velocity
grid v.  Two references come from the oracle (the C++ restatement of the
reference):

* tangent runs (PortGrid precision TANGENT): the FP32 forward map, its values
  bit-identical to the reference, with FP64 derivatives along
  port.tangent_lanes() directions per run carried through the same upwind
  sides, Godunov selections, trims and topology.  The time steps carry
  derivatives too: a CFL-limited substep depends on the velocity through
  max |v|^2, and the last substep of an interval on the substeps before it.
  This is the FP64 reference gradient of the map the adjoint differentiates.
* central differences of the oracle's FP64 run (time in FP64 as well) with
  the band of the tangent run imposed on every trim (replay_topology): a
  voxel crossing the trimming threshold would make L jump by O(gamma^2), so
  the difference quotient sees only the smooth part of the map.

Probe directions are unit vectors.  A velocity probe is perturbed in the
FP32 grid the field reads, so its direction is the one realised by the two
rounded grids, (v+ - v-) / 2h in FP64.
"""
import numpy as np

from openvdb_gb300 import Field

RK3, RK1 = 2, 0


def unit_rows(x):
    x = np.asarray(x, np.float64)
    n = np.linalg.norm(x.reshape(x.shape[0], -1), axis=1)
    return x / n.reshape((-1,) + (1,) * (x.ndim - 1))


def velocity_probe(vel, direction, h):
    """(v+, v-, realised direction) for a central difference of step h."""
    vp = (vel.astype(np.float64) + h * direction).astype(np.float32)
    vm = (vel.astype(np.float64) - h * direction).astype(np.float32)
    return vp, vm, (vp.astype(np.float64) - vm.astype(np.float64)) / (2.0 * h)


class Problem:
    def __init__(self, template, vel, times, target_fn, cfl=0.0, threads=0):
        from oracle import port
        self.port = port
        self.template = template
        self.vel = np.ascontiguousarray(vel, np.float32)
        self.times = [float(t) for t in times]
        self.target_fn = target_fn
        self.cfl = float(cfl)
        self.threads = threads
        self.source = None  # a tangent run whose trims the differences replay
        self.substeps = None

    def run(self, precision, phi0, vel=None, dphi=None, dv=None, replay=None, record=False):
        g = self.port.PortGrid(self.template, threads=self.threads, precision=precision)
        g.set_active_values(np.asarray(phi0, np.float64))
        if precision == self.port.TANGENT:
            g.set_tangents(np.zeros((1, g.counts().active_voxel_count)) if dphi is None else dphi)
            g.set_velocity_tangent(dv)
        if record:
            g.record_topology()
        if replay is not None:
            g.replay_topology(replay)
        field = Field.dense(self.vel if vel is None else vel)
        n = 0
        for a, b in zip(self.times[:-1], self.times[1:]):
            n += g.advect(field, a, b, temporal=RK3, tracker_temporal=RK1, norm_count=1, cfl=self.cfl)
        return g, n

    def residual(self, g):
        host = g.to_host()
        return g.active_values() - self.target_fn(host.active_coords()), host

    def loss(self, g):
        r, _ = self.residual(g)
        return float(np.dot(r, r))

    def tangents(self, phi0, dphi=None, dv=None):
        """dL/dphi0 . dphi[k] or dL/dv . dv[k] for every row k (FP64)."""
        rows = dphi if dphi is not None else dv
        lanes = self.port.tangent_lanes()
        out = []
        for a in range(0, len(rows), lanes):
            chunk = rows[a:a + lanes]
            g, n = self.run(self.port.TANGENT, phi0, dphi=chunk if dphi is not None else None,
                            dv=chunk if dv is not None else None, record=self.source is None)
            if self.source is None:
                self.source, self.substeps = g, n
            assert n == self.substeps
            r, _ = self.residual(g)
            out.extend(2.0 * (g.active_tangents()[:len(chunk)] @ r))
        return np.array(out)

    def difference(self, phi0, h, dphi=None, vp=None, vm=None):
        """(L(+h) - L(-h)) / 2h of the FP64 run with the tangent run's trims,
        or None when the two runs take other substep counts."""
        assert self.source is not None, "tangents() first"
        phi0 = np.asarray(phi0, np.float64)
        Ls = []
        for sgn, v in ((1.0, vp), (-1.0, vm)):
            p = phi0 + sgn * h * dphi if dphi is not None else phi0
            g, n = self.run(64, p, vel=v, replay=self.source)
            if n != self.substeps or g.topology_count() != self.source.topology_count():
                return None
            Ls.append(self.loss(g))
        return (Ls[0] - Ls[1]) / (2.0 * h)


def relative_errors(x, ref, gnorm, n):
    """|x - ref| against max(|ref|, a tenth of the typical |g . d| of a unit
    direction d in n dimensions, |g| / sqrt(n))."""
    floor = 0.1 * gnorm / np.sqrt(n)
    return np.abs(np.asarray(x) - ref) / np.maximum(np.abs(ref), max(floor, 1e-300))
