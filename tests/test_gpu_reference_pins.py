"""The reference's own known-answer checks for this path, restated and
applied to the device output:

* tracker resize (openvdb/unittest/TestTools.cc:233-284): a sphere with
  FIRST_BIAS / TVD_RK1 tracker; resize() keeps half width 3 and returns false;
  resize(4) returns true, sets the background to 4 dx exactly, keeps active
  values within +-(gamma + dx) and the first-order Godunov |grad phi| within
  [0.4, 1.1] (tools::CheckRange, tools::CheckNormGrad, tools/Diagnostics.h);
* morphing statistics (TestTools.cc:378-420): a sphere morphed into an
  offset sphere with HJWENO5 / TVD_RK3 and a TVD_RK2 tracker for t < 0.05/dx
  in steps of 0.1 ends with invDx*(phi - target) within +-0.5 and a mean
  within 0.02 over the active voxels of both grids.

The same checks run on the reference's own output (the compiled reference,
where it was built) so that the restated checks are themselves pinned.
"""
import numpy as np
import pytest

from oracle import refpy

from openvdb_gb300 import DeviceLevelSet, LevelSetMorphing, LevelSetTracker, fixtures
from openvdb_gb300._abi import FIRST_BIAS, HJWENO5_BIAS, MODE_PARITY, TVD_RK1, TVD_RK2, TVD_RK3


def dense_values(g, lo, hi):
    """Values of host grid g (ValueAccessor::getValue) on the index box [lo, hi)."""
    lo, hi = np.asarray(lo), np.asarray(hi)
    shape = tuple(hi - lo)
    out = np.full(shape, g.background, np.float32)
    ax = [np.arange(lo[a], hi[a]) for a in range(3)]
    # upper-node tiles, then lower-node tiles, then leaves (finer levels override)
    for origins, tiles, dim, child in ((g.upper_origins, g.upper_tiles, 4096, 128),
                                       (g.lower_origins, g.lower_tiles, 128, 8)):
        n = dim // child
        for o, t in zip(origins, tiles.reshape(len(origins), -1)):
            sel = [(ax[a] >= o[a]) & (ax[a] < o[a] + dim) for a in range(3)]
            if not all(s.any() for s in sel):
                continue
            ix = [(ax[a][sel[a]] - o[a]) // child for a in range(3)]
            idx = (ix[0][:, None, None] * n + ix[1][None, :, None]) * n + ix[2][None, None, :]
            vals = t[idx]
            block = out[np.ix_(sel[0], sel[1], sel[2])]
            out[np.ix_(sel[0], sel[1], sel[2])] = np.where(vals != 0.0, vals, block)
    for o, v in zip(g.leaf_origins, g.leaf_values.reshape(-1, 8, 8, 8)):
        s = [slice(o[a] - lo[a], o[a] - lo[a] + 8) for a in range(3)]
        if all(0 <= o[a] - lo[a] and o[a] + 8 <= hi[a] for a in range(3)):
            out[s[0], s[1], s[2]] = v
    return out


def box_of(*grids, pad=2):
    o = np.concatenate([g.leaf_origins for g in grids])
    return o.min(0) - pad - 8, o.max(0) + 8 + pad + 8


def norm_grad_sqrd(g, dx):
    """invdx2 * ISGradientNormSqrd<FIRST_BIAS> at every active voxel
    (tools::CheckNormGrad, tools/Diagnostics.h:428-487; the Godunov norm of
    one-sided first differences, math/Operators.h)."""
    lo, hi = box_of(g)
    v = dense_values(g, lo, hi)
    coords = g.active_coords() - lo
    c = v[coords[:, 0], coords[:, 1], coords[:, 2]]
    out = c > 0
    nsq = np.zeros_like(c)
    for a in range(3):
        e = np.zeros(3, int)
        e[a] = 1
        p, m = coords + e, coords - e
        dp = v[p[:, 0], p[:, 1], p[:, 2]] - c
        dm = c - v[m[:, 0], m[:, 1], m[:, 2]]
        am = np.where(out, np.maximum(dm, 0), np.minimum(dm, 0))
        ap = np.where(out, np.minimum(dp, 0), np.maximum(dp, 0))
        nsq = nsq + np.maximum(am * am, ap * ap)
    return np.float32(1.0 / dx ** 2) * nsq


SPHERE128 = dict(radius=0.15, center=(0.35, 0.35, 0.35), dx=1.0 / (128 - 1))
SPHERE64 = dict(radius=0.15, c1=(0.35, 0.35, 0.35), c2=(0.4, 0.4, 0.4), dx=1.0 / (64 - 1))


def check_resize(resize, host, half_width, dx):
    """TestTools.cc:240-283 on a tracker given as callables."""
    gamma = np.float32(3.0) * np.float32(dx)
    assert np.float32(host().background) == gamma and half_width() == 3.0
    assert not resize(3)
    g = host()
    act = g.active_values()
    assert act.min() >= -gamma and act.max() <= gamma
    ng2 = norm_grad_sqrd(g, dx)
    assert ng2.min() >= np.float32(0.9) ** 2 and ng2.max() <= np.float32(1.1) ** 2, (ng2.min(), ng2.max())
    assert resize(4)
    g = host()
    assert np.float32(g.background) == np.float32(4 * np.float32(dx)) and half_width() == 4.0
    act = g.active_values()
    lim = np.float32(gamma + np.float32(dx))
    assert act.min() >= -lim and act.max() <= lim
    ng2 = norm_grad_sqrd(g, dx)
    assert ng2.min() >= np.float32(0.4) ** 2 and ng2.max() <= np.float32(1.1) ** 2, (ng2.min(), ng2.max())


def morph_loop(step_fn, empty, dx):
    """for (t = 0, dt = 0.1f; !empty && t < 0.05f/dx; t += dt) advect(t, t + dt)."""
    t_max = np.float32(0.05) / np.float32(dx)
    t, dt = np.float32(0.0), np.float32(0.1)
    n = 0
    while not empty() and t < t_max:
        step_fn(float(t), float(np.float32(t + dt)))
        t = np.float32(t + dt)
        n += 1
    return n


def check_morph(g, target, dx):
    """TestTools.cc:405-417: math::Stats of invDx*(phi - target(ijk))."""
    lo, hi = box_of(g, target)
    tv = dense_values(target, lo, hi)
    cs = g.active_coords() - lo
    ct = target.active_coords() - lo
    inv = np.float32(1.0 / np.float32(dx))
    s = np.concatenate([inv * (g.active_values() - tv[cs[:, 0], cs[:, 1], cs[:, 2]]),
                        inv * (target.active_values() - tv[ct[:, 0], ct[:, 1], ct[:, 2]])])
    s = s.astype(np.float64)
    assert abs(s.min()) <= 0.5 and abs(s.max()) <= 0.5 and abs(s.mean()) <= 0.02, \
        (s.min(), s.max(), s.mean())
    return s.min(), s.max(), s.mean()


@pytest.mark.gpu
def test_tracker_resize_pins():
    c = SPHERE128
    dev = DeviceLevelSet(fixtures.sphere(c["radius"], c["center"], c["dx"], 3.0))
    dev.set_precision(MODE_PARITY)
    tr = LevelSetTracker(dev)
    tr.setSpatialScheme(FIRST_BIAS)
    tr.setTemporalScheme(TVD_RK1)
    check_resize(tr.resize, dev.to_host, tr.getHalfWidth, c["dx"])


@pytest.mark.gpu
def test_morph_statistics_pins():
    c = SPHERE64
    source = fixtures.sphere(c["radius"], c["c1"], c["dx"], 3.0)
    target = fixtures.sphere(c["radius"], c["c2"], c["dx"], 3.0)
    dev, tgt = DeviceLevelSet(source), DeviceLevelSet(target)
    dev.set_precision(MODE_PARITY)
    m = LevelSetMorphing(dev, tgt)
    m.setSpatialScheme(HJWENO5_BIAS)
    m.setTemporalScheme(TVD_RK3)
    m.setTrackerSpatialScheme(HJWENO5_BIAS)
    m.setTrackerTemporalScheme(TVD_RK2)
    assert morph_loop(m.advect, lambda: dev.leaf_count() == 0, c["dx"]) == 32
    print("morph statistics min %.4f max %.4f avg %.5f" % check_morph(dev.to_host(), target, c["dx"]))


needs_ref = pytest.mark.skipif(not refpy.available(), reason="compiled reference not built here")


@needs_ref
def test_reference_resize_pins():
    """The restated resize checks hold on the reference tracker's own output."""
    c = SPHERE128
    ref = refpy.RefGrid.sphere(c["radius"], c["center"], c["dx"], 3.0)
    kw = dict(spatial=FIRST_BIAS, temporal=TVD_RK1)
    check_resize(lambda n: ref.resize(n, **kw), ref.to_host,
                 lambda: float(np.float32(ref.to_host().background) / np.float32(c["dx"])), c["dx"])


@needs_ref
def test_reference_morph_pins():
    """The restated morph statistics hold on the reference morph's own output."""
    c = SPHERE64
    src = refpy.RefGrid.sphere(c["radius"], c["c1"], c["dx"], 3.0)
    tgt = refpy.RefGrid.sphere(c["radius"], c["c2"], c["dx"], 3.0)
    kw = dict(spatial=HJWENO5_BIAS, temporal=TVD_RK3, tracker_spatial=HJWENO5_BIAS,
              tracker_temporal=TVD_RK2)
    assert morph_loop(lambda a, b: src.morph(tgt, a, b, **kw), lambda: src.counts().leaf_count == 0,
                      c["dx"]) == 32
    check_morph(src.to_host(), tgt.to_host(), c["dx"])
