"""The double-word WENO5 of the PARITY kernels against the reference formula (CPU).

The PARITY kernels evaluate math::WENO5<float> (math/FiniteDifference.h:301-321),
whose weights the reference computes in FP64, as double-word FP32 pairs with
an error bound (openvdb_gb300/csrc/weno_exact.h): where the bound decides the
rounding the result must be the reference's float bit for bit; the rest (a
small fraction) goes to the FP64 formula.  The oracle's restatement of the
formula is the reference here (pinned against the compiled reference through
the golden digests).  Inputs: seeded operand distributions of the stencil —
uniform differences, differences of float sphere distances clamped to the
band, smooth slopes, zeros with jumps and tiny values, and clamped random
walks.
"""
import ctypes as C

import numpy as np
import pytest

from openvdb_gb300 import _lib

port = pytest.importorskip("oracle.port")
if not port.available():
    pytest.skip("oracle port not built", allow_module_level=True)


def _exact(v):
    v = np.ascontiguousarray(v, np.float32)
    out = np.empty(v.shape[0], np.float32)
    dec = np.empty(v.shape[0], np.uint8)
    P = C.POINTER
    rc = _lib.lib().gbls_host_weno5_exact(v.shape[0], v.ctypes.data_as(P(C.c_float)),
                                          out.ctypes.data_as(P(C.c_float)), dec.ctypes.data_as(P(C.c_uint8)))
    assert rc == 0
    return out, dec.astype(bool)


def _inputs(kind, n, rng):
    if kind == "uniform":
        return rng.uniform(-1.0, 1.0, (n, 5)).astype(np.float32)
    if kind == "sphere_lines":
        # seven values along an axis through points near a sphere surface,
        # float distances clamped to the band +-3, then the FD operand order
        R = rng.uniform(5.0, 105.0, n)
        c = rng.uniform(-10.0, 10.0, (n, 3))
        d = rng.normal(size=(n, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        p = np.rint(c + d * (R + rng.uniform(-3.0, 3.0, n))[:, None])
        ax = rng.integers(0, 3, n)
        phi = np.empty((n, 7), np.float32)
        for k in range(7):
            q = p.copy()
            q[np.arange(n), ax] += k - 3
            phi[:, k] = np.clip((np.linalg.norm(q - c, axis=1) - R).astype(np.float32), -3.0, 3.0)
        D = np.diff(phi, axis=1)
        return np.concatenate([D[:, ::-1][:, :5], D[:, :5]]).astype(np.float32)
    if kind == "smooth":
        k = np.arange(5)
        a, b, c = rng.uniform(-1, 1, n), 1e-2 * rng.uniform(-1, 1, n), 1e-3 * rng.uniform(-1, 1, n)
        return (a[:, None] + b[:, None] * k + c[:, None] * k * k + 1e-7 * rng.uniform(-1, 1, (n, 5))).astype(np.float32)
    if kind == "zeros_jumps":
        r = rng.integers(0, 4, (n, 5))
        v = np.where(r == 1, 3.0 * rng.uniform(-1, 1, (n, 5)),
                     np.where(r == 2, 1e-7 * rng.uniform(-1, 1, (n, 5)), rng.uniform(-1, 1, (n, 5))))
        v[r == 0] = 0.0
        v[: n // 50] = 0.0  # all five zero: signed-zero results
        v[: n // 100] *= -1.0
        return v.astype(np.float32)
    if kind == "walks":
        base = rng.uniform(-3, 3, n).astype(np.float32)
        steps = rng.uniform(-0.2, 0.2, (n, 6)).astype(np.float32)
        phi = np.clip(base[:, None] + np.cumsum(steps, axis=1), -3.0, 3.0).astype(np.float32)
        return np.diff(phi, axis=1).astype(np.float32)
    raise ValueError(kind)


@pytest.mark.parametrize("kind", ["uniform", "sphere_lines", "smooth", "zeros_jumps", "walks"])
def test_exact_weno5_matches_reference(kind):
    rng = np.random.Generator(np.random.PCG64(20261204))
    v = _inputs(kind, 400_000, rng)
    ref = port.weno5(v)
    got, dec = _exact(v)
    bad = np.nonzero(dec & (got.view(np.uint32) != ref.view(np.uint32)))[0]
    assert bad.size == 0, "decided results differ from the reference: %s" % [
        (v[i].tolist(), float(got[i]), float(ref[i])) for i in bad[:5]]
    undecided = 1.0 - dec.mean()
    print("%s: %d evaluations, %.2e left to FP64" % (kind, v.shape[0], undecided))
    assert undecided < 2e-3


@pytest.mark.parametrize("kind", ["uniform", "sphere_lines", "smooth", "zeros_jumps", "walks"])
def test_weno5_sign_is_certain(kind):
    """Where weno5_sign certifies a sign, the reference's result has it (a
    zero of either sign counts for both)."""
    rng = np.random.Generator(np.random.PCG64(7))
    v = _inputs(kind, 200_000, rng)
    ref = port.weno5(v)
    sign = np.empty(v.shape[0], np.int8)
    P = C.POINTER
    assert _lib.lib().gbls_host_weno5_sign(v.shape[0], v.ctypes.data_as(P(C.c_float)),
                                           sign.ctypes.data_as(P(C.c_int8))) == 0
    assert not np.any((sign == 1) & (ref < 0)), "certified >= 0 but negative"
    assert not np.any((sign == -1) & (ref > 0)), "certified <= 0 but positive"
    assert not np.any((sign == 2) & (ref != 0)), "certified zero but not zero"
    assert np.array_equal(sign == 2, np.all(v == 0, axis=1)), "a zero certificate other than five zero operands"
    print("%s: sign certified for %.1f%%" % (kind, 100.0 * np.mean(sign != 0)))


@pytest.mark.parametrize("kind", ["uniform", "sphere_lines", "smooth", "zeros_jumps", "walks"])
def test_weno5_sign_pair_is_certain(kind):
    """The renormalisation's certificate for a line's backward (D0..D4) and
    forward (D5..D1) operands at once: every certified sign agrees with the
    reference's result, zeros are certified exactly for five zero operands,
    and it certifies as often as two separate certificates."""
    rng = np.random.Generator(np.random.PCG64(11))
    v = _inputs(kind, 200_000, rng)
    # lines of six differences: five operands and one more of the same kind
    d = np.ascontiguousarray(np.concatenate([v, np.roll(v[:, :1], 1, axis=0)], axis=1), np.float32)
    bd = np.ascontiguousarray(d[:, :5])
    fd = np.ascontiguousarray(d[:, [5, 4, 3, 2, 1]])
    sb = np.empty(d.shape[0], np.int8)
    sf = np.empty(d.shape[0], np.int8)
    P = C.POINTER
    assert _lib.lib().gbls_host_weno5_sign_pair(d.shape[0], d.ctypes.data_as(P(C.c_float)),
                                                sb.ctypes.data_as(P(C.c_int8)), sf.ctypes.data_as(P(C.c_int8))) == 0
    for ops, sign in ((bd, sb), (fd, sf)):
        ref = port.weno5(ops)
        assert not np.any((sign == 1) & (ref < 0)), "certified >= 0 but negative"
        assert not np.any((sign == -1) & (ref > 0)), "certified <= 0 but positive"
        assert not np.any((sign == 2) & (ref != 0)), "certified zero but not zero"
        assert np.array_equal(sign == 2, np.all(ops == 0, axis=1))
        single = np.empty(ops.shape[0], np.int8)
        assert _lib.lib().gbls_host_weno5_sign(ops.shape[0], ops.ctypes.data_as(P(C.c_float)),
                                               single.ctypes.data_as(P(C.c_int8))) == 0
        assert abs(np.mean(sign != 0) - np.mean(single != 0)) < 1e-3


@pytest.mark.parametrize("e", [-120, -100, -90, -60, -30, 10, 20, 24, 28, 30, 36, 45, 60, 90])
def test_exact_weno5_scaled_operands(e):
    """Operands scaled by 2^e: far from the level-set range the weights
    reach the subnormal range (large differences) or the candidate sums and
    the numerator approach underflow (tiny ones).  Every decided result is
    still the reference's; the rest go to the FP64 formula."""
    rng = np.random.Generator(np.random.PCG64(200 + e))
    v = np.concatenate([_inputs(k, 60_000, rng) for k in ("uniform", "zeros_jumps", "walks")])
    v = (v * np.float32(2.0 ** e)).astype(np.float32)
    ref = port.weno5(v)
    got, dec = _exact(v)
    bad = np.nonzero(dec & (got.view(np.uint32) != ref.view(np.uint32)))[0]
    assert bad.size == 0, [(v[i].tolist(), float(got[i]), float(ref[i])) for i in bad[:5]]


@pytest.mark.parametrize("e", [-149, -135, -126, -100, -40, 20, 60, 100, 126])
def test_weno5_sign_scaled_operands(e):
    """The sign certificates (single and paired) at operands scaled by 2^e,
    down to subnormal differences: no certified sign contradicts the
    reference's result."""
    rng = np.random.Generator(np.random.PCG64(300 + e))
    v = np.concatenate([_inputs(k, 40_000, rng) for k in ("uniform", "zeros_jumps", "walks", "smooth")])
    v = np.ascontiguousarray((v.astype(np.float64) * 2.0 ** e).astype(np.float32))
    d = np.ascontiguousarray(np.concatenate([v, np.roll(v[:, :1], 1, axis=0)], axis=1), np.float32)
    P = C.POINTER
    sb = np.empty(d.shape[0], np.int8)
    sf = np.empty(d.shape[0], np.int8)
    s1 = np.empty(v.shape[0], np.int8)
    assert _lib.lib().gbls_host_weno5_sign_pair(d.shape[0], d.ctypes.data_as(P(C.c_float)),
                                                sb.ctypes.data_as(P(C.c_int8)), sf.ctypes.data_as(P(C.c_int8))) == 0
    assert _lib.lib().gbls_host_weno5_sign(v.shape[0], v.ctypes.data_as(P(C.c_float)),
                                           s1.ctypes.data_as(P(C.c_int8))) == 0
    for ops, sign in ((np.ascontiguousarray(d[:, :5]), sb), (np.ascontiguousarray(d[:, [5, 4, 3, 2, 1]]), sf), (v, s1)):
        ref = port.weno5(ops)
        assert not np.any((sign == 1) & (ref < 0))
        assert not np.any((sign == -1) & (ref > 0))
        assert not np.any((sign == 2) & (ref != 0))
