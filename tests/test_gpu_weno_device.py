"""The PARITY kernels' WENO5 on the device against the oracle, operand by
operand (gbls_weno5_exact_device): the double-word evaluation of
csrc/weno_exact.h with its rounding-decision bound and the FP64 formula for
the undecided evaluations must give math::WENO5<float>'s float
(math/FiniteDifference.h:301-321) bit for bit on every input, at the
operand distributions of the stencil and scaled far towards underflow and
overflow.  Complements the advection digests, which reach the same code
through whole time steps.
"""
import ctypes as C

import numpy as np
import pytest

from openvdb_gb300 import _lib

torch = pytest.importorskip("torch")
port = pytest.importorskip("oracle.port")
from test_weno_exact import _exact, _inputs  # noqa: E402


def _device(v):
    dv = torch.from_numpy(np.ascontiguousarray(v, np.float32)).cuda()
    out = torch.empty(v.shape[0], dtype=torch.float32, device="cuda")
    dec = torch.empty(v.shape[0], dtype=torch.uint8, device="cuda")
    rc = _lib.lib().gbls_weno5_exact_device(C.c_void_p(dv.data_ptr()), v.shape[0], C.c_void_p(out.data_ptr()),
                                            C.c_void_p(dec.data_ptr()), None)
    assert rc == 0, _lib.lib().gbls_last_error()
    return out.cpu().numpy(), dec.cpu().numpy().astype(bool)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["uniform", "sphere_lines", "smooth", "zeros_jumps", "walks"])
@pytest.mark.parametrize("scale", [1.0, 2.0 ** -60, 2.0 ** 30, 2.0 ** 40, 2.0 ** 60, 1e-30, 1e30])
def test_device_weno5_equals_reference(kind, scale):
    rng = np.random.Generator(np.random.PCG64(1000 + abs(int(np.log2(scale)))))
    v = (_inputs(kind, 500_000, rng) * np.float32(scale)).astype(np.float32)
    ref = port.weno5(v)
    got, dec = _device(v)
    # bit for bit; where the reference's result is a NaN (operands so large
    # that its double weights overflow) any NaN matches
    bad = np.nonzero((got.view(np.uint32) != ref.view(np.uint32)) & ~(np.isnan(got) & np.isnan(ref)))[0]
    assert bad.size == 0, [(v[i].tolist(), float(got[i]), float(ref[i]), bool(dec[i])) for i in bad[:5]]
    # the host evaluation decides the same evaluations up to the reciprocal's
    # last bit (correctly rounded there, the hardware approximation here)
    hv, hdec = _exact(v)
    assert np.mean(dec != hdec) < 1e-4
    if scale == 1.0:
        assert 1.0 - dec.mean() < 2e-3


@pytest.mark.gpu
def test_device_weno5_empty_and_null():
    assert _lib.lib().gbls_weno5_exact_device(None, 0, None, None, None) == 0
    assert _lib.lib().gbls_weno5_exact_device(None, 5, None, None, None) != 0
