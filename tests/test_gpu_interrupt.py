"""The interrupter (util/NullInterrupter.h) on the device path: advect stops
at a substep boundary when wasInterrupted() answers true, returns the
substeps done (tools/LevelSetAdvect.h:350, the loop condition), keeps the
level set valid, and start/end calls stay balanced."""
import pytest

from openvdb_gb300 import PARITY, DeviceLevelSet, Field, LevelSetAdvection, fixtures
from openvdb_gb300.levelset import TVD_RK3
from openvdb_gb300.grid import bitwise_equal


class Stopper:
    def __init__(self, allow):
        self.allow = allow  # wasInterrupted calls answered False before the first True
        self.calls = 0
        self.depth = 0
        self.max_depth = 0
        self.names = []

    def start(self, name):
        self.depth += 1
        self.max_depth = max(self.max_depth, self.depth)
        self.names.append(name)

    def end(self):
        self.depth -= 1

    def wasInterrupted(self, percent=-1):
        self.calls += 1
        return self.calls > self.allow


def _advection(grid, stopper):
    dev = DeviceLevelSet(grid)
    dev.set_precision(PARITY)
    adv = LevelSetAdvection(dev, Field.constant_field((0.9, -0.4, 0.3)), stopper)
    adv.setTemporalScheme(TVD_RK3)
    adv.setNormCount(1)
    return dev, adv


@pytest.mark.gpu
def test_interrupt_before_first_substep_leaves_grid_unchanged():
    g = fixtures.sphere(10.0, (1.0, 2.0, 3.0))
    st = Stopper(allow=0)
    dev, adv = _advection(g, st)
    assert adv.advect(0.0, 2.0) == 0
    assert bitwise_equal(dev.to_host(), g)


@pytest.mark.gpu
def test_interrupt_after_k_substeps():
    g = fixtures.sphere(10.0, (1.0, 2.0, 3.0))
    dev, adv = _advection(g, Stopper(allow=10 ** 9))
    full = adv.advect(0.0, 2.0)
    assert full >= 3
    for k in (1, 2):
        st = Stopper(allow=k)
        dev, adv = _advection(g, st)
        assert adv.advect(0.0, 2.0) == k
        assert st.depth == 0 and st.max_depth >= 1
        assert any("TVD_RK3" in n for n in st.names) and any("Pruning" in n for n in st.names)
        out = dev.to_host()
        assert out.active_voxel_count() > 0 and not bitwise_equal(out, g)
        # the handle stays usable: a new call continues from the stop
        st.allow = 10 ** 9
        assert adv.advect(1.0, 2.0) >= 1
