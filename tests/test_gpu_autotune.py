"""Launch-shape autotuner: every launch configuration gives the same bits
(the shapes change speed only), the tuner picks one from timings of the
current level set and caches it per device and workload class."""
import itertools
import os

import pytest


def _run(cfg):
    from openvdb_gb300 import PARITY, DeviceLevelSet, LevelSetAdvection, Field, autotune, digest, fixtures
    c, r = fixtures.sixty_four_spheres(seed=2024)
    d = DeviceLevelSet(fixtures.union_of_spheres(c[:4], r[:4], 1.0, 3.0))
    d.set_precision(PARITY)
    autotune.apply(d.handle, cfg)
    adv = LevelSetAdvection(d, Field.deformation(domain=1024.0, period=100.0, scale=1.0))
    adv.setTemporalScheme(2)
    adv.setTrackerTemporalScheme(0)
    adv.setNormCount(1)
    adv.cfl = 0.5
    n = adv.advect(0.0, 1.0)
    assert autotune.get(d.handle) == cfg
    return n, digest(d.to_host())


@pytest.mark.gpu
def test_every_launch_configuration_gives_the_same_bits():
    """Every value of every parameter (the others at their defaults), and
    the RK stage's register budgets crossed with its CTAs per leaf."""
    from openvdb_gb300 import autotune
    ref = _run(dict(autotune.DEFAULT))
    cfgs = []
    for name, values in autotune.CANDIDATES.items():
        for v in values:
            if v != autotune.DEFAULT[name]:
                cfgs.append(dict(autotune.DEFAULT, **{name: v}))
    for rk, parts in itertools.product(autotune.CANDIDATES["stencil_min_ctas_rk"], (2, 4)):
        cfgs.append(dict(autotune.DEFAULT, stencil_min_ctas_rk=rk, rk_ctas_per_leaf=parts))
    for cfg in cfgs:
        assert _run(cfg) == ref, cfg


@pytest.mark.gpu
def test_tuner_searches_then_caches(tmp_path, monkeypatch):
    from openvdb_gb300 import PARITY, DeviceLevelSet, Field, autotune, fixtures
    from openvdb_gb300.levelset import DeviceField
    monkeypatch.setenv("GBLS_TUNE_CACHE", str(tmp_path / "launch.json"))
    c, r = fixtures.sixty_four_spheres(seed=2024)
    d = DeviceLevelSet(fixtures.union_of_spheres(c[:8], r[:8], 1.0, 3.0))
    d.set_precision(PARITY)
    f = DeviceField(Field.deformation(domain=1024.0, period=100.0, scale=1.0))
    before = d.to_host()
    res = autotune.tune(d.handle, f._h, PARITY, d.leaf_count(), reps=2)
    assert res["source"] == "search"
    assert len(res["timings_ms"]) == sum(len(v) for v in autotune.CANDIDATES.values())
    assert all(t > 0 for t in res["timings_ms"].values())
    for k, v in res["config"].items():
        assert v in autotune.CANDIDATES[k]
    assert autotune.get(d.handle) == res["config"]
    print("tuned:", res["config"], {k: round(v, 4) for k, v in res["timings_ms"].items()})
    # timing leaves the level set as it was
    from openvdb_gb300 import digest
    assert digest(d.to_host()) == digest(before)
    again = autotune.tune(d.handle, f._h, PARITY, d.leaf_count())
    assert again["source"] == "cache" and again["config"] == res["config"]
    assert os.path.exists(str(tmp_path / "launch.json"))
