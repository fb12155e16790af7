"""The oracle's C++ restatement against the reference's golden digests (CPU)."""
import json
import os

import pytest

from cases import CASES, make_field, make_fixture
from openvdb_gb300.grid import digest, summary

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "parity_cases.json")))

port = pytest.importorskip("oracle.port")
if not port.available():
    pytest.skip("oracle port not built", allow_module_level=True)


def run_port(name, threads=0):
    case, gold = CASES[name], GOLD[name]
    host = make_fixture(case["fixture"])
    g = port.PortGrid(host, threads)
    if case.get("large"):
        # the 11.7 M-voxel benchmark workload: its first two unit steps keep
        # the CPU suite short (the GPU tests cover every step)
        gold = gold[:3]
    field = make_field(case["field"])
    sp, tp, tsp, ttp, nc = case["schemes"]
    trim = 3
    for step, (op, rec) in enumerate(zip(case["ops"], gold[1:]), start=1):
        if op[0] == "state":
            s = op[1]
            nc = s.get("norm_count", nc)
            ttp = s.get("tr_temporal", ttp)
            trim = s.get("trim", trim)
            continue
        kw = dict(spatial=tsp, temporal=ttp, norm_count=nc, trim=trim)
        if op[0] == "advect":
            n = g.advect(field, op[1], op[2], spatial=sp, temporal=tp, tracker_spatial=tsp,
                         tracker_temporal=ttp, norm_count=nc, cfl=case.get("cfl", 0.0))
            assert n == rec["count"], (name, step, n, rec["count"])
        elif op[0] == "track":
            g.track(**kw)
        elif op[0] == "normalize":
            g.normalize(**kw)
        elif op[0] == "prune":
            g.prune(**kw)
        elif op[0] == "dilate":
            g.dilate(op[1], **kw)
        h = g.to_host()
        assert digest(h) == rec["digest"], (name, step, op, summary(h), rec["summary"])


@pytest.mark.parametrize("name", [n for n, c in CASES.items() if c.get("port", True)])
def test_port_matches_reference(name):
    run_port(name)


def test_port_fixture_equals_reference_union():
    """The oracle's own rasteriser (the reference arm's input, built without
    the product library) gives the 64-sphere input of the reference's
    csgUnion bit for bit."""
    c, r = port.sixty_four_spheres(seed=2024)
    g = port.PortGrid.spheres(c, r, 1.0, 3.0)
    assert digest(g.to_host()) == GOLD["bench64_cfl05"][0]["digest"]
    c8, r8 = __import__("cases").union8()
    g8 = port.PortGrid.spheres(c8, r8, 1.0, 3.0)
    assert digest(g8.to_host()) == GOLD["union8_deformation"][0]["digest"]


def test_port_thread_independent():
    run_port("sphere20_deformation", threads=1)


@pytest.mark.parametrize("key", ["__batch__", "__batch_cfl05__"])
def test_port_batch_instances_match_reference(key):
    from cases import BATCH, BATCH_CFL, make_batch
    spec = BATCH_CFL if key == "__batch_cfl05__" else BATCH
    grids, fields = make_batch()
    sp, tp, tsp, ttp, nc = spec["schemes"]
    for g, f, rec in zip(grids, fields, GOLD[key]):
        p = port.PortGrid(g)
        for step, (t0, t1) in enumerate(spec["ops"], start=1):
            n = p.advect(f, t0, t1, spatial=sp, temporal=tp, tracker_spatial=tsp, tracker_temporal=ttp,
                         norm_count=nc, cfl=spec.get("cfl", 0.0))
            assert n == rec[step]["count"]
            assert digest(p.to_host()) == rec[step]["digest"]
