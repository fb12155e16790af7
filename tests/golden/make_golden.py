"""Generate tests/golden/parity_cases.json from the reference implementation.

Runs every case of tests/golden/cases.py through the UNMODIFIED reference
(tools::LevelSetAdvection / tools::LevelSetTracker / tools::LevelSetMorphing compiled from the
reference checkout into oracle/_ref/libvdbref.so by oracle/ref/build_ref.py)
and records the digest of the grid after each operation.  The input level
sets come from openvdb_gb300.fixtures; for spheres the generator first
checks that they equal the reference's own createLevelSetSphere bit for bit.
Each case also runs with one and with all oracle threads, which must agree.

Usage: python tests/golden/make_golden.py [--filters-only | --only=case1,case2]
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

from cases import (BATCH, BATCH_CFL, CASES, FILTER_CASES, MORPH_CASES, VOLUME_CASES, box_mask, make_batch,  # noqa: E402
                   make_field, make_fixture, make_volume, union8)
from openvdb_gb300.grid import bitwise_equal, digest, summary  # noqa: E402
from oracle import refpy  # noqa: E402


def run_reference(name, case, threads):
    refpy.set_threads(threads)
    fx = case["fixture"]
    host = make_fixture(fx)
    if fx[0] == "sphere":
        ref_sphere = refpy.RefGrid.sphere(fx[1], fx[2], fx[3], fx[4]).to_host()
        assert bitwise_equal(host, ref_sphere), "fixture differs from createLevelSetSphere: " + name
    if fx[0] in ("union8", "sixty_four"):
        # the union fixtures equal the reference's csgUnion of createLevelSetSphere
        from openvdb_gb300 import fixtures
        c, r = union8() if fx[0] == "union8" else fixtures.sixty_four_spheres(seed=fx[1])
        ref_union = refpy.RefGrid.union_of_spheres(c, r).to_host()
        assert bitwise_equal(host, ref_union), "fixture differs from csgUnion of the spheres: " + name
    g = refpy.RefGrid.from_host(host)
    assert bitwise_equal(g.to_host(), host), "round trip through the reference grid: " + name
    field = make_field(case["field"])
    sp, tp, tsp, ttp, nc = case["schemes"]
    trim = 3
    out = [{"op": "input", "digest": digest(host), "summary": summary(host)}]
    for op in case["ops"]:
        rec = {"op": list(op) if op[0] != "state" else ["state", op[1]]}
        if op[0] == "state":
            s = op[1]
            nc = s.get("norm_count", nc)
            ttp = s.get("tr_temporal", ttp)
            trim = s.get("trim", trim)
            out.append(rec)
            continue
        kw = dict(spatial=tsp, temporal=ttp, norm_count=nc, trim=trim)
        if op[0] == "advect" and case["field"][0] == "enright":
            rec["count"] = g.advect_enright(op[1], op[2], spatial=sp, temporal=tp, tracker_spatial=tsp,
                                            tracker_temporal=ttp, norm_count=nc, cfl=case.get("cfl", 0.0))
        elif op[0] == "advect":
            rec["count"] = g.advect(field, op[1], op[2], spatial=sp, temporal=tp, tracker_spatial=tsp,
                                    tracker_temporal=ttp, norm_count=nc, cfl=case.get("cfl", 0.0))
        elif op[0] == "track":
            g.track(**kw)
        elif op[0] == "normalize":
            g.normalize(**kw)
        elif op[0] == "prune":
            g.prune(**kw)
        elif op[0] == "dilate":
            g.dilate(op[1], **kw)
        elif op[0] == "normalize_masked":
            g.normalize_masked(*box_mask(g.to_host(), op[1], op[2]), **kw)
        else:
            raise ValueError(op)
        h = g.to_host()
        rec["digest"] = digest(h)
        rec["summary"] = summary(h)
        out.append(rec)
    return out


def run_volume(case, threads):
    """tools::VolumeAdvection on the case's volume: digest after every call."""
    refpy.set_threads(threads)
    host = make_volume(case["volume"])
    g = refpy.RefGrid.from_host(host)
    assert bitwise_equal(g.to_host(), host), "round trip through the reference grid"
    field = make_field(case["field"])
    out = [{"op": "input", "digest": digest(host), "summary": summary(host)}]
    for op in case["ops"]:
        _, integ, lim, sub, dt = op
        mv = g.volume_advect(field, dt, integrator=integ, limiter=lim, substeps=sub)
        h = g.to_host()
        out.append({"op": list(op), "digest": digest(h), "summary": summary(h), "max_velocity": mv})
    return out


def main():
    nthreads = os.cpu_count() or 1
    only = [a.split("=", 1)[1].split(",") for a in sys.argv if a.startswith("--only=")]
    if only:  # recompute the named advection / tracker cases, keep the rest
        path = os.path.join(HERE, "parity_cases.json")
        result = json.load(open(path))
        for name in only[0]:
            a = run_reference(name, CASES[name], 1)
            b = run_reference(name, CASES[name], nthreads)
            assert a == b, "reference result depends on the thread count: " + name
            result[name] = a
            print("%-32s ops=%d final active=%s" % (name, len(a) - 1, a[-1].get("summary", {}).get("active")))
        with open(path, "w") as f:
            json.dump(result, f, indent=1, sort_keys=True)
        return
    if "--batch-cfl-only" in sys.argv:  # recompute the imposed-CFL batch case, keep the rest
        path = os.path.join(HERE, "parity_cases.json")
        result = json.load(open(path))
        result["__batch_cfl05__"] = run_batch(BATCH_CFL)
        with open(path, "w") as f:
            json.dump(result, f, indent=1, sort_keys=True)
        return
    if "--volumes-only" in sys.argv:  # recompute the VolumeAdvection cases, keep the rest
        path = os.path.join(HERE, "parity_cases.json")
        result = json.load(open(path))
        vol = {}
        for name, case in VOLUME_CASES.items():
            a = run_volume(case, 1)
            b = run_volume(case, nthreads)
            assert a == b, "reference result depends on the thread count: " + name
            vol[name] = a
            print("%-32s ops=%d final active=%s leaves=%s" % (name, len(a) - 1, a[-1]["summary"]["active"],
                                                             a[-1]["summary"]["leaves"]))
        result["__volume__"] = vol
        with open(path, "w") as f:
            json.dump(result, f, indent=1, sort_keys=True)
        return
    if "--filters-only" in sys.argv:  # recompute the LevelSetFilter cases, keep the rest
        path = os.path.join(HERE, "parity_cases.json")
        result = json.load(open(path))
        filt = {}
        for name, case in FILTER_CASES.items():
            a = run_filter(case, 1)
            b = run_filter(case, nthreads)
            assert a == b, "reference result depends on the thread count: " + name
            filt[name] = a
            print("%-32s ops=%d final active=%s" % (name, len(a) - 1, a[-1]["summary"]["active"]))
        result["__filter__"] = filt
        with open(path, "w") as f:
            json.dump(result, f, indent=1, sort_keys=True)
        return
    result = {}
    for name, case in CASES.items():
        a = run_reference(name, case, 1)
        b = run_reference(name, case, nthreads)
        assert a == b, "reference result depends on the thread count: " + name
        result[name] = a
        last = a[-1]
        print("%-32s ops=%d final leaves=%s active=%s" % (name, len(a) - 1, last.get("summary", {}).get("leaves"),
                                                          last.get("summary", {}).get("active")))
    result["__batch__"] = run_batch()
    result["__batch_cfl05__"] = run_batch(BATCH_CFL)
    morph = {}
    for name, case in MORPH_CASES.items():
        a = run_morph(name, case, 1)
        b = run_morph(name, case, nthreads)
        assert a == b, "reference result depends on the thread count: " + name
        morph[name] = a
        print("%-32s ops=%d final active=%s" % (name, len(a) - 1, a[-1]["summary"]["active"]))
    result["__morph__"] = morph
    result["__volume__"] = {name: run_volume(case, nthreads) for name, case in VOLUME_CASES.items()}
    filt = {}
    for name, case in FILTER_CASES.items():
        a = run_filter(case, 1)
        b = run_filter(case, nthreads)
        assert a == b, "reference result depends on the thread count: " + name
        filt[name] = a
        print("%-32s ops=%d final active=%s" % (name, len(a) - 1, a[-1]["summary"]["active"]))
    result["__filter__"] = filt
    with open(os.path.join(HERE, "parity_cases.json"), "w") as f:
        json.dump(result, f, indent=1, sort_keys=True)


def run_morph(name, case, threads):
    """A LevelSetMorphing case: digests after every advect(t0, t1) call."""
    refpy.set_threads(threads)
    src, tgt = make_fixture(case["source"]), make_fixture(case["target"])
    g = refpy.RefGrid.from_host(src)
    target = refpy.RefGrid.from_host(tgt)
    mask = refpy.RefGrid.from_host(make_fixture(case["mask"])) if "mask" in case else None
    sp, tp, tsp, ttp, nc = case["schemes"]
    out = [{"op": "input", "digest": digest(src), "target": digest(tgt), "summary": summary(src)}]
    for op in case["ops"]:
        kw = {}
        if len(op) > 3:
            kw = dict(mask=mask, mask_range=op[3], invert=op[4])
        n = g.morph(target, op[1], op[2], spatial=sp, temporal=tp, tracker_spatial=tsp, tracker_temporal=ttp,
                    norm_count=nc, **kw)
        h = g.to_host()
        out.append({"op": list(op), "count": n, "digest": digest(h), "summary": summary(h)})
    return out


def run_filter(case, threads):
    """A LevelSetFilter case: digests after every filter call."""
    refpy.set_threads(threads)
    src = make_fixture(case["fixture"])
    g = refpy.RefGrid.from_host(src)
    mask = refpy.RefGrid.from_host(make_fixture(case["mask"])) if "mask" in case else None
    tsp, ttp, nc = case["tracker"]
    out = [{"op": "input", "digest": digest(src), "summary": summary(src)}]
    for op in case["ops"]:
        kw = {}
        if len(op) > 3:
            kw = dict(mask=mask, mask_range=op[3], invert=op[4])
        g.filter(op[0], op[1], op[2], spatial=tsp, temporal=ttp, norm_count=nc, **kw)
        h = g.to_host()
        out.append({"op": [list(x) if isinstance(x, tuple) else x for x in op], "digest": digest(h),
                    "summary": summary(h)})
    return out


def run_batch(spec=BATCH):
    """Each instance of the batch case advected alone by the reference."""
    grids, fields = make_batch()
    sp, tp, tsp, ttp, nc = spec["schemes"]
    out = []
    for g, f in zip(grids, fields):
        r = refpy.RefGrid.from_host(g)
        rec = [{"op": "input", "digest": digest(g), "summary": summary(g)}]
        for t0, t1 in spec["ops"]:
            n = r.advect(f, t0, t1, spatial=sp, temporal=tp, tracker_spatial=tsp, tracker_temporal=ttp,
                         norm_count=nc, cfl=spec.get("cfl", 0.0))
            h = r.to_host()
            rec.append({"op": ["advect", t0, t1], "count": n, "digest": digest(h), "summary": summary(h)})
        out.append(rec)
    print("batch: %d instances" % len(out))
    return out


if __name__ == "__main__":
    main()
