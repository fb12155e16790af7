"""FP64 error statement per configuration (test infrastructure).

The device PARITY path is bit-identical to the reference and to the oracle's
FP32 instance on every pinned case, including the 64-sphere benchmark window;
the oracle's FP64 instance runs the same scheme (same loop, constants,
operation order and time stepping) in double.  This script runs both
instances on the same inputs and reports, per configuration, the largest
|phi_FP32 - phi_FP64| over voxels active in both (in units of the band width
gamma), and the number of voxels whose active state differs.

    python -m oracle.fp64_error [config ...]     (configs: 1 2 3)

Configuration 1: sphere r=64 at the origin, constant velocity (1, 0.5, 0.25),
10 unit steps.  Configuration 2: the 64-sphere union (seed 2024), LeVeque
deformation on 1024^3 with T = 100, the benchmark's 25 unit steps.
Configuration 3: the first 64 of the 512 batched instances (seed 7), 50 unit
steps each.  All RK3-HJWENO5 at CFL 0.5, tracker RK1 with one
renormalisation.
"""
import json
import sys
import time

import numpy as np

from oracle import build_oracle, port


def _compare(a, b, gamma=3.0):
    """(max |a - b| over voxels active in both, active-state differences,
    voxels in both, the 99.99th percentile of |a - b| and the number of voxels
    where it exceeds 1e-5 gamma)."""
    ha, hb = a.to_host(), b.to_host()
    ka = {tuple(o): i for i, o in enumerate(ha.leaf_origins.tolist())}
    common = [(ka[tuple(o)], j) for j, o in enumerate(hb.leaf_origins.tolist()) if tuple(o) in ka]
    ia = np.array([c[0] for c in common], dtype=np.int64)
    ib = np.array([c[1] for c in common], dtype=np.int64)
    ma, mb = ha.active_mask_bool()[ia], hb.active_mask_bool()[ib]
    both = ma & mb
    d = np.abs(ha.leaf_values[ia][both].astype(np.float64) - hb.leaf_values[ib][both].astype(np.float64))
    flips = int((ma ^ mb).sum()) + int(ha.active_voxel_count() - ma.sum()) + int(hb.active_voxel_count() - mb.sum())
    p = float(np.percentile(d, 99.99)) if d.size else 0.0
    return (float(d.max()) if d.size else 0.0), flips, int(both.sum()), p, int((d > 1e-5 * gamma).sum())


def _run(make, field, steps, gamma=3.0):
    grids = [make(32), make(64)]
    worst, flips, worst_p, worst_big, per_step = 0.0, 0, 0.0, 0, []
    t = 0.0
    for k in range(steps):
        for g in grids:
            g.advect(field, t, t + 1.0, temporal=port.TVD_RK3, tracker_temporal=port.TVD_RK1, norm_count=1,
                     cfl=0.5)
        t += 1.0
        d, f, n, p, big = _compare(*grids, gamma=gamma)
        worst, flips, worst_p, worst_big = max(worst, d), max(flips, f), max(worst_p, p), max(worst_big, big)
        per_step.append({"step": k + 1, "max_dphi_over_gamma": d / gamma, "flips": f, "voxels": n,
                         "p9999_over_gamma": p / gamma, "voxels_above_1e-5_gamma": big})
    return {"max_dphi_over_gamma": worst / gamma, "max_flips": flips, "p9999_over_gamma": worst_p / gamma,
            "max_voxels_above_1e-5_gamma": worst_big, "steps": per_step}


def config1():
    f = port.FieldDesc()
    f.kind = 0
    f.constant[:] = (1.0, 0.5, 0.25)
    return _run(lambda p: port.PortGrid.spheres([[0.0, 0.0, 0.0]], [64.0], precision=p), f, 10)


def config2():
    c, r = port.sixty_four_spheres(seed=2024)
    return _run(lambda p: port.PortGrid.spheres(c, r, precision=p), port.deformation(), 25)


def config3(count=64):
    from openvdb_gb300 import fixtures
    specs, fields = fixtures.batch_instances(n=512, seed=7)
    out = []
    for spec, field in list(zip(specs, fields))[:count]:
        host = fixtures.build_instance(spec)
        fd = field.desc()
        r = _run(lambda p, h=host: port.PortGrid(h, precision=p), fd, 50)
        out.append({k: r[k] for k in ("max_dphi_over_gamma", "max_flips", "p9999_over_gamma",
                                       "max_voxels_above_1e-5_gamma")})
    return {"instances": count, "max_dphi_over_gamma": max(o["max_dphi_over_gamma"] for o in out),
            "max_flips": max(o["max_flips"] for o in out),
            "p9999_over_gamma": max(o["p9999_over_gamma"] for o in out),
            "max_voxels_above_1e-5_gamma": max(o["max_voxels_above_1e-5_gamma"] for o in out),
            "per_instance": out}


def main(argv):
    build_oracle.build()
    which = argv or ["1", "2", "3"]
    for c in which:
        t0 = time.time()
        res = {"1": config1, "2": config2, "3": config3}[c]()
        res = {"config": int(c), "seconds": round(time.time() - t0, 1), **res}
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
