"""Times the compiled reference (oracle/_ref/libvdbref.so: the reference's own
LevelSetAdvection / LevelSetTracker built from its sources, TBB replaced by
the oracle's std::thread shim) against the oracle's C++ restatement on the
64-sphere benchmark workload, at one thread and at all host threads.

Each run builds the input (untimed), advects `--warmup` untimed unit steps,
then times `--steps` unit steps advect(t, t+1) at CFL 0.5 (HJWENO5 + TVD_RK3,
tracker HJWENO5 + TVD_RK1, one renormalisation), and prints one JSON line
per (implementation, threads) with voxel-updates/s.  Test infrastructure:
needs the reference checkout's build (oracle/ref/build_ref.py).

  python oracle/time_cpu.py [--steps 1] [--warmup 1] [--threads 1,8]
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import port, refpy  # noqa: E402


def run_port(threads, warmup, steps):
    c, r = port.sixty_four_spheres(seed=2024)
    g = port.PortGrid.spheres(c, r, 1.0, 3.0, threads)
    field = port.deformation(1024.0, 100.0, 1.0)
    t = 0.0
    for _ in range(warmup):
        port._unit_step(g, field, t)
        t += 1.0
    g.updates = 0
    substeps = []
    t0 = time.perf_counter()
    for _ in range(steps):
        substeps.append(port._unit_step(g, field, t))
        t += 1.0
    return g.updates, time.perf_counter() - t0, substeps


def run_reference(threads, warmup, steps):
    from openvdb_gb300.fields import Field
    refpy.set_threads(threads)
    c, r = port.sixty_four_spheres(seed=2024)
    g = refpy.RefGrid.union_of_spheres(c, r)
    field = Field.deformation(domain=1024.0, period=100.0, scale=1.0)
    t = 0.0
    kw = dict(temporal=port.TVD_RK3, tracker_temporal=port.TVD_RK1, norm_count=1, cfl=0.5)
    for _ in range(warmup):
        g.advect(field, t, t + 1.0, **kw)
        t += 1.0
    substeps = []
    t0 = time.perf_counter()
    for _ in range(steps):
        substeps.append(g.advect(field, t, t + 1.0, **kw))
        t += 1.0
    return time.perf_counter() - t0, substeps


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--threads", default="1,%d" % (os.cpu_count() or 1))
    args = ap.parse_args()
    for th in [int(x) for x in args.threads.split(",")]:
        # the two are bit-identical, so the port's count of voxel-updates
        # (active voxels at every substep start) is the reference's too
        u, el_port, sub_port = run_port(th, args.warmup, args.steps)
        el_ref, sub_ref = run_reference(th, args.warmup, args.steps)
        assert sub_ref == sub_port, (sub_ref, sub_port)
        for name, el in (("reference", el_ref), ("port", el_port)):
            print(json.dumps({"impl": name, "threads": th, "voxel_updates_per_s": u / el, "seconds": el,
                              "steps": args.steps, "warmup": args.warmup, "substeps": sub_port,
                              "host": os.uname().machine, "cpus": os.cpu_count()}), flush=True)


if __name__ == "__main__":
    main()
