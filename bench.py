"""Benchmark: narrow-band level-set advection (RK3-HJWENO5 + track) on one GB300.

Workload (the 64-sphere configuration): the union of 64 spheres with seeded
centres U[0,1024]^3 and radii U[20,80] voxels (half-width 3, voxel size 1),
advected by LeVeque's divergence-free deformation field on the unit cube
mapped to 1024^3, scaled by cos(pi t / 100) (1 voxel per time unit per unit
of field), HJWENO5 + TVD-RK3 with CFL 0.5, tracker HJWENO5 + TVD-RK1 with one
renormalisation per substep.  One bench step = advect(t, t+1) (all CFL
substeps of one time unit, each followed by the tracker pass).

Metric: voxel-updates/s = sum over substeps of the active voxels at the
substep start / device time (CUDA events on the library stream, L2 flushed
between steps).  `e2e` runs the same steps through the host-facing API: the
level set is uploaded from host arrays, advected and downloaded every step.

  python bench.py [--steps K] [--warmup W] [--mode fast|parity] [--impl reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "narrow-band voxel-updates/s per RK3-HJWENO5 step (FP32)"
UNIT = "voxel-updates/s"
WORKLOAD = {"workload": "64-sphere union, LeVeque deformation x cos(pi t/100), 1024^3 domain",
            "spheres": 64, "seed": 2024, "domain": 1024, "radii": [20, 80], "half_width": 3,
            "spatial": "HJWENO5", "temporal": "TVD_RK3", "cfl": 0.5, "tracker": "HJWENO5/TVD_RK1",
            "norm_count": 1, "l2": "flushed between steps (256 MiB write)"}


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.proc = None
        self.lines = []
        self.device = device

    def _gpu_id(self):
        """The sampled GPU by UUID: CUDA's device order need not be nvidia-smi's."""
        try:
            import torch
            return "GPU-%s" % torch.cuda.get_device_properties(self.device).uuid
        except Exception:
            return os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self._gpu_id(),
                                          "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---- replicas over torchrun ranks --------------------------------------------
# The path is not sharded: with N ranks every rank advects its own copy of the
# workload on its own GPU (weak scaling), the timed regions are bracketed by
# barriers, and the line reports the units of all ranks over the slowest
# rank's time.

def dist_setup():
    """(rank, world size, torch.distributed or None) from the torchrun
    environment; one process per GPU (LOCAL_RANK)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, None
    import torch
    import torch.distributed as dist
    if not dist.is_initialized():
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend, init_method="env://")
    return dist.get_rank(), ws, dist


def dist_barrier(dist):
    if dist is not None:
        dist.barrier()


def replica_totals(units, seconds, dist):
    """(sum of units over ranks, max of seconds over ranks)."""
    if dist is None:
        return float(units), float(seconds)
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    u = torch.tensor([float(units)], dtype=torch.float64, device=dev)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(u.item()), float(t.item())


def measured_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def workload_config(args):
    """The `config` both arms print: the workload, the arithmetic mode and the
    timed window (unit steps t = warmup .. warmup + steps)."""
    cfg = dict(WORKLOAD)
    cfg.update({"mode": args.mode, "t_start": float(args.warmup), "unit_steps": int(args.steps)})
    return cfg


def build_workload():
    from openvdb_gb300 import Field, fixtures
    centers, radii = fixtures.sixty_four_spheres(seed=2024)
    host = fixtures.union_of_spheres(centers, radii, 1.0, 3.0)
    field = Field.deformation(domain=1024.0, period=100.0, scale=1.0)
    return host, field


def make_advection(dev, field, cfl=0.5):
    from openvdb_gb300 import LevelSetAdvection
    from openvdb_gb300.levelset import HJWENO5_BIAS, TVD_RK1, TVD_RK3
    adv = LevelSetAdvection(dev, field)
    adv.setSpatialScheme(HJWENO5_BIAS)
    adv.setTemporalScheme(TVD_RK3)
    adv.setTrackerSpatialScheme(HJWENO5_BIAS)
    adv.setTrackerTemporalScheme(TVD_RK1)
    adv.setNormCount(1)
    adv.cfl = cfl
    return adv


def host_bytes(g):
    return int(sum(getattr(g, k).nbytes for k in ("leaf_origins", "leaf_masks", "leaf_values",
                                                   "lower_origins", "lower_tiles", "upper_origins",
                                                   "upper_tiles", "root_tile_origins", "root_tile_values")))


def run_gb300(args):
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from openvdb_gb300 import FAST, PARITY, DeviceLevelSet
    from openvdb_gb300.levelset import DeviceField

    torch.cuda.init()
    dev_index = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev_index)
    rank, world, dist = dist_setup()
    t_build = time.perf_counter()
    host, field = build_workload()
    t_build = time.perf_counter() - t_build
    dev = DeviceLevelSet(host, device=dev_index)
    mode = FAST if args.mode == "fast" else PARITY
    dev.set_precision(mode)
    stream = torch.cuda.Stream()
    dev.set_stream(stream.cuda_stream)
    dfield = DeviceField(field)
    adv = make_advection(dev, dfield, cfl=args.cfl)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > L2

    t = 0.0
    for _ in range(args.warmup):
        adv.advect(t, t + 1.0)
        t += 1.0
    torch.cuda.synchronize()
    # launch shapes chosen on the warmed-up level set (cached per device)
    from openvdb_gb300 import autotune
    tuning = autotune.tune(dev.handle, dfield._h, mode, dev.leaf_count())
    torch.cuda.synchronize()

    dev.reset_stats()
    dev.set_profiling(True)
    clocks = ClockSampler(dev_index)
    clocks.start()
    torch.cuda.synchronize()
    dist_barrier(dist)
    times = []
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        adv.advect(t, t + 1.0)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
        t += 1.0
    torch.cuda.synchronize()
    dist_barrier(dist)
    clk = clocks.stop()
    dev.set_profiling(False)
    st = dev.stats()
    all_updates, total = replica_totals(st["voxel_updates"], sum(times), dist)
    value = all_updates / total

    peak, peak_kind = measured_peaks()
    rk_gbs = st["rk_bytes"] / (st["rk_ms"] / 1e3) / 1e9 if st["rk_ms"] > 0 else 0.0
    norm_gbs = st["norm_bytes"] / (st["norm_ms"] / 1e3) / 1e9 if st["norm_ms"] > 0 else 0.0
    dominant = "rk_stage" if st["rk_ms"] >= st["norm_ms"] else "normalize"
    achieved = rk_gbs if dominant == "rk_stage" else norm_gbs
    launches = st["rk_launches"] if dominant == "rk_stage" else st["norm_launches"]
    traffic = None
    # DRAM bytes per launch of the dominant kernel from one ncu capture
    # (profiles/traffic.txt: "<kernel>_<mode> <bytes>" per line)
    tp = os.path.join(HERE, "profiles", "traffic.txt")
    if os.path.exists(tp):
        for line in open(tp):
            f = line.split()
            if len(f) == 2 and f[0] == dominant + "_" + args.mode:
                traffic = int(f[1])

    # FP32-pipe roof of the dominant kernel: FP32 thread instructions per
    # voxel-stage from one ncu capture (profiles/fp32_ops.txt: "<kernel>_<mode>
    # <count>" per line) times the voxel-stages per second it sustained here,
    # against 152 SMs x 128 FP32 lanes x the SM clock sampled under load
    roof32 = None
    fp = os.path.join(HERE, "profiles", "fp32_ops.txt")
    if os.path.exists(fp) and clk and clk.get("sm_mhz"):
        kms = st["rk_ms"] if dominant == "rk_stage" else st["norm_ms"]
        stages = 3 * st["voxel_updates"] if dominant == "rk_stage" else st["dilated_voxels"]
        for line in open(fp):
            f = line.split()
            if len(f) == 2 and f[0] == dominant + "_" + args.mode and kms > 0:
                ach = float(f[1]) * stages / (kms / 1e3) / 1e9
                pk = 152 * 128 * clk["sm_mhz"] * 1e6 / 1e9
                roof32 = {"bound": "fp32", "kernel": dominant, "achieved": ach, "peak": pk,
                          "unit": "G thread-inst/s", "frac": ach / pk,
                          "inst_per_voxel_stage": float(f[1]), "peak_source": "152 SMs x 128 lanes x sampled SM clock"}

    # end to end through the host-facing API: upload, advect one time unit, download
    e2e = None
    if args.e2e_steps > 0:
        # the level set lives in page-locked host memory; each step uploads
        # it, advects one time unit and downloads the result into the same
        # buffers (an in-place update of the host grid)
        # A long-lived LevelSetAdvection object re-uploads its grid on every
        # advect call (gbls_upload keeps the handle's device allocations).
        from openvdb_gb300 import HostArena
        arena = HostArena(pinned=True)
        g = dev.to_host(arena)
        d = DeviceLevelSet(g, device=dev_index)
        d.set_precision(mode)
        autotune.apply(d.handle, tuning["config"])  # the launch shapes of the device-timed steps
        a = make_advection(d, dfield, cfl=args.cfl)
        # one untimed step of the same loop: the handle's scratch reaches its working size
        d.upload(g)
        a.advect(t, t + 1.0)
        g = d.to_host(arena)
        torch.cuda.synchronize()
        te = t + 1.0
        e2e_updates = 0
        h2d = d2h = 0
        dist_barrier(dist)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            h2d += host_bytes(g)
            d.upload(g)
            d.reset_stats()
            a.advect(te, te + 1.0)
            e2e_updates += d.stats()["voxel_updates"]
            g = d.to_host(arena)
            d2h += host_bytes(g)
            te += 1.0
        el = time.perf_counter() - t0
        d.close()
        e2e_all, el = replica_totals(e2e_updates, el, dist)
        e2e = {"value": e2e_all / el, "unit": UNIT, "h2d_bytes_per_step": h2d // args.e2e_steps,
               "d2h_bytes_per_step": d2h // args.e2e_steps, "steps": args.e2e_steps}

    cfg = workload_config(args)
    run = {"active_voxels_initial": int(host.active_voxel_count()), "leaves_initial": int(host.leaf_count),
           "fixture_build_s": round(t_build, 2), "substeps": int(st["substeps"]),
           "active_voxels_end": int(st["active_voxels"]),
           "rho_dilated": (st["dilated_voxels"] / st["voxel_updates"]) if st["voxel_updates"] else None,
           "replicas": world}
    if dist is not None:
        dist_barrier(dist)
        dist.destroy_process_group()
    if rank != 0:
        return
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded fixtures)",
        "config": cfg, "run": run,
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak,
                     "peak_source": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "launches": int(launches),
                     "rk_stage_gbs": rk_gbs, "normalize_gbs": norm_gbs,
                     "rk_stage_ms": st["rk_ms"], "normalize_ms": st["norm_ms"],
                     "step_ms_total": 1e3 * total},
        "roofline_fp32": roof32,
        "launch_config": tuning,
        "e2e": e2e,
        "gpu_launches": int(st["kernel_launches"]),
        "clocks": clk,
        "cpu_baseline": cpu_baseline(args) if args.cpu_baseline else None,
    }
    if args.extras:
        def extra(fn, *a, **kw):
            # a failing extra reports its error instead of losing the line
            try:
                return fn(*a, **kw)
            except Exception as e:  # noqa: BLE001
                return {"error": "%s: %s" % (type(e).__name__, e)}
        out["config1"] = extra(config1_sphere, mode, args.mode, args.cfl)
        out["adjoint"] = extra(adjoint_cost, mode, args.mode)
        out["batched"] = extra(batch_measure, args, steps=3, warmup=3, cpu=False)
        out["fp64_error"] = extra(fp64_errors, args.cfl)
        if args.mode != "fast":
            out["fast"] = extra(fast_line, args.cfl)
    print(json.dumps(out))


def config1_sphere(mode, mode_name, cfl, steps=10):
    """The small configuration: a radius-64 sphere (voxel size 1, half width 3)
    advected by the constant velocity (1, 0.5, 0.25) for 10 unit steps, RK3,
    tracker RK1 with one renormalisation; CUDA events around the 10 calls."""
    import torch
    from openvdb_gb300 import DeviceLevelSet, Field, fixtures
    from openvdb_gb300.levelset import DeviceField
    dev = DeviceLevelSet(fixtures.sphere(64.0, (0.0, 0.0, 0.0)))
    dev.set_precision(mode)
    stream = torch.cuda.Stream()
    dev.set_stream(stream.cuda_stream)
    adv = make_advection(dev, DeviceField(Field.constant_field((1.0, 0.5, 0.25))), cfl=cfl)
    adv.advect(-1.0, 0.0)  # warm-up on the same level set, before t = 0
    torch.cuda.synchronize()
    dev.reset_stats()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for t in range(steps):
        adv.advect(float(t), float(t + 1))
    e1.record(stream)
    e1.synchronize()
    st = dev.stats()
    ms = e0.elapsed_time(e1)
    return {"workload": "sphere r=64, constant velocity (1, 0.5, 0.25), 10 unit steps, RK3-HJWENO5, CFL %g" % cfl,
            "mode": mode_name, "value": st["voxel_updates"] / (ms / 1e3), "unit": UNIT, "ms": ms,
            "substeps": int(st["substeps"]), "active_voxels_end": int(st["active_voxels"])}


def fast_line(cfl, steps=10, warmup=3):
    """The same workload and window in FAST mode (FP32 WENO5 weights, not
    bit-identical: its deviation is stated in the design notes), timed like
    the headline: throughput and the FAST RK stage's HBM roofline."""
    import torch
    from openvdb_gb300 import FAST, DeviceLevelSet
    from openvdb_gb300.levelset import DeviceField
    host, field = build_workload()
    dev = DeviceLevelSet(host)
    dev.set_precision(FAST)
    stream = torch.cuda.Stream()
    dev.set_stream(stream.cuda_stream)
    adv = make_advection(dev, DeviceField(field), cfl=cfl)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    t = 0.0
    for _ in range(warmup):
        adv.advect(t, t + 1.0)
        t += 1.0
    torch.cuda.synchronize()
    dev.reset_stats()
    dev.set_profiling(True)
    total = 0.0
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        adv.advect(t, t + 1.0)
        e1.record(stream)
        e1.synchronize()
        total += e0.elapsed_time(e1) / 1e3
        t += 1.0
    dev.set_profiling(False)
    st = dev.stats()
    peak, kind = measured_peaks()
    gbs = st["rk_bytes"] / (st["rk_ms"] / 1e3) / 1e9 if st["rk_ms"] > 0 else 0.0
    dev.close()
    return {"mode": "fast", "value": st["voxel_updates"] / total, "unit": UNIT, "ms_per_step": 1e3 * total / steps,
            "rk_stage_gbs": gbs, "rk_stage_hbm_frac": gbs / peak, "peak_source": kind,
            "note": "not bit-identical to the reference (FP32 WENO5 weights)"}


def _band_error(h32, h64, v64, gamma):
    """The FP32 run (HostGrid h32) against the FP64 run (band h64, its active
    values v64 in canonical order): max and 99.99th percentile of |phi32 -
    phi64| / gamma over voxels active in both, voxels above 1e-5 gamma, and
    active-state differences."""
    import numpy as np
    m64 = h64.active_mask_bool()
    dense64 = np.zeros(m64.shape, np.float64)
    dense64[m64] = v64  # leaf-major, voxel-minor: the canonical order
    k64 = {tuple(o): i for i, o in enumerate(h64.leaf_origins.tolist())}
    m32 = h32.active_mask_bool()
    pairs = [(i, k64[tuple(o)]) for i, o in enumerate(h32.leaf_origins.tolist()) if tuple(o) in k64]
    i32 = np.array([p[0] for p in pairs], np.int64)
    i64 = np.array([p[1] for p in pairs], np.int64)
    a, b = m32[i32], m64[i64]
    both = a & b
    d = np.abs(h32.leaf_values[i32][both].astype(np.float64) - dense64[i64][both]) / gamma
    flips = int((a ^ b).sum()) + int(m32.sum() - a.sum()) + int(m64.sum() - b.sum())
    return {"max_dphi_over_gamma": float(d.max()) if d.size else 0.0,
            "p9999_over_gamma": float(np.percentile(d, 99.99)) if d.size else 0.0,
            "voxels_above_1e-5_gamma": int((d > 1e-5).sum()), "active_state_differences": flips,
            "voxels_compared": int(both.sum())}


def fp64_errors(cfl, n_batch=16):
    """The FP32 PARITY run's error against the device's FP64 instance (the
    same scheme with the values in double, bit-identical to the oracle's
    FP64 run), per configuration: configuration 1 (10 unit steps), the
    64-sphere benchmark window from t = 0 (25 unit steps) and the first
    n_batch instances of the batch (50 unit steps each, on their own
    handles); the worst step, and for the batch the worst instance."""
    import torch
    from openvdb_gb300 import FP64, PARITY, DeviceLevelSet, Field, fixtures
    from openvdb_gb300.levelset import DeviceField
    out = {}
    cases = {"config1": (lambda: fixtures.sphere(64.0, (0.0, 0.0, 0.0)), lambda: Field.constant_field((1.0, 0.5, 0.25)),
                         10),
             "config2": (lambda: build_workload()[0], lambda: build_workload()[1], 25)}
    # configuration 3: the first instances of the 512-instance batch, each on its own handle
    specs, fields = fixtures.batch_instances(n=512, seed=7)
    for i in range(n_batch):
        cases["config3_%d" % i] = ((lambda sp=specs[i]: fixtures.build_instance(sp)), (lambda f=fields[i]: f), 50)
    for name, (make_grid, make_field, steps) in cases.items():
        g, f = make_grid(), DeviceField(make_field())
        runs = []
        for mode in (PARITY, FP64):
            d = DeviceLevelSet(g)
            d.set_precision(mode)
            runs.append((d, make_advection(d, f, cfl=cfl)))
        worst, t64, upd64 = None, 0.0, 0
        for step in range(steps):
            for k, (d, adv) in enumerate(runs):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                d.reset_stats()
                adv.advect(float(step), float(step + 1))
                torch.cuda.synchronize()
                if k == 1:
                    t64 += time.perf_counter() - t0
                    upd64 += d.stats()["voxel_updates"]
            e = _band_error(runs[0][0].to_host(), runs[1][0].to_host(), runs[1][0].active_values_f64(),
                            float(g.background))
            if worst is None:
                worst = dict(e)
            else:
                for key in ("max_dphi_over_gamma", "p9999_over_gamma"):
                    worst[key] = max(worst[key], e[key])
                for key in ("voxels_above_1e-5_gamma", "active_state_differences"):
                    worst[key] = max(worst[key], e[key])
        worst["steps"] = steps
        worst["fp64_voxel_updates_per_s"] = upd64 / t64 if t64 > 0 else None
        out[name] = worst
        for d, _ in runs:
            d.close()
    inst = [out.pop(k) for k in list(out) if k.startswith("config3_")]
    if inst:
        out["config3"] = {"instances": len(inst), "steps": 50,
                          "max_dphi_over_gamma": max(e["max_dphi_over_gamma"] for e in inst),
                          "p9999_over_gamma": max(e["p9999_over_gamma"] for e in inst),
                          "voxels_above_1e-5_gamma": max(e["voxels_above_1e-5_gamma"] for e in inst),
                          "active_state_differences": max(e["active_state_differences"] for e in inst)}
    return out


def fp64_errors_dense(cfl):
    """The same statement for the adjoint configurations' forward runs (PARITY
    against FP64, dense velocity grids): configuration 4 (radius-40 sphere in
    128^3, smoothed-noise velocity, 20 steps, every step checked) and
    configuration 5 (radius-160 sphere in 512^3, the inverse problem's initial
    velocity, 200 steps, every 10th step checked)."""
    from openvdb_gb300 import FP64, PARITY, DeviceLevelSet, Field, fixtures
    from openvdb_gb300.levelset import DeviceField
    template, vel, _, _ = fixtures.adjoint_128()
    cases = {"config4": (template, vel, 20, 1),
             "config5": (fixtures.sphere(160.0, (256.0, 256.0, 256.0)), _initial_velocity(512, 0.05, 5), 200, 10)}
    out = {}
    for name, (g, v, steps, every) in cases.items():
        f = DeviceField(Field.dense(v, (0, 0, 0), (0.0, 0.0, 0.0)))
        runs = []
        for mode in (PARITY, FP64):
            d = DeviceLevelSet(g)
            d.set_precision(mode)
            runs.append((d, make_advection(d, f, cfl=cfl)))
        worst = None
        for step in range(steps):
            for d, adv in runs:
                adv.advect(float(step), float(step + 1))
            if (step + 1) % every and step + 1 != steps:
                continue
            e = _band_error(runs[0][0].to_host(), runs[1][0].to_host(), runs[1][0].active_values_f64(),
                            float(g.background))
            if worst is None:
                worst = dict(e)
            else:
                for key in ("max_dphi_over_gamma", "p9999_over_gamma", "voxels_above_1e-5_gamma",
                            "active_state_differences"):
                    worst[key] = max(worst[key], e[key])
        worst.update({"steps": steps, "checked_every": every})
        out[name] = worst
        for d, _ in runs:
            d.close()
        del f
    return out


def run_fp64_errors(args):
    """--workload fp64errors: the FP32 (PARITY) run's error against the
    device's FP64 instance for configurations 1-5, one JSON line."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    torch.cuda.init()
    torch.cuda.set_device(0)
    out = {"metric": "max |phi_FP32 - phi_FP64| / band width and active-state differences, per configuration",
           "unit": "band width", "cfl": args.cfl}
    out.update(fp64_errors(args.cfl))
    out.update(fp64_errors_dense(args.cfl))
    print(json.dumps(out))


def adjoint_cost(mode, mode_name, reps=3):
    """The 128^3 adjoint configuration (20 unit steps of RK3-HJWENO5, dense
    128^3 x 3 velocity): plain forward, recorded forward and reverse sweep of
    the device-resident tape, each timed with CUDA events on the stream the
    tape runs on (best of `reps`); cost_ratio = (recorded forward + adjoint) /
    plain forward."""
    import torch
    from openvdb_gb300 import fixtures
    from openvdb_gb300.adjoint import DeviceTape
    template, vel, target, times = fixtures.adjoint_128()
    tape = DeviceTape(template, vel.shape, mode=mode)
    phi0 = torch.tensor(template.active_values(), device="cuda")
    v = torch.tensor(vel, device="cuda")
    phiT = tape.forward(phi0, v, times, record=True)  # warm-up; the loss gradient at its end
    coords = tape.dev.to_host().active_coords()
    dl = (2.0 * (phiT - torch.tensor(target(coords), dtype=torch.float32, device="cuda"))).contiguous()
    tape.backward(dl)
    stream = torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
    best = None
    for _ in range(reps):
        torch.cuda.synchronize()
        ev[0].record(stream)
        tape.forward(phi0, v, times, record=False)
        ev[1].record(stream)
        ev[2].record(stream)
        tape.forward(phi0, v, times, record=True)
        ev[3].record(stream)
        tape.backward(dl)
        ev[4].record(stream)
        ev[4].synchronize()
        r = (ev[0].elapsed_time(ev[1]), ev[2].elapsed_time(ev[3]), ev[3].elapsed_time(ev[4]))
        if best is None or sum(r[1:]) / r[0] < sum(best[1:]) / best[0]:
            best = r
    fwd, rec, adj = best
    return {"workload": "adjoint 128^3: sphere r=40 -> 5%-perturbed sphere r=44, smoothed-noise velocity "
                        "(sigma 4, amplitude 1), 20 unit steps, RK3-HJWENO5, tracker RK1",
            "mode": mode_name, "forward_ms": fwd, "recorded_forward_ms": rec, "adjoint_ms": adj,
            "cost_ratio": (rec + adj) / fwd, "substeps": int(sum(tape.substeps)),
            "timing": "CUDA events on the tape's stream, best of %d" % reps}


BATCH_WORKLOAD = {"workload": "512 seeded instances (50/50 sphere/torus, R log-uniform [8,128], tube ratio "
                              "U[0.2,0.4]), constant + rotation velocity per instance, one batch handle",
                  "instances": 512, "seed": 7, "half_width": 3, "spatial": "HJWENO5", "temporal": "TVD_RK3",
                  "cfl": 0.5, "tracker": "HJWENO5/TVD_RK1", "norm_count": 1,
                  "l2": "flushed between steps (256 MiB write)"}


def batch_measure(args, steps, warmup, cpu=True):
    """The batched configuration: every instance advanced by one time unit per
    step, each with its own CFL substeps, in one gbls_batch_advect call.
    Returns the line's fields."""
    import torch
    from openvdb_gb300 import FAST, PARITY, fixtures
    from openvdb_gb300.levelset import DeviceBatch

    t_build = time.perf_counter()
    specs, fields = fixtures.batch_instances(n=512, seed=7)
    grids = [fixtures.build_instance(sp) for sp in specs]
    t_build = time.perf_counter() - t_build
    b = DeviceBatch(grids)
    b.set_precision(FAST if args.mode == "fast" else PARITY)
    b.set_tracker(norm_count=1)
    stream = torch.cuda.Stream()
    b.set_stream(stream.cuda_stream)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    t = 0.0
    for _ in range(warmup):
        b.advect(fields, t, t + 1.0, cfl=args.cfl)
        t += 1.0
    torch.cuda.synchronize()
    from openvdb_gb300 import autotune
    from openvdb_gb300.levelset import DeviceField
    timing_field = DeviceField(fields[0])  # launch timing only: any device-evaluated field
    tuning = autotune.tune(b.handle, timing_field._h, FAST if args.mode == "fast" else PARITY,
                           sum(b.counts(i).leaf_count for i in range(b.n)))
    torch.cuda.synchronize()
    b.reset_stats()
    b.set_profiling(True)
    clocks = ClockSampler(0)
    clocks.start()
    times, subs = [], []
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        counts = b.advect(fields, t, t + 1.0, cfl=args.cfl)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
        subs.append(max(counts))
        t += 1.0
    torch.cuda.synchronize()
    clk = clocks.stop()
    b.set_profiling(False)
    st = b.stats()
    total = sum(times)
    peak, peak_kind = measured_peaks()
    rk_gbs = st["rk_bytes"] / (st["rk_ms"] / 1e3) / 1e9 if st["rk_ms"] > 0 else 0.0
    norm_gbs = st["norm_bytes"] / (st["norm_ms"] / 1e3) / 1e9 if st["norm_ms"] > 0 else 0.0
    active = sum(b.counts(i).active_voxel_count for i in range(b.n))
    cfg = dict(BATCH_WORKLOAD)
    cfg.update({"mode": args.mode, "active_voxels_initial": int(sum(g.active_voxel_count() for g in grids)),
                "active_voxels_end": int(active), "fixture_build_s": round(t_build, 2),
                "instance_substeps": int(st["substeps"]), "max_substeps_per_step": int(max(subs)),
                "t_start": float(t - steps)})
    out = {
        "metric": METRIC, "value": st["voxel_updates"] / total, "unit": UNIT, "n_gpus": 1, "steps": steps,
        "warmup": warmup, "ms_per_step": 1e3 * total / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded fixtures)",
        "config": cfg,
        "roofline": {"bound": "hbm", "kernel": "rk_stage", "achieved": rk_gbs, "peak": peak,
                     "peak_source": peak_kind, "unit": "GB/s", "frac": rk_gbs / peak, "traffic": None,
                     "launches": int(st["rk_launches"]), "rk_stage_gbs": rk_gbs, "normalize_gbs": norm_gbs,
                     "rk_stage_ms": st["rk_ms"], "normalize_ms": st["norm_ms"], "step_ms_total": 1e3 * total},
        "launch_config": tuning,
        "e2e": None,
        "gpu_launches": int(st["kernel_launches"]),
        "clocks": clk,
        "cpu_baseline": None,
    }
    if cpu and args.cpu_baseline:
        from oracle import build_oracle, port
        build_oracle.build()
        out["cpu_baseline"] = port.bench_batch_sample(args.cpu_seconds)
    return out


def run_batch(args):
    import torch
    import __graft_entry__
    __graft_entry__.build()
    torch.cuda.init()
    torch.cuda.set_device(0)
    print(json.dumps(batch_measure(args, args.steps, args.warmup)))


ADJOINT_WORKLOAD = {"workload": "inverse problem: sphere r=160 -> torus R=160 r=48 (y axis) in 512^3, dense "
                                "512^3 x 3 velocity (seeded separable sine modes, amplitude 0.05), 200 unit "
                                "steps, checkpoint every 10, normalised gradient descent on the velocity",
                    "domain": 512, "steps": 200, "checkpoint_every": 10, "spatial": "HJWENO5",
                    "temporal": "TVD_RK3", "cfl": 0.5, "tracker": "HJWENO5/TVD_RK1", "norm_count": 1}


def run_profile_case(args):
    """Small cases for ncu captures (inputs still larger than L2), one JSON
    line each: sphere16 = the first 16 of the 64 benchmark spheres (3.25 M
    active voxels), one advect(0, 0.2) call (one CFL substep: 3 RK stages, 1
    renormalisation) of the benchmark scheme; adjoint128 = one best-of-1 pass
    of the 128^3 adjoint configuration."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from openvdb_gb300 import FAST, PARITY, DeviceLevelSet, Field, fixtures
    from openvdb_gb300.levelset import DeviceField
    torch.cuda.init()
    mode = FAST if args.mode == "fast" else PARITY
    if args.workload == "adjoint128":
        print(json.dumps(adjoint_cost(mode, args.mode, reps=1)))
        return
    c, r = fixtures.sixty_four_spheres(seed=2024)
    d = DeviceLevelSet(fixtures.union_of_spheres(c[:16], r[:16], 1.0, 3.0))
    d.set_precision(mode)
    before = (d.active_voxel_count(), d.leaf_count())
    a = make_advection(d, DeviceField(Field.deformation(domain=1024.0, period=100.0, scale=1.0)), cfl=args.cfl)
    n = a.advect(0.0, 0.2)
    torch.cuda.synchronize()
    print(json.dumps({"workload": "sphere16: 16 of the 64 benchmark spheres, advect(0, 0.2)", "mode": args.mode,
                      "active_before": before[0], "leaves_before": before[1], "substeps": n,
                      "active_after": d.active_voxel_count(), "leaves_after": d.leaf_count()}))
    d.close()


def _initial_velocity(n, amp, seed):
    """Seeded smooth velocity: per component a sum of three separable sine modes."""
    rng = np.random.Generator(np.random.PCG64(seed))
    x = np.arange(n, dtype=np.float64) * (2.0 * np.pi / n)
    vel = np.zeros((n, n, n, 3), np.float32)
    for c in range(3):
        acc = np.zeros((n, n, n), np.float32)
        for _ in range(3):
            k = rng.integers(1, 4, 3)
            ph = rng.uniform(0.0, 2.0 * np.pi, 3)
            a = rng.uniform(-1.0, 1.0)
            fx, fy, fz = (np.sin(k[i] * x + ph[i]).astype(np.float32) for i in range(3))
            acc += np.float32(a) * fx[:, None, None] * fy[None, :, None] * fz[None, None, :]
        vel[..., c] = amp * acc / 3.0
    return vel


def run_adjoint(args):
    """Checkpointed adjoint at scale: `--steps` gradient-descent iterations, each a
    200-step forward pass (checkpoints every 10 steps) and the reverse sweep."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from openvdb_gb300 import FAST, fixtures
    from openvdb_gb300.adjoint import CheckpointedAdvection

    torch.cuda.init()
    torch.cuda.set_device(0)
    n, c = 512, np.array([256.0, 256.0, 256.0])
    template = fixtures.sphere(160.0, tuple(c))
    vel = _initial_velocity(n, 0.05, 5)

    def target(coords):
        d = coords.astype(np.float64) - c
        q = np.sqrt(d[:, 0] ** 2 + d[:, 2] ** 2) - 160.0
        return np.sqrt(q * q + d[:, 1] ** 2) - 48.0

    times = [float(t) for t in range(201)]
    ck = CheckpointedAdvection(template, vel, every=10, mode=FAST, cfl=args.cfl)
    v_dev = torch.from_numpy(vel).cuda()
    phi0 = template.active_values().copy()
    total = torch.cuda.mem_get_info()[1]
    min_free = total
    hist, t_fwd, t_adj, vu_fwd, vu_adj, subs = [], 0.0, 0.0, 0, 0, []
    for it in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        phiT, gT = ck.forward(phi0, times)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        min_free = min(min_free, torch.cuda.mem_get_info()[0])
        d = phiT.astype(np.float64) - target(gT.active_coords())
        hist.append(float((d * d).sum()))
        _, dvel, rec = ck.backward((2.0 * d).astype(np.float32))
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        min_free = min(min_free, torch.cuda.mem_get_info()[0])
        t_fwd += t1 - t0
        t_adj += t2 - t1
        vu_fwd += ck.voxel_updates
        vu_adj += ck.recorded_voxel_updates
        subs.append(ck.substeps)
        gmax = float(dvel.abs().max())
        if gmax > 0:
            v_dev -= (0.05 / gmax) * dvel
        del dvel
        ck.set_velocity(v_dev.cpu().numpy())
        print("iteration %d: L %.6g, %d substeps, forward %.2f s, adjoint %.2f s"
              % (it, hist[-1], ck.substeps, t1 - t0, t2 - t1), file=sys.stderr, flush=True)
    cfg = dict(ADJOINT_WORKLOAD)
    cfg.update({"iterations": args.steps, "active_voxels_initial": int(phi0.size)})
    out = {"metric": "checkpointed adjoint: forward voxel-updates/s, (recorded forward + adjoint) / forward time",
           "forward_value": vu_fwd / t_fwd, "unit": UNIT,
           "adjoint_value": vu_adj / t_adj,
           "cost_ratio": (t_fwd + t_adj) / t_fwd, "forward_s_per_iteration": t_fwd / args.steps,
           "adjoint_s_per_iteration": t_adj / args.steps, "substeps_per_iteration": subs,
           "loss_first": hist[0], "loss_last": hist[-1], "loss": hist,
           "peak_device_gb": (total - min_free) / 1e9, "dtype": "f32", "data": "synthetic (seeded fixtures)",
           "config": cfg}
    print(json.dumps(out))


def cpu_baseline(args):
    """The oracle's CPU restatement of the path on a bounded sample."""
    try:
        from oracle import port
    except ImportError:
        return None
    if not port.available():
        return None
    return port.bench_sample(seconds=args.cpu_seconds)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    try:
        from oracle import port
        ok = port.available()
    except ImportError:
        ok = False
    if not ok:
        print(json.dumps({"impl": "reference", "unavailable": "CPU oracle port not built on this host"}))
        return
    res = port.bench_reference(steps=args.steps, warmup=args.warmup)
    ref_args = argparse.Namespace(**vars(args))
    ref_args.mode = "parity"  # the reference's arithmetic
    out = {"impl": "reference", "metric": METRIC, "value": res["value"], "unit": UNIT, "higher_is_better": True,
           "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["ms_per_step"],
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded fixtures)",
           "config": workload_config(ref_args),
           "run": {"substeps": res["substeps"], "t_start": res["t_start"]},
           "cpu_baseline": res["cpu_baseline"],
           "e2e": {"value": res["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="parity", choices=["fast", "parity"],
                    help="parity: bit-identical to the reference (default); fast: FP32 WENO5 weights")
    ap.add_argument("--cfl", type=float, default=0.5)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-baseline", type=int, default=1)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--extras", type=int, default=1,
                    help="add the 128^3 adjoint cost ratio and the batched 512-instance figures to the line")
    ap.add_argument("--workload", default="sphere64",
                    choices=["sphere64", "batch512", "adjoint512", "fp64errors", "sphere16", "adjoint128"],
                    help="sphere64: the headline 64-sphere line; batch512: the batched configuration; "
                         "adjoint512: the checkpointed inverse problem (--steps = iterations); "
                         "fp64errors: the FP32 run's error against the device FP64 instance, configurations 1-5; "
                         "sphere16 / adjoint128: small cases for ncu captures")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        {"batch512": run_batch, "adjoint512": run_adjoint, "fp64errors": run_fp64_errors,
         "sphere16": run_profile_case, "adjoint128": run_profile_case}.get(args.workload, run_gb300)(args)


if __name__ == "__main__":
    main()
