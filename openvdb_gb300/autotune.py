"""Launch-shape autotuner for the advection kernels (no reference counterpart).

Four launch parameters change speed, not results (gbls_launch_config): the
register budget of the PARITY RK-stage and renormalisation kernels, given as
the minimum resident 64-thread CTAs per SM (0 = none, the compiler's
heuristic; 1 = unconstrained; 14 or 16), the leaves per CTA of the CFL
maximum (8, 16, 32 or 64), and the CTAs per leaf of the PARITY RK stage (1,
2 or 4: each CTA stages the whole leaf and takes every k-th group of 64
active voxels, more parallelism where a level set has few leaves).  Each
parameter drives one kernel, so the search is coordinate-wise:
gbls_time_launch_config times one RK stage, one renormalisation stage and one
CFL maximum of the handle's current level set under each candidate, and the
fastest value per parameter wins.  The choice is cached per device, precision
mode and workload size class (log2 of the leaf count) in a JSON file:
$GBLS_TUNE_CACHE, else ~/.cache/openvdb_gb300/launch_config.json.

The renormalisation kernel keeps one leaf per CTA (its output layout needs
every voxel's result of the leaf), and the staging depth is one leaf: a
persistent, software-pipelined stencil kernel with deeper staging was
measured slower.
"""
import ctypes as C
import json
import math
import os

from . import _abi
from ._lib import lib

CANDIDATES = {
    "stencil_min_ctas_rk": (0, 1, 14, 16),
    "stencil_min_ctas_norm": (0, 1, 14, 16),
    "cfl_leaves_per_block": (8, 16, 32, 64),
    "rk_ctas_per_leaf": (1, 2, 4),
}
DEFAULT = {"stencil_min_ctas_rk": 0, "stencil_min_ctas_norm": 0, "cfl_leaves_per_block": 32, "rk_ctas_per_leaf": 1}
# which of the three timed kernels each parameter drives
_TIMED = {"stencil_min_ctas_rk": 0, "stencil_min_ctas_norm": 1, "cfl_leaves_per_block": 2, "rk_ctas_per_leaf": 0}


def _check(rc):
    if rc != 0:
        raise RuntimeError("gbls error %d: %s" % (rc, lib().gbls_last_error().decode()))


def _struct(cfg):
    c = _abi.LaunchConfig()
    for k in DEFAULT:
        setattr(c, k, int(cfg[k]))
    return c


def get(handle):
    c = _abi.LaunchConfig()
    _check(lib().gbls_get_launch_config(handle, C.byref(c)))
    return {k: int(getattr(c, k)) for k in DEFAULT}


def apply(handle, cfg):
    _check(lib().gbls_set_launch_config(handle, C.byref(_struct(cfg))))


def time_config(handle, field_handle, cfg, reps=5):
    """Mean ms per launch of (RK stage, renormalisation stage, CFL maximum)."""
    ms = (C.c_float * 3)()
    _check(lib().gbls_time_launch_config(handle, field_handle, C.byref(_struct(cfg)), int(reps), ms))
    return [float(x) for x in ms]


def cache_path():
    return os.environ.get("GBLS_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "openvdb_gb300",
                                                             "launch_config.json")


def _device_name():
    try:
        import torch
        return torch.cuda.get_device_name(torch.cuda.current_device())
    except Exception:
        return "cuda"


def cache_key(mode, leaf_count):
    return "%s|mode=%d|leaves=2^%d" % (_device_name(), int(mode), max(0, int(math.log2(max(1, leaf_count)))))


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(db):
    p = cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + ".tmp"
        with open(tmp, "w") as f:
            json.dump(db, f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass  # a read-only home: the choice still applies to this handle


def tune(handle, field_handle, mode, leaf_count, reps=5, use_cache=True):
    """Choose and apply the launch configuration for this handle's workload.
    Returns {"config": ..., "source": "cache" | "search", "timings_ms": ...}."""
    key = cache_key(mode, leaf_count)
    db = _load() if use_cache else {}
    if use_cache and key in db:
        cfg = {k: int(db[key]["config"].get(k, DEFAULT[k])) for k in DEFAULT}
        apply(handle, cfg)
        return {"config": cfg, "source": "cache", "key": key}
    cfg = dict(DEFAULT)
    timings = {}
    for name, values in CANDIDATES.items():
        best, best_ms = None, None
        for v in values:
            trial = dict(cfg)
            trial[name] = v
            t = time_config(handle, field_handle, trial, reps)[_TIMED[name]]
            timings["%s=%d" % (name, v)] = t
            if best_ms is None or t < best_ms:
                best, best_ms = v, t
        cfg[name] = best
    apply(handle, cfg)
    if use_cache:
        db = _load()
        db[key] = {"config": cfg, "timings_ms": timings}
        _store(db)
    return {"config": cfg, "source": "search", "key": key, "timings_ms": timings}
