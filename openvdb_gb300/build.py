"""Build the in-tree native library openvdb_gb300/libgbls.so.

CUDA sources are compiled for sm_103a only; the parity-mode stencil unit is
compiled with -fmad=false, and every host unit with -ffp-contract=off so host
float arithmetic (CFL time steps, fixture rasterisation) rounds identically on
x86-64 and aarch64.  Incremental: a unit is rebuilt when it or any header of
the package or include/ is newer than its object.
"""
import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbls.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I" + os.path.join(REPO, "include")]
CXX_FLAGS = ["-std=c++17", "-O3", "-fPIC", "-ffp-contract=off", "-pthread",
             "-I" + os.path.join(REPO, "include")]
PER_UNIT = {"stencil_parity.cu": ["-fmad=false"], "stencil_exact.cu": ["-fmad=false"], "volume.cu": ["-fmad=false"],
            "nanovdb_device.cu": ["-fmad=false"], "stencil_f64.cu": ["-fmad=false"]}


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
            + glob.glob(os.path.join(REPO, "include", "*.h")))


def build(verbose=False, force=False):
    os.makedirs(OBJ, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cc")))
    hdr_time = max([os.path.getmtime(h) for h in _headers()] + [os.path.getmtime(__file__)])
    nvcc = _nvcc()

    def unit(src):
        name = os.path.basename(src)
        obj = os.path.join(OBJ, name + ".o")
        if (not force and os.path.exists(obj)
                and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_time)):
            return obj, 0, ""
        if src.endswith(".cu"):
            cmd = [nvcc] + ARCH + NVCC_FLAGS + PER_UNIT.get(name, []) + ["-c", src, "-o", obj]
        else:
            cmd = ["g++"] + CXX_FLAGS + ["-c", src, "-o", obj]
        p = subprocess.run(cmd, capture_output=True, text=True)
        msg = p.stdout + p.stderr
        return obj, p.returncode, (" ".join(cmd) + "\n" + msg) if (p.returncode or verbose) else ""

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        results = list(ex.map(unit, srcs))
    for obj, rc, msg in results:
        if msg and (rc or verbose):
            print(msg[-6000:])
        if rc:
            raise RuntimeError("compilation failed: " + obj)
    objs = [r[0] for r in results]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode:
            print(p.stdout + p.stderr)
            raise RuntimeError("link failed")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
