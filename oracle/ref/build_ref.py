#!/usr/bin/env python3
"""Build recipe for the reference oracle (oracle/_ref/libvdbref.so).

Compiles the UNMODIFIED OpenVDB level-set advection path from the reference
checkout in place (nothing is copied into this repository) together with
oracle/ref/ref_harness.cc and the project-written TBB-API shim in
oracle/ref/tbbshim.  Outputs go only to oracle/_ref/ (git-ignored).

Steps:
  1. configure openvdb/openvdb/version.h.in -> oracle/_ref/gen/openvdb/version.h
     (ABI 13, no Blosc/zlib/delayed loading/Imath, no explicit instantiation,
     x86 instruction set 0 so the same source builds on aarch64);
  2. compile the minimal .cc set the path links against plus the harness with
     -O3 -ffp-contract=off (no -march), so x86 and aarch64 agree bitwise;
  3. link a shared library.

The reference checkout is found at $GBLS_REFERENCE_ROOT or /root/reference.
Without it the script exits with status 2 and builds nothing.
"""
import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
REPO = os.path.dirname(ORACLE)
OUT = os.path.join(ORACLE, "_ref")

REF_SOURCES = [
    "openvdb/openvdb/Grid.cc",
    "openvdb/openvdb/Metadata.cc",
    "openvdb/openvdb/MetaMap.cc",
    "openvdb/openvdb/Platform.cc",
    "openvdb/openvdb/math/Maps.cc",
    "openvdb/openvdb/math/Transform.cc",
    "openvdb/openvdb/util/Formats.cc",
    "openvdb/openvdb/util/Assert.cc",
    "ext/imath/openvdb/math/Half.cc",
    "openvdb/openvdb/io/Compression.cc",
    "openvdb/openvdb/io/GridDescriptor.cc",
]


def reference_root():
    return os.environ.get("GBLS_REFERENCE_ROOT", "/root/reference")


def configure_version_header(ref):
    cm = open(os.path.join(ref, "CMakeLists.txt")).read()
    ver = {}
    for key in ("MAJOR", "MINOR", "PATCH"):
        m = re.search(r"set\(OpenVDB_%s_VERSION (\d+)\)" % key, cm)
        ver[key] = int(m.group(1))
    text = open(os.path.join(ref, "openvdb/openvdb/version.h.in")).read()
    subs = {
        "${OpenVDB_MAJOR_VERSION}": str(ver["MAJOR"]),
        "${OpenVDB_MINOR_VERSION}": str(ver["MINOR"]),
        "${OpenVDB_PATCH_VERSION}": str(ver["PATCH"]),
        "${OPENVDB_ABI_VERSION_NUMBER}": str(ver["MAJOR"]),
        "${OPENVDB_PACKED_VERSION}": str((ver["MAJOR"] << 24) | (ver["MINOR"] << 16) | ver["PATCH"]),
        "${OPENVDB_NAMESPACE_SUFFIX}": "",
        "${OPENVDB_X86_INSTRSET}": "0",
    }
    for k, v in subs.items():
        text = text.replace(k, v)
    text = re.sub(r"@[A-Z_]+@", "", text)
    text = re.sub(r"#cmakedefine (\w+)", r"/* #undef \1 */", text)
    dst = os.path.join(OUT, "gen", "openvdb")
    os.makedirs(dst, exist_ok=True)
    path = os.path.join(dst, "version.h")
    if not os.path.exists(path) or open(path).read() != text:
        with open(path, "w") as f:
            f.write(text)


def build(verbose=False):
    ref = reference_root()
    if not os.path.isfile(os.path.join(ref, "openvdb/openvdb/tools/LevelSetAdvect.h")):
        print("reference checkout not found at %s; oracle/_ref not built" % ref)
        return 2
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    configure_version_header(ref)
    flags = [
        "-std=c++17", "-O3", "-ffp-contract=off", "-fPIC", "-w",
        "-DOPENVDB_USE_DELAYED_LOADING=0",
        "-I" + os.path.join(OUT, "gen"),
        "-I" + os.path.join(OUT, "gen", "openvdb"),
        "-I" + os.path.join(HERE, "tbbshim"),
        "-I" + os.path.join(ref, "openvdb"),
        "-I" + os.path.join(ref, "ext/imath"),
        "-I" + os.path.join(ref, "nanovdb"),
        "-I" + os.path.join(REPO, "include"),
        "-pthread",
    ]
    flags = [f for f in flags if not f.startswith("-DOPENVDB_USE_DELAYED")]
    srcs = [os.path.join(ref, s) for s in REF_SOURCES] + [os.path.join(HERE, "ref_harness.cc"),
                                                       os.path.join(HERE, "io_stubs.cc"),
                                                       os.path.join(HERE, "nano_harness.cc")]
    hdr_deps = [os.path.join(HERE, "ref_harness.cc"), os.path.join(REPO, "include", "gbls.h"),
                os.path.join(REPO, "include", "gbls_fields.h")]

    def obj_of(src):
        name = os.path.relpath(src, ref) if src.startswith(ref) else os.path.basename(src)
        return os.path.join(OUT, "obj", name.replace("/", "_") + ".o")

    def compile_one(src):
        obj = obj_of(src)
        deps = [src] + (hdr_deps if src.endswith("ref_harness.cc") else [])
        if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
            return 0, ""
        cmd = ["g++"] + flags + ["-c", src, "-o", obj]
        p = subprocess.run(cmd, capture_output=True, text=True)
        return p.returncode, (" ".join(cmd) + "\n" + p.stderr) if p.returncode else ""

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        results = list(ex.map(compile_one, srcs))
    for rc, msg in results:
        if rc:
            print(msg[-8000:])
            return 1
    lib = os.path.join(OUT, "libvdbref.so")
    objs = [obj_of(s) for s in srcs]
    if not os.path.exists(lib) or any(os.path.getmtime(o) > os.path.getmtime(lib) for o in objs):
        cmd = ["g++", "-shared", "-pthread", "-o", lib] + objs
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode:
            print(p.stderr[-8000:])
            return 1
    if verbose:
        print("built", lib)
    return 0


if __name__ == "__main__":
    sys.exit(build(verbose=True))
