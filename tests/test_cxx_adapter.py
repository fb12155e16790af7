"""The C++ drop-in headers (include/openvdb_gb300/LevelSetAdvect.h,
LevelSetTracker.h, LevelSetMorph.h, LevelSetFilter.h, VolumeAdvect.h,
GridExchange.h) compiled against the reference's own
OpenVDB headers and run on the host: grid <-> exchange-format conversion
equal to the library's fixtures, exception mapping, constructor checks and
DiscreteField sampling (tests/cxx/adapter_test.cc).

Needs the reference checkout and the compiled reference oracle
(oracle/_ref/libvdbref.so, which carries the OpenVDB symbols); skipped where
either is absent.
"""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
from oracle.ref.build_ref import reference_root  # noqa: E402

REF = reference_root()
REFLIB = os.path.join(REPO, "oracle", "_ref", "libvdbref.so")


def test_cxx_adapter(tmp_path):
    if not os.path.isfile(os.path.join(REF, "openvdb", "openvdb", "tools", "LevelSetAdvect.h")):
        pytest.skip("reference headers not present")
    if not os.path.exists(REFLIB):
        pytest.skip("oracle/_ref not built")
    from openvdb_gb300 import build
    lib = build.build()
    exe = str(tmp_path / "adapter_test")
    cmd = ["g++", "-std=c++17", "-O1", "-w", "-pthread",
           "-I" + os.path.join(REPO, "oracle", "_ref", "gen"),
           "-I" + os.path.join(REPO, "oracle", "_ref", "gen", "openvdb"),
           "-I" + os.path.join(REPO, "oracle", "ref", "tbbshim"),
           "-I" + os.path.join(REF, "openvdb"), "-I" + os.path.join(REF, "ext", "imath"),
           "-I" + os.path.join(REPO, "include"),
           os.path.join(HERE, "cxx", "adapter_test.cc"), "-o", exe,
           REFLIB, lib, "-Wl,-rpath," + os.path.dirname(REFLIB) + ":" + os.path.dirname(lib)]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, " ".join(cmd) + "\n" + p.stderr[-6000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("ok ") == 11
