"""Build recipe for the oracle's C++ restatement (oracle/_build/liboracle_port.so).

Test infrastructure: the CPU restatement of the reference path used as the
parity oracle where the compiled reference is unavailable and as the timed
CPU baseline.  Built with -O3 -ffp-contract=off and no -march so it gives
identical bits on x86-64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liboracle_port.so")
SRC = os.path.join(HERE, "port", "levelset_port.cc")


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    deps = [SRC, os.path.join(HERE, "port", "port_impl.h"), os.path.join(HERE, "port", "fixture_port.h"),
            os.path.join(REPO, "include", "gbls.h"),
            os.path.join(REPO, "include", "gbls_fields.h")]
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["g++", "-std=c++17", "-O3", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
           "-I" + os.path.join(REPO, "include"), SRC, "-o", LIB]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode:
        print(" ".join(cmd) + "\n" + p.stderr[-6000:])
        raise RuntimeError("oracle port build failed")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
