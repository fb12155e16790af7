"""The C ABI library loads and exports every function include/*.h declares;
the ctypes mirrors have the C layouts (CPU only, no device calls)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from openvdb_gb300 import _abi
from openvdb_gb300._lib import LIB_PATH, lib

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(REPO, "include")


def declared_functions():
    names = set()
    for f in os.listdir(INCLUDE):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(INCLUDE, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:int|const char\*|void)\s+(gbls_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = C.CDLL(LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    assert len(declared_functions()) >= 25


def test_abi_version():
    assert lib().gbls_abi_version() == _abi.GBLS_ABI_VERSION


def test_struct_layouts_match_c():
    prog = r'''
#include <stdio.h>
#include <stddef.h>
#include "gbls.h"
int main(void) {
  printf("%zu %zu %zu %zu\n", sizeof(gbls_grid_desc), sizeof(gbls_grid_counts), sizeof(gbls_field_desc), sizeof(gbls_interrupter));
  printf("%zu %zu %zu %zu\n", offsetof(gbls_grid_desc, leaf_count), offsetof(gbls_grid_desc, root_tile_values), offsetof(gbls_field_desc, dense_values), offsetof(gbls_field_desc, center));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        open(c, "w").write(prog)
        exe = os.path.join(d, "l")
        subprocess.check_call(["gcc", "-I", INCLUDE, c, "-o", exe])
        out = subprocess.check_output([exe]).decode().split()
    got = [int(x) for x in out]
    want = [C.sizeof(_abi.GridDesc), C.sizeof(_abi.GridCounts), C.sizeof(_abi.FieldDesc),
            C.sizeof(_abi.Interrupter), _abi.GridDesc.leaf_count.offset,
            _abi.GridDesc.root_tile_values.offset, _abi.FieldDesc.dense_values.offset,
            _abi.FieldDesc.center.offset]
    assert got == want


def test_null_arguments_are_rejected_without_a_device():
    L = lib()
    assert L.gbls_create(None, None) == _abi.ERR_INVALID_ARGUMENT
    assert L.gbls_track(None) == _abi.ERR_INVALID_ARGUMENT
    assert L.gbls_destroy(None) == _abi.OK
    assert b"null" in L.gbls_last_error()
