"""ctypes binding of the native library openvdb_gb300/libgbls.so (include/gbls.h).

The library is built in-tree by openvdb_gb300/build.py.  Loading fails loudly
when it is missing: there is no fallback implementation.
"""
import ctypes as C
import os

from . import _abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgbls.so")
_lib = None


class GblsError(RuntimeError):
    """A gbls_* call returned a non-zero status."""

    def __init__(self, code, msg):
        super().__init__("gbls error %d: %s" % (code, msg))
        self.code = code


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("openvdb_gb300 native library not built (%s); run "
                          "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    P = C.POINTER
    vp = C.c_void_p
    sig = {
        "gbls_abi_version": ([], C.c_int),
        "gbls_last_error": ([], C.c_char_p),
        "gbls_set_device": ([C.c_int], C.c_int),
        "gbls_create": ([P(_abi.GridDesc), P(vp)], C.c_int),
        "gbls_upload": ([vp, P(_abi.GridDesc)], C.c_int),
        "gbls_destroy": ([vp], C.c_int),
        "gbls_get_counts": ([vp, P(_abi.GridCounts)], C.c_int),
        "gbls_download": ([vp, P(_abi.GridDesc)], C.c_int),
        "gbls_set_stream": ([vp, vp], C.c_int),
        "gbls_set_tracker_state": ([vp, C.c_int, C.c_int, C.c_int, C.c_int], C.c_int),
        "gbls_get_tracker_state": ([vp] + [P(C.c_int)] * 4, C.c_int),
        "gbls_set_trimming": ([vp, C.c_int], C.c_int),
        "gbls_set_precision": ([vp, C.c_int], C.c_int),
        "gbls_get_active_values_f64": ([vp, vp], C.c_int),
        "gbls_set_launch_config": ([vp, P(_abi.LaunchConfig)], C.c_int),
        "gbls_volume_advect": ([vp, vp, C.c_int, C.c_int, C.c_int, C.c_double, P(C.c_double)], C.c_int),
        "gbls_create_volume": ([P(_abi.GridDesc), P(vp)], C.c_int),
        "gbls_get_launch_config": ([vp, P(_abi.LaunchConfig)], C.c_int),
        "gbls_time_launch_config": ([vp, vp, P(_abi.LaunchConfig), C.c_int, P(C.c_float)], C.c_int),
        "gbls_set_interrupter": ([vp, P(_abi.Interrupter)], C.c_int),
        "gbls_track": ([vp], C.c_int),
        "gbls_normalize": ([vp], C.c_int),
        "gbls_normalize_masked": ([vp, C.c_int64, vp, vp], C.c_int),
        "gbls_prune": ([vp], C.c_int),
        "gbls_dilate": ([vp, C.c_int], C.c_int),
        "gbls_erode": ([vp, C.c_int], C.c_int),
        "gbls_resize": ([vp, C.c_uint32, P(C.c_int)], C.c_int),
        "gbls_field_create": ([P(_abi.FieldDesc), P(vp)], C.c_int),
        "gbls_field_destroy": ([vp], C.c_int),
        "gbls_advect": ([vp, vp, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float,
                         P(C.c_uint64)], C.c_int),
        "gbls_filter": ([vp, C.c_int, C.c_int, C.c_float], C.c_int),
        "gbls_filter_masked": ([vp, C.c_int, C.c_int, C.c_float, vp, C.c_float, C.c_float, C.c_int], C.c_int),
        "gbls_morph": ([vp, vp, vp, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                        P(C.c_uint64)], C.c_int),
        "gbls_get_stats": ([vp, P(_abi.Stats)], C.c_int),
        "gbls_reset_stats": ([vp], C.c_int),
        "gbls_set_profiling": ([vp, C.c_int], C.c_int),
        "gbls_host_sphere": ([C.c_float, P(C.c_float), C.c_float, C.c_float, P(vp)], C.c_int),
        "gbls_host_union_of_spheres": ([C.c_int64, P(C.c_float), P(C.c_float), C.c_float,
                                        C.c_float, P(vp)], C.c_int),
        "gbls_host_torus": ([C.c_float, C.c_float, P(C.c_float), C.c_float, C.c_float, P(vp)],
                            C.c_int),
        "gbls_batch_create": ([C.c_int32, P(_abi.GridDesc), P(vp)], C.c_int),
        "gbls_batch_instances": ([vp, P(C.c_int32)], C.c_int),
        "gbls_batch_get_counts": ([vp, C.c_int32, P(_abi.GridCounts)], C.c_int),
        "gbls_batch_download": ([vp, C.c_int32, P(_abi.GridDesc)], C.c_int),
        "gbls_batch_advect": ([vp, P(_abi.FieldDesc), C.c_int, C.c_int, C.c_float, C.c_float,
                               C.c_float, P(C.c_uint64)], C.c_int),
        "gbls_count_active_noalloc": ([vp, P(C.c_int64)], C.c_int),
        "gbls_host_grid_view": ([vp, P(_abi.GridDesc)], C.c_int),
        "gbls_host_weno5_exact": ([C.c_int64, P(C.c_float), P(C.c_float), P(C.c_uint8)], C.c_int),
        "gbls_host_weno5_sign": ([C.c_int64, P(C.c_float), P(C.c_int8)], C.c_int),
        "gbls_host_weno5_sign_pair": ([C.c_int64, P(C.c_float), P(C.c_int8), P(C.c_int8)], C.c_int),
        "gbls_weno5_exact_device": ([C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
        "gbls_host_sample_enright": ([vp, C.c_int64, P(C.c_int32), C.c_float, P(C.c_float)], None),
        "gbls_host_grid_free": ([vp], C.c_int),
        "gbls_host_last_error": ([], C.c_char_p),
        "gbls_vdb_write": ([C.c_char_p, C.c_int32, P(_abi.GridDesc), P(C.c_char_p)], C.c_int),
        "gbls_vdb_grid_count": ([C.c_char_p, P(C.c_int32)], C.c_int),
        "gbls_vdb_grid_info": ([C.c_char_p, C.c_int32, C.c_char_p, C.c_int64, C.c_char_p, C.c_int64,
                                C.c_char_p, C.c_int64], C.c_int),
        "gbls_vdb_read": ([C.c_char_p, C.c_char_p, C.c_int32, P(vp)], C.c_int),
        "gbls_nanovdb_export": ([P(_abi.GridDesc), C.c_char_p, C.c_int32, C.c_int32, vp, C.c_int64,
                                 P(C.c_int64)], C.c_int),
        "gbls_nanovdb_import": ([vp, C.c_int64, P(vp)], C.c_int),
        "gbls_nanovdb_export_device": ([vp, C.c_int32, C.c_char_p, C.c_int32, C.c_int32, vp, C.c_int64,
                                        P(C.c_int64)], C.c_int),
        "gbls_nanovdb_export_index_device": ([vp, C.c_int32, C.c_char_p, C.c_int32, C.c_int32, C.c_int32,
                                              C.c_int32, vp, C.c_int64, P(C.c_int64)], C.c_int),
        "gbls_create_from_nanovdb": ([vp, C.c_int64, P(vp)], C.c_int),
        "gbls_nanovdb_probe": ([vp, C.c_int64, vp, C.c_int64, vp, vp, vp, vp], C.c_int),
        "gbls_nanovdb_export_index": ([P(_abi.GridDesc), C.c_char_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                       vp, C.c_int64, P(C.c_int64)], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def check(rc, host=False):
    if rc != 0:
        L = lib()
        msg = (L.gbls_host_last_error() if host else L.gbls_last_error()).decode()
        raise GblsError(rc, msg)
    return rc


def exported_symbols():
    """Names of the gbls_* functions the binding declares."""
    lib()
    return [n for n in dir(_lib) if n.startswith("gbls_")]
