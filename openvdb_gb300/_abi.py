"""ctypes mirror of include/gbls.h (structures and constants).

Field order and types must match the C declarations exactly; the layout is
checked against the compiled library in tests/test_abi.py.
"""
import ctypes as C

GBLS_ABI_VERSION = 4

# status codes
OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_VALUE = 2
ERR_RUNTIME = 3
ERR_CUDA = 4
ERR_OUT_OF_MEMORY = 5
ERR_INTERRUPTED = 6
ERR_DOMAIN = 7
ERR_UNSUPPORTED = 8
ERR_DEVICE_CHECK = 9

# math::BiasedGradientScheme (math/FiniteDifference.h:164-171)
FIRST_BIAS, SECOND_BIAS, THIRD_BIAS, WENO5_BIAS, HJWENO5_BIAS = 0, 1, 2, 3, 4
# math::TemporalIntegrationScheme (math/FiniteDifference.h:233-238)
TVD_RK1, TVD_RK2, TVD_RK3 = 0, 1, 2
# lstrack::TrimMode (tools/LevelSetTracker.h:45-50)
TRIM_NONE, TRIM_INTERIOR, TRIM_EXTERIOR, TRIM_ALL = 0, 1, 2, 3
MODE_PARITY, MODE_FAST, MODE_FP64 = 0, 1, 2
MAP_UNIFORM_SCALE, MAP_UNIFORM_SCALE_TRANSLATE, MAP_TRANSLATION = 0, 1, 2
FIELD_CONSTANT, FIELD_DENSE, FIELD_DEFORMATION, FIELD_ROTATION, FIELD_HOST_SAMPLED = 0, 1, 2, 3, 4


class GridDesc(C.Structure):
    _fields_ = [
        ("voxel_size", C.c_double),
        ("translation", C.c_double * 3),
        ("map_type", C.c_int32),
        ("background", C.c_float),
        ("leaf_count", C.c_int64),
        ("leaf_origins", C.POINTER(C.c_int32)),
        ("leaf_masks", C.POINTER(C.c_uint64)),
        ("leaf_values", C.POINTER(C.c_float)),
        ("lower_count", C.c_int64),
        ("lower_origins", C.POINTER(C.c_int32)),
        ("lower_tiles", C.POINTER(C.c_float)),
        ("upper_count", C.c_int64),
        ("upper_origins", C.POINTER(C.c_int32)),
        ("upper_tiles", C.POINTER(C.c_float)),
        ("root_tile_count", C.c_int64),
        ("root_tile_origins", C.POINTER(C.c_int32)),
        ("root_tile_values", C.POINTER(C.c_float)),
    ]


class GridCounts(C.Structure):
    _fields_ = [
        ("leaf_count", C.c_int64),
        ("lower_count", C.c_int64),
        ("upper_count", C.c_int64),
        ("root_tile_count", C.c_int64),
        ("active_voxel_count", C.c_int64),
        ("background", C.c_float),
    ]


class FieldDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("constant", C.c_float * 3),
        ("dense_origin", C.c_int32 * 3),
        ("dense_dims", C.c_int32 * 3),
        ("dense_values", C.POINTER(C.c_float)),
        ("dense_background", C.c_float * 3),
        ("domain", C.c_float),
        ("period", C.c_float),
        ("scale", C.c_float),
        ("omega", C.c_float * 3),
        ("center", C.c_float * 3),
        ("dense_map_type", C.c_int32),
        ("dense_voxel_size", C.c_double),
        ("dense_translation", C.c_double * 3),
        ("host_sample", C.c_void_p),
        ("host_user", C.c_void_p),
    ]


class LaunchConfig(C.Structure):
    """gbls_launch_config: launch shapes of the stencil and CFL kernels."""
    _fields_ = [("stencil_min_ctas_rk", C.c_int32), ("stencil_min_ctas_norm", C.c_int32),
                ("cfl_leaves_per_block", C.c_int32), ("rk_ctas_per_leaf", C.c_int32)]


class HostMap(C.Structure):
    """gbls_host_map: index -> world, x * scale + translation."""
    _fields_ = [("scale", C.c_double), ("translation", C.c_double * 3)]


# gbls_host_sample_fn: (user, n, ijk[n][3] int32, t, velocity[n][3] float)
HOST_SAMPLE = C.CFUNCTYPE(None, C.c_void_p, C.c_int64, C.POINTER(C.c_int32), C.c_float, C.POINTER(C.c_float))


INTERRUPT_START = C.CFUNCTYPE(None, C.c_void_p, C.c_char_p)
INTERRUPT_END = C.CFUNCTYPE(None, C.c_void_p)
INTERRUPT_CHECK = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int)


class Interrupter(C.Structure):
    _fields_ = [
        ("start", INTERRUPT_START),
        ("end", INTERRUPT_END),
        ("was_interrupted", INTERRUPT_CHECK),
        ("user", C.c_void_p),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("substeps", C.c_uint64),
        ("voxel_updates", C.c_uint64),
        ("kernel_launches", C.c_uint64),
        ("rk_launches", C.c_uint64),
        ("norm_launches", C.c_uint64),
        ("rk_ms", C.c_double),
        ("norm_ms", C.c_double),
        ("rk_bytes", C.c_double),
        ("norm_bytes", C.c_double),
        ("dilated_voxels", C.c_uint64),
        ("active_voxels", C.c_int64),
        ("leaves", C.c_int64),
    ]
