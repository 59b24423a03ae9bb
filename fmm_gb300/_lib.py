"""ctypes binding of the C ABI declared in include/fmm_gpu.h.

The shared library is built in-tree (fmm_gb300/_build/libfmm_gb300.so) by
``fmm_gb300.build``.  There is no CPU fallback: if the library is missing or
cannot be loaded, importing this module's ``lib()`` raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfmm_gb300.so")

# status codes (include/fmm_gpu.h)
FMM_OK = 0
FMM_EINVAL = -1
FMM_ENOTSUP = -2
FMM_ENOMEM = -3
FMM_ECUDA = -4
FMM_EDEPTH = -5
FMM_EORDER = -6
FMM_ETIMEOUT = -7


class FmmOpts(ctypes.Structure):
    """Mirror of ``struct fmm_opts``."""

    _fields_ = [
        ("version", ctypes.c_int),
        ("coef_mode", ctypes.c_int),
        ("excl_mode", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("centroid_mode", ctypes.c_int),
        ("mac_mode", ctypes.c_int),
        ("selector", ctypes.c_int),
        ("target_rel_err", ctypes.c_double),
        ("stream", ctypes.c_void_p),
        ("autotune", ctypes.c_int),
        ("reserved", ctypes.c_int * 7),
    ]


# every symbol include/fmm_gpu.h declares
EXPORTED = [
    "fmm_field_direct",
    "fmm_field_fmm",
    "fmm_field_direct_device",
    "fmm_field_fmm_device",
    "fmm_field_fmm_batched",
    "fmm_field_direct_targets_device",
    "fmm_field_direct_targets_noalloc",
    "fmm_last_stats",
    "fmm_release_workspace",
    "fmm_get_boxes",
    "fmm_get_multipoles",
    "fmm_interpolate_electron_fields",
    "fmm_debug_tree",
    "fmm_measure_fma_peak",
    "fmm_launch_count",
    "fmm_selector_load",
    "fmm_selector_param_count",
    "fmm_mlp_param_count",
    "fmm_mlp_forward",
    "fmm_mlp_grad",
    "fmm_mlp_train",
    "fmm_selector_collect",
    "fmm_set_p2p_shape",
    "fmm_plan_create",
    "fmm_plan_create_batched",
    "fmm_plan_execute",
    "fmm_plan_execute_device",
    "fmm_plan_kernels",
    "fmm_plan_destroy",
    "fmm_strerror",
    "fmm_version",
]

_lib = None


class FmmError(RuntimeError):
    def __init__(self, status, what):
        self.status = status
        super().__init__("%s failed: %s (status %d)" % (what, strerror(status), status))


def lib():
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("fmm_gb300 CUDA library not built: %s is missing "
                          "(run `python -m fmm_gb300.build`)" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    d = ctypes.POINTER(ctypes.c_double)
    i32 = ctypes.POINTER(ctypes.c_int32)
    i64 = ctypes.c_int64
    c = ctypes.c_int
    cs = ctypes.c_char_p
    op = ctypes.POINTER(FmmOpts)
    L.fmm_field_direct.argtypes = [c, i64, d, c, d, c, i32, c, d, cs, c, d, op]
    L.fmm_field_fmm.argtypes = [c, i64, d, c, d, c, i32, ctypes.c_double, c, c, c, d, cs, c, d, c, d, op]
    L.fmm_field_direct_device.argtypes = [i64, ctypes.c_void_p, c, ctypes.c_void_p, c, ctypes.c_void_p, c,
                                          ctypes.c_void_p, cs, c, ctypes.c_void_p, op]
    L.fmm_field_fmm_device.argtypes = [i64, ctypes.c_void_p, c, ctypes.c_void_p, c, ctypes.c_void_p,
                                       ctypes.c_double, c, c, c, ctypes.c_void_p, cs, c, ctypes.c_void_p, op]
    L.fmm_field_direct_targets_device.argtypes = [i64, ctypes.c_void_p, c, ctypes.c_void_p, c, ctypes.c_void_p,
                                                  i64, ctypes.c_void_p, c, ctypes.c_void_p, cs, c,
                                                  ctypes.c_void_p, op]
    L.fmm_field_direct_targets_noalloc.argtypes = L.fmm_field_direct_targets_device.argtypes
    L.fmm_field_fmm_batched.argtypes = [c, ctypes.POINTER(ctypes.c_int64), d, c, d, c, i32, ctypes.c_double, c, c, c,
                                        d, cs, c, d, op]
    L.fmm_field_fmm_batched.restype = c
    L.fmm_last_stats.argtypes = [d, c]
    L.fmm_release_workspace.argtypes = []
    i64p = ctypes.POINTER(ctypes.c_int64)
    vp = ctypes.c_void_p
    L.fmm_get_boxes.argtypes = [i64, d, i64, d, ctypes.c_double, c, c, i64p, vp, vp, vp, op]
    L.fmm_get_boxes.restype = c
    L.fmm_get_multipoles.argtypes = [c, i64, d, c, c, d, i64, d, ctypes.c_double, c, c, i64p, vp, vp, vp, op]
    L.fmm_get_multipoles.restype = c
    L.fmm_interpolate_electron_fields.argtypes = [c, i64, d, i64, c, d, vp, ctypes.c_double, c, c, c, d, op]
    L.fmm_interpolate_electron_fields.restype = c
    L.fmm_release_workspace.restype = c
    L.fmm_set_p2p_shape.argtypes = [c, c, c]
    L.fmm_set_p2p_shape.restype = c
    L.fmm_plan_create.argtypes = [i64, d, c, c, i32, ctypes.c_double, c, c, c, cs, c, d, op,
                                  ctypes.POINTER(ctypes.c_void_p)]
    L.fmm_plan_create.restype = c
    L.fmm_plan_create_batched.argtypes = [c, ctypes.POINTER(ctypes.c_int64), d, c, c, i32, ctypes.c_double, c, c, c,
                                          cs, c, d, op, ctypes.POINTER(ctypes.c_void_p)]
    L.fmm_plan_create_batched.restype = c
    L.fmm_plan_execute.argtypes = [ctypes.c_void_p, d, d]
    L.fmm_plan_execute.restype = c
    L.fmm_plan_execute_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.fmm_plan_execute_device.restype = c
    L.fmm_plan_kernels.argtypes = [ctypes.c_void_p]
    L.fmm_plan_kernels.restype = c
    L.fmm_plan_destroy.argtypes = [ctypes.c_void_p]
    L.fmm_plan_destroy.restype = None
    L.fmm_measure_fma_peak.argtypes = [c, d]
    L.fmm_launch_count.restype = ctypes.c_int64
    L.fmm_launch_count.argtypes = []
    L.fmm_strerror.restype = ctypes.c_char_p
    L.fmm_strerror.argtypes = [c]
    L.fmm_version.restype = ctypes.c_char_p
    for name in ("fmm_field_direct", "fmm_field_fmm", "fmm_field_direct_device", "fmm_field_fmm_device",
                 "fmm_field_direct_targets_device", "fmm_field_direct_targets_noalloc", "fmm_last_stats",
                 "fmm_measure_fma_peak"):
        getattr(L, name).restype = c
    _lib = L
    return L


def strerror(status):
    try:
        return lib().fmm_strerror(int(status)).decode()
    except ImportError:
        return "status %d" % status


def check(status, what):
    if status != FMM_OK:
        raise FmmError(status, what)
