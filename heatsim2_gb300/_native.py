"""ctypes binding of libhs2g.so (the C ABI declared in include/hs2g.h).

There is no CPU fallback: if the library has not been built (``python -m heatsim2_gb300.build``) or cannot be
loaded, every entry point raises ``NativeLibraryError``.
"""
import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_NAME = "libhs2g.so"
LIB_PATH = os.path.join(HERE, LIB_NAME)

# constants mirrored from include/hs2g.h
ABI_VERSION = 1
OK = 0
ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_EXTERIOR, ERR_KTYPE, ERR_UNALIGNED, ERR_FORM, ERR_CAPACITY, ERR_STATE = \
    -1, -2, -3, -4, -5, -6, -7, -8, -9
ERR_TIMEOUT = -10
DEVICE, SYNC, REUSE, SCHEDULED = 1, 2, 4, 8
SHAPED_IMPULSE = 5
K_ENTRIES = 10
FORM_LEN = 1 + 2 * K_ENTRIES
MAX_ZERO_FORMS = 24
MAX_CLASSES = 256

EXPORTED = ("hs2g_abi_version", "hs2g_last_error", "hs2g_create_classes", "hs2g_create_dense", "hs2g_destroy",
            "hs2g_set_stream", "hs2g_shape", "hs2g_step", "hs2g_run", "hs2g_source_table", "hs2g_get_faces",
            "hs2g_device_bytes", "hs2g_run_timed", "hs2g_fp64_fma_rate", "hs2g_step_static",
            "hs2g_batch_create", "hs2g_batch_destroy", "hs2g_batch_layout", "hs2g_batch_device_bytes",
            "hs2g_batch_set_temperature", "hs2g_batch_get_temperature", "hs2g_batch_set_sources",
            "hs2g_batch_set_clock", "hs2g_batch_run", "hs2g_batch_autotune",
            "hs2g_adjoint_create", "hs2g_adjoint_destroy", "hs2g_adjoint_set_stream", "hs2g_adjoint_layout",
            "hs2g_adjoint_device_bytes", "hs2g_adjoint_set_parameters", "hs2g_adjoint_forward",
            "hs2g_adjoint_backward", "hs2g_create_rows", "hs2g_selftest_wait", "hs2g_run_surface",
            "hs2g_surface_temperature", "hs2g_set_source_classes", "hs2g_source_zdecay", "hs2g_source_point",
            "hs2g_adjoint_set_faces", "hs2g_set_schedule", "hs2g_set_clock", "hs2g_get_clock")
STATIC_MAX_VOXELS = 1 << 20


class NativeLibraryError(RuntimeError):
    pass


class Hs2gError(RuntimeError):
    """A failing hs2g_* call; ``code`` is the HS2G_ERR_* value."""

    def __init__(self, code, message):
        super().__init__("%s (hs2g error %d)" % (message, code))
        self.code = code


class Material(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("k", ctypes.c_double * K_ENTRIES), ("capacity", ctypes.c_double)]


class FaceForm(ctypes.Structure):
    _fields_ = [("normal", ctypes.c_double * FORM_LEN), ("nzero", ctypes.c_int32),
                ("zero_code", ctypes.c_int32 * MAX_ZERO_FORMS),
                ("zero", (ctypes.c_double * FORM_LEN) * MAX_ZERO_FORMS)]


class ClassProblem(ctypes.Structure):
    _fields_ = [("nz", ctypes.c_int64), ("ny", ctypes.c_int64), ("nx", ctypes.c_int64),
                ("nmat", ctypes.c_int32), ("nbnd", ctypes.c_int32),
                ("materials", ctypes.POINTER(Material)), ("forms", ctypes.POINTER(FaceForm)),
                ("material", ctypes.c_void_p), ("boundary_z", ctypes.c_void_p), ("boundary_y", ctypes.c_void_p),
                ("boundary_x", ctypes.c_void_p), ("volumetric", ctypes.c_void_p)]


class RowsProblem(ctypes.Structure):
    _fields_ = [("nz", ctypes.c_int64), ("ny", ctypes.c_int64), ("nx", ctypes.c_int64)] + \
               [(n, ctypes.c_void_p) for n in ("zlo", "zhi", "ylo", "yhi", "xlo", "xhi", "capacity", "fixed",
                                               "volumetric")]


class AdjointGrid(ctypes.Structure):
    _fields_ = [("nz", ctypes.c_int64), ("ny", ctypes.c_int64), ("nx", ctypes.c_int64),
                ("dz", ctypes.c_double), ("dy", ctypes.c_double), ("dx", ctypes.c_double)]


class DenseProblem(ctypes.Structure):
    _fields_ = [("nz", ctypes.c_int64), ("ny", ctypes.c_int64), ("nx", ctypes.c_int64),
                ("Gz", ctypes.c_void_p), ("Gy", ctypes.c_void_p), ("Gx", ctypes.c_void_p),
                ("capacity", ctypes.c_void_p), ("fixed", ctypes.c_void_p), ("volumetric", ctypes.c_void_p)]


_lib = None
_lock = threading.Lock()


def lib_path():
    return LIB_PATH


def load():
    """Load libhs2g.so (once) and declare its signatures.  Raises NativeLibraryError when it is missing."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise NativeLibraryError("%s is not built; run `python -m heatsim2_gb300.build` (needs nvcc)" % LIB_PATH)
        try:
            L = ctypes.CDLL(LIB_PATH)
        except OSError as e:
            raise NativeLibraryError("cannot load %s: %s" % (LIB_PATH, e))
        vp, i32, i64, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
        L.hs2g_abi_version.restype = i32
        L.hs2g_last_error.restype = ctypes.c_char_p
        L.hs2g_create_classes.argtypes = [ctypes.POINTER(ClassProblem), i32, ctypes.POINTER(vp)]
        L.hs2g_create_classes.restype = i32
        L.hs2g_create_dense.argtypes = [ctypes.POINTER(DenseProblem), i32, ctypes.POINTER(vp)]
        L.hs2g_create_dense.restype = i32
        L.hs2g_create_rows.argtypes = [ctypes.POINTER(RowsProblem), i32, ctypes.POINTER(vp)]
        L.hs2g_create_rows.restype = i32
        L.hs2g_selftest_wait.argtypes = [i32, i64, i32, ctypes.POINTER(ctypes.c_int)]
        L.hs2g_selftest_wait.restype = i32
        L.hs2g_destroy.argtypes = [vp]
        L.hs2g_destroy.restype = None
        L.hs2g_set_stream.argtypes = [vp, vp]
        L.hs2g_set_stream.restype = i32
        L.hs2g_shape.argtypes = [vp, ctypes.POINTER(ctypes.c_int64)]
        L.hs2g_shape.restype = i32
        L.hs2g_step.argtypes = [vp, vp, vp, vp, vp, vp, i32]
        L.hs2g_step.restype = i32
        L.hs2g_run.argtypes = [vp, i32, vp, vp, vp, i32, vp, i32]
        L.hs2g_run.restype = i32
        L.hs2g_run_surface.argtypes = [vp, i32, vp, vp, vp, dp, vp, i32]
        L.hs2g_run_surface.restype = i32
        L.hs2g_surface_temperature.argtypes = [i32, i64, i64, i64, vp, dp, vp, vp, i32]
        L.hs2g_surface_temperature.restype = i32
        L.hs2g_source_table.argtypes = [i32, vp, vp, dp, dp, dp, vp]
        L.hs2g_source_table.restype = i32
        L.hs2g_set_source_classes.argtypes = [vp, vp, i32]
        L.hs2g_set_source_classes.restype = i32
        L.hs2g_set_schedule.argtypes = [vp, ctypes.c_int64, vp, i32]
        L.hs2g_set_schedule.restype = i32
        L.hs2g_set_clock.argtypes = [vp, ctypes.c_int64]
        L.hs2g_set_clock.restype = i32
        L.hs2g_get_clock.argtypes = [vp, ctypes.POINTER(ctypes.c_int64)]
        L.hs2g_get_clock.restype = i32
        L.hs2g_source_zdecay.argtypes = [vp, i32, vp, dp, dp, dp, dp, dp, dp, i32]
        L.hs2g_source_zdecay.restype = i32
        L.hs2g_source_point.argtypes = [vp, i32, vp, i64, vp, dp, dp, i32]
        L.hs2g_source_point.restype = i32
        L.hs2g_adjoint_set_faces.argtypes = [vp, i32, vp, vp, vp, vp, vp, i32]
        L.hs2g_adjoint_set_faces.restype = i32
        L.hs2g_get_faces.argtypes = [vp, vp, vp, vp, vp, vp]
        L.hs2g_get_faces.restype = i32
        L.hs2g_run_timed.argtypes = [vp, i32, vp, vp, vp, i32, vp]
        L.hs2g_run_timed.restype = i32
        L.hs2g_fp64_fma_rate.argtypes = [i32, vp]
        L.hs2g_fp64_fma_rate.restype = i32
        L.hs2g_step_static.argtypes = [i64, i64, i64, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        L.hs2g_step_static.restype = i32
        L.hs2g_batch_create.argtypes = [i32, ctypes.POINTER(ClassProblem), i32, i32, ctypes.POINTER(vp)]
        L.hs2g_batch_create.restype = i32
        L.hs2g_batch_destroy.argtypes = [vp]
        L.hs2g_batch_destroy.restype = None
        L.hs2g_batch_layout.argtypes = [vp, vp, vp]
        L.hs2g_batch_layout.restype = i32
        L.hs2g_batch_device_bytes.argtypes = [vp]
        L.hs2g_batch_device_bytes.restype = i64
        L.hs2g_batch_set_temperature.argtypes = [vp, vp, i32]
        L.hs2g_batch_set_temperature.restype = i32
        L.hs2g_batch_get_temperature.argtypes = [vp, vp, i32]
        L.hs2g_batch_get_temperature.restype = i32
        L.hs2g_batch_set_sources.argtypes = [vp, i32, i32, vp]
        L.hs2g_batch_set_sources.restype = i32
        L.hs2g_batch_set_clock.argtypes = [vp, i32]
        L.hs2g_batch_set_clock.restype = i32
        L.hs2g_batch_run.argtypes = [vp, i32, i32, ctypes.POINTER(dp)]
        L.hs2g_batch_run.restype = i32
        L.hs2g_batch_autotune.argtypes = [vp, ctypes.c_char_p, i32]
        L.hs2g_batch_autotune.restype = i32
        L.hs2g_adjoint_create.argtypes = [i32, ctypes.POINTER(AdjointGrid), dp, i32, ctypes.POINTER(vp)]
        L.hs2g_adjoint_create.restype = i32
        L.hs2g_adjoint_destroy.argtypes = [vp]
        L.hs2g_adjoint_destroy.restype = None
        L.hs2g_adjoint_set_stream.argtypes = [vp, vp]
        L.hs2g_adjoint_set_stream.restype = i32
        L.hs2g_adjoint_layout.argtypes = [vp, vp]
        L.hs2g_adjoint_layout.restype = i32
        L.hs2g_adjoint_device_bytes.argtypes = [vp]
        L.hs2g_adjoint_device_bytes.restype = i64
        L.hs2g_adjoint_set_parameters.argtypes = [vp, vp, vp, vp, i32]
        L.hs2g_adjoint_set_parameters.restype = i32
        L.hs2g_adjoint_forward.argtypes = [vp, i32, vp, vp, vp, i32, vp, vp, i32, ctypes.POINTER(dp)]
        L.hs2g_adjoint_forward.restype = i32
        L.hs2g_adjoint_backward.argtypes = [vp, vp, vp, vp, vp, i32, ctypes.POINTER(dp)]
        L.hs2g_adjoint_backward.restype = i32
        L.hs2g_device_bytes.argtypes = [vp]
        L.hs2g_device_bytes.restype = i64
        if L.hs2g_abi_version() != ABI_VERSION:
            raise NativeLibraryError("libhs2g ABI version %d, expected %d" % (L.hs2g_abi_version(), ABI_VERSION))
        _lib = L
        return L


def check(rc):
    """Raise Hs2gError for a negative return code; return rc otherwise."""
    if rc < 0:
        msg = _lib.hs2g_last_error().decode(errors="replace") if _lib is not None else "unknown error"
        raise Hs2gError(rc, msg)
    return rc
