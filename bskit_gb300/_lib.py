"""ctypes binding of ``libbskit_gb300.so`` (the C ABI in include/bskit_gb300.h).

The library is the only compute path: there is no CPU fallback.  Importing
this module never needs a GPU, but loading fails loudly when the library has
not been built.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libbskit_gb300.so")

BSK_OK = 0
BSK_ERR_ARG = 1
BSK_ERR_OOM = 2
BSK_ERR_CUDA = 3
BSK_ERR_CUFFT = 4
BSK_ERR_TIMEOUT = 5
BSK_ERR_UNSUPPORTED = 6
BSK_ERR_STATE = 7

PREC_FP64 = 0
PREC_FP32 = 1
PREC_BF16X3 = 2
PREC_BF16 = 3
PRECISIONS = {"fp64": PREC_FP64, "fp32": PREC_FP32, "bf16x3": PREC_BF16X3, "bf16": PREC_BF16}

GRID_REDUCED = 0
GRID_NATIVE = 1
GRID_REDUCED_SINGLE = 2

INFO_NMESH, INFO_NGRID, INFO_NSHELLS, INFO_QMAX, INFO_FOOTPRINT, INFO_CHUNK, INFO_DEVICE, \
    INFO_STREAM = range(8)
INFO_COUNT = 8

# (name, restype, argtypes) for every exported entry point
_VP = ctypes.c_void_p
_I64 = ctypes.c_int64
_INT = ctypes.c_int
SIGNATURES = [
    ("bsk_version", _INT, []),
    ("bsk_last_error", _INT, [ctypes.c_char_p, ctypes.c_size_t]),
    ("bsk_plan_create", _INT, [_INT, ctypes.c_double, _INT, _VP, _INT, ctypes.c_size_t,
                               ctypes.POINTER(_VP)]),
    ("bsk_plan_destroy", _INT, [_VP]),
    ("bsk_plan_query", _INT, [_VP, _VP]),
    ("bsk_shell_mode_counts", _INT, [_VP, _VP]),
    ("bsk_triset_create", _INT, [_VP, _I64, _VP, ctypes.POINTER(_VP)]),
    ("bsk_triset_destroy", _INT, [_VP]),
    ("bsk_triset_size", _I64, [_VP]),
    ("bsk_paint", _INT, [_VP, _INT, _VP, _VP]),
    ("bsk_paint_cic", _INT, [_VP, _INT, _VP, _INT, _VP]),
    ("bsk_triset_schedule", _INT, [_VP, _VP]),
    ("bsk_triset_levels", _INT, [_VP, _VP, _INT]),
    ("bsk_paint_subbox", _INT, [_VP, _INT, _VP, _INT, _INT, _INT, _INT, _VP]),
    ("bsk_compensate_cic", _INT, [_INT, _INT, _VP, _VP, _VP]),
    ("bsk_measure_b", _INT, [_VP, _VP, _INT, _INT, _INT, _INT, _VP, _VP]),
    ("bsk_measure_b_range", _INT, [_VP, _VP, _INT, _INT, _INT, _INT, _I64, _I64, _VP, _VP]),
    ("bsk_gridinfo", _INT, [_VP, _VP, _VP, _VP, _VP]),
    ("bsk_normalize", _INT, [_I64, _VP, _VP, _VP, _VP]),
    ("bsk_contract", _INT, [_VP, _VP, _VP, _VP, _VP, _I64, _INT, _VP, _VP]),
    ("bsk_copy_field", _INT, [_VP, _INT, _INT, _VP, _VP]),
    ("bsk_sync_check", _INT, [_VP]),
    ("bsk_contract_noalloc", _INT, [_INT, _I64, _VP, _VP, _VP, _VP, _I64, _INT, _VP, _VP]),
]

_lib = None


class BskError(RuntimeError):
    """Error status returned by the C ABI; ``code`` is the bsk_status value."""

    def __init__(self, code, msg):
        super().__init__("bskit_gb300 error %d: %s" % (code, msg))
        self.code = code


def load():
    """Load the shared library (once) and declare the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            "libbskit_gb300.so is not built (expected at %s); run "
            "`python -m bskit_gb300.build` -- there is no CPU fallback" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error():
    buf = ctypes.create_string_buffer(1024)
    load().bsk_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


class BskArgumentError(BskError, ValueError):
    """BSK_ERR_ARG: the cases bskit raises ValueError for."""


def check(status):
    if status == BSK_ERR_ARG:
        raise BskArgumentError(status, last_error())
    if status != BSK_OK:
        raise BskError(status, last_error())
    return status


def call(name, *args):
    return check(getattr(load(), name)(*args))
