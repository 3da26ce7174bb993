"""ctypes binding of libphcuda.so (the C-ABI declared in include/phcuda.h).

This module is the Python twin of the Crystal `lib LibPhCuda` block that a
`Phase::CuNArray` would use.  Loading fails loudly when the shared library has
not been built: there is no CPU fallback anywhere in this package.
"""
import ctypes
import os

from . import errors

MAX_RANK = 8
MAX_INPUTS = 4
MAX_INSTR = 24

# element types
BOOL, I32, I64, F32, F64 = 0, 1, 2, 3, 4
DTYPE_NAMES = {BOOL: "Bool", I32: "Int32", I64: "Int64", F32: "Float32", F64: "Float64"}
DTYPE_SIZE = {BOOL: 1, I32: 4, I64: 8, F32: 4, F64: 8}
# an index operand (an input whose Int32 value is offset + coordinate . stride)
INDEX = 5

# status codes
OK = 0
ERR_SHAPE, ERR_DIM, ERR_INDEX, ERR_OVERFLOW, ERR_DIVZERO, ERR_ARGUMENT = 1, 2, 3, 4, 5, 6
ERR_UNBOUNDED, ERR_EMPTY, ERR_UNSUPPORTED, ERR_OOM, ERR_TIMEOUT, ERR_CUDA = 7, 8, 9, 10, 11, 12
ERR_OOB, ERR_INVALID, ERR_NOT_INIT = 13, 14, 15

ST_OVERFLOW, ST_DIVZERO, ST_ARGUMENT, ST_TIMEOUT, ST_OOB = 1, 2, 4, 8, 16

# binary operators (order of src/multi_indexable.cr:958-981)
(OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_FLOORDIV, OP_MOD, OP_POW, OP_WADD, OP_WSUB, OP_WMUL, OP_WPOW,
 OP_AND, OP_OR, OP_XOR, OP_GT, OP_LT, OP_GE, OP_LE, OP_CMP, OP_EQ) = range(20)
UOP_POS, UOP_NEG, UOP_NOT = 0, 1, 2
RED_SUM, RED_MAX, RED_MIN, RED_ARGMAX, RED_ARGMIN = 0, 1, 2, 3, 4

I_LD, I_ST0, I_ST1, I_CVT, I_NEG, I_NOT, I_POS, I_SEL = 64, 65, 66, 67, 68, 69, 70, 71
SRC_IMM, SRC_S0, SRC_S1 = 8, 9, 10

TASK_EVAL, TASK_REDUCE = 0, 1

TUNE_FEATURES = 24
MLP_H1 = 64
MLP_H2 = 64
MLP_PARAMS = MLP_H1 * TUNE_FEATURES + MLP_H1 + MLP_H2 * MLP_H1 + MLP_H2 + MLP_H2 + 1


class View(ctypes.Structure):
    _fields_ = [
        ("base", ctypes.c_void_p),
        ("dtype", ctypes.c_int32),
        ("rank", ctypes.c_int32),
        ("offset", ctypes.c_int64),
        ("shape", ctypes.c_int64 * MAX_RANK),
        ("stride", ctypes.c_int64 * MAX_RANK),
    ]


class _Imm(ctypes.Union):
    _fields_ = [("f", ctypes.c_double), ("i", ctypes.c_int64)]


class Instr(ctypes.Structure):
    _fields_ = [
        ("op", ctypes.c_uint8),
        ("src", ctypes.c_uint8),
        ("type", ctypes.c_uint8),
        ("btype", ctypes.c_uint8),
        ("flags", ctypes.c_uint8),
        ("pad", ctypes.c_uint8 * 3),
        ("imm", _Imm),
    ]


class Program(ctypes.Structure):
    _fields_ = [
        ("n_instr", ctypes.c_int32),
        ("out_type", ctypes.c_int32),
        ("code", Instr * MAX_INSTR),
    ]


class Scalar(ctypes.Structure):
    _fields_ = [("dtype", ctypes.c_int32), ("pad", ctypes.c_int32), ("v", _Imm)]


class Task(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("red_op", ctypes.c_int32),
        ("axis", ctypes.c_int32),
        ("n_inputs", ctypes.c_int32),
        ("prog", ctypes.c_int32),
        ("chunk", ctypes.c_int32),
        ("layout", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("inp", View * MAX_INPUTS),
        ("out", View),
    ]


def _lib_path():
    here = os.path.dirname(os.path.abspath(__file__))
    return os.path.join(here, "_lib", "libphcuda.so")


_lib = None

# (name, argtypes)
_P = ctypes.POINTER
_vp = ctypes.c_void_p
_SIGS = [
    ("phcu_init", [ctypes.c_int32]),
    ("phcu_shutdown", []),
    ("phcu_set_stream", [_vp]),
    ("phcu_get_stream", [_P(_vp)]),
    ("phcu_sync", []),
    ("phcu_last_error", [ctypes.c_char_p, ctypes.c_size_t]),
    ("phcu_status_word", [_P(ctypes.c_uint32), ctypes.c_int32]),
    ("phcu_version", [_P(ctypes.c_int32), _P(ctypes.c_int32)]),
    ("phcu_device_info", [_P(ctypes.c_int32), _P(ctypes.c_int64), _P(ctypes.c_int32), _P(ctypes.c_int32)]),
    ("phcu_alloc", [ctypes.c_size_t, _P(_vp)]),
    ("phcu_free", [_vp]),
    ("phcu_host_alloc", [ctypes.c_size_t, _P(_vp)]),
    ("phcu_host_free", [_vp]),
    ("phcu_upload", [_vp, _vp, ctypes.c_size_t]),
    ("phcu_download", [_vp, _vp, ctypes.c_size_t]),
    ("phcu_download_async", [_vp, _vp, ctypes.c_size_t]),
    ("phcu_upload_async", [_vp, _vp, ctypes.c_size_t]),
    ("phcu_transfer_wait", []),
    ("phcu_memset", [_vp, ctypes.c_int32, ctypes.c_size_t]),
    ("phcu_copy", [_P(View), _P(View)]),
    ("phcu_fill", [_P(View), _P(Scalar)]),
    ("phcu_eval", [_P(Program), _P(View), ctypes.c_int32, _P(View)]),
    ("phcu_binary", [ctypes.c_int32, _P(View), _P(View), _P(View)]),
    ("phcu_binary_scalar", [ctypes.c_int32, _P(View), _P(Scalar), ctypes.c_int32, _P(View)]),
    ("phcu_unary", [ctypes.c_int32, _P(View), _P(View)]),
    ("phcu_result_dtype", [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _P(ctypes.c_int32)]),
    ("phcu_reduce", [ctypes.c_int32, _P(View), ctypes.c_int32, _P(View)]),
    ("phcu_reduce_noalloc", [ctypes.c_int32, _P(View), ctypes.c_int32, _P(View)]),
    ("phcu_heat_step", [_vp, _vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_float]),
    ("phcu_heat_run", [_vp, _vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_float, ctypes.c_int32, ctypes.c_int32]),
    ("phcu_heat_run_f64", [_vp, _vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_double, ctypes.c_int32,
                           ctypes.c_int32]),
    ("phcu_graph_begin", []),
    ("phcu_graph_end", [_P(_vp)]),
    ("phcu_graph_launch", [_vp]),
    ("phcu_graph_destroy", [_vp]),
    ("phcu_timer_start", [_P(_vp)]),
    ("phcu_timer_stop", [_vp, _P(ctypes.c_float)]),
    ("phcu_launch_count", [_P(ctypes.c_uint64)]),
    ("phcu_l2_flush", []),
    ("phcu_batch_prepare", [_P(Task), ctypes.c_int32, _P(Program), ctypes.c_int32, _P(_vp)]),
    ("phcu_batch_launch", [_vp, ctypes.c_int32]),
    ("phcu_batch_info", [_vp, _P(ctypes.c_int64), _P(ctypes.c_int64), _P(ctypes.c_int64)]),
    ("phcu_batch_destroy", [_vp]),
    ("phcu_batch_run", [_P(Task), ctypes.c_int32, _P(Program), ctypes.c_int32, ctypes.c_int32]),
    ("phcu_tune_n_configs", [_P(ctypes.c_int32)]),
    ("phcu_tune_features", [_P(Task), ctypes.c_int32, _P(ctypes.c_float)]),
    ("phcu_tune_measure", [_P(Task), _P(Program), ctypes.c_int32, _P(ctypes.c_float)]),
    ("phcu_task_run_config", [_P(Task), _P(Program), ctypes.c_int32]),
    ("phcu_mlp_init", [_vp, ctypes.c_uint64]),
    ("phcu_mlp_forward", [_vp, _vp, ctypes.c_int32, _vp]),
    ("phcu_mlp_grad", [_vp, _vp, _vp, ctypes.c_int32, _vp, _P(ctypes.c_float)]),
    ("phcu_mlp_train", [_vp, _vp, _vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_float,
                        ctypes.c_uint64, _P(ctypes.c_float)]),
]


def exported_names():
    return [n for n, _ in _SIGS]


def load(path=None):
    """Loads libphcuda.so (raises if it is missing: no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or _lib_path()
    if not os.path.exists(path):
        raise RuntimeError(
            "libphcuda.so is not built (%s); run __graft_entry__.build() or ph-core_gb300/build.py" % path)
    lib = ctypes.CDLL(path)
    for name, args in _SIGS:
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.argtypes = args
        fn.restype = ctypes.c_int32
    _lib = lib
    return lib


def last_error():
    buf = ctypes.create_string_buffer(512)
    load().phcu_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def check(rc, what=""):
    """Raises the Phase exception matching a C-ABI status code."""
    if rc == OK:
        return
    msg = last_error() or ("phcu status %d" % rc)
    if what:
        msg = "%s: %s" % (what, msg)
    raise errors.from_status(rc, msg)


def call(name, *args):
    rc = getattr(load(), name)(*args)
    check(rc, name)
    return rc
