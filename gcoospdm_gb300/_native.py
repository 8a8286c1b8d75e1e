"""ctypes binding of the C ABI in include/gcoo.h (libgcoo.so, built in-tree).

The library is loaded on first use. There is no fallback: if the shared
library is missing or fails to load, every call raises ``NativeLibraryError``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(_HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libgcoo.so")
BASELINES_PATH = os.path.join(BUILD_DIR, "libgcoo_baselines.so")
MAIN_PATH = os.path.join(BUILD_DIR, "gcoo_main")

GCOO_SUCCESS = 0
STATUS_NAMES = {
    0: "GCOO_SUCCESS", 1: "GCOO_ERROR_INVALID_VALUE", 2: "GCOO_ERROR_ALLOC", 3: "GCOO_ERROR_CUDA",
    4: "GCOO_ERROR_NOT_BUILT", 5: "GCOO_ERROR_UNSUPPORTED", 6: "GCOO_ERROR_FORMAT",
    7: "GCOO_ERROR_TIMEOUT", 8: "GCOO_ERROR_CAPACITY",
}
PREC = {"fp32": 0, "bf16": 1, "split_bf16": 2, "fp8_b": 3}
ENGINE = {"auto": 0, "cuda_core": 1, "tensor": 2}

# Every symbol include/gcoo.h declares (checked by the CPU test suite).
EXPORTS = (
    "gcoo_abi_version", "gcoo_status_string", "gcoo_last_error", "gcoo_params_default",
    "gcoo_set_allocator", "gcoo_create", "gcoo_create_coo", "gcoo_build", "gcoo_export", "gcoo_spdm", "gcoo_spdm_ex",
    "gcoo_prepare", "gcoo_multiply_by", "gcoo_destroy", "gcoo_spdm_left", "gcoo_query_engine", "gcoo_kernel_launches",
    "gcoo_check_bounded_wait", "gcoo_check_arrays",
    "gcoo_device_status",
    "gcoo_convert_count", "gcoo_convert_count_static", "gcoo_convert_scatter", "gcoo_spdm_view", "gcoo_error_norm",
    "gcoo_batch_create", "gcoo_batch_run", "gcoo_batch_launches", "gcoo_batch_destroy",
    "gcoo_session_create", "gcoo_session_multiply", "gcoo_session_stats", "gcoo_session_destroy",
    "gcoo_autotune", "gcoo_autotune_save", "gcoo_autotune_load", "gcoo_autotune_clear",
    "gcoo_read_matrix_market", "gcoo_free_host",
)


class NativeLibraryError(RuntimeError):
    pass


class GcooError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class Params(C.Structure):
    _fields_ = [("rows_per_group", C.c_int32), ("vec", C.c_int32), ("warps", C.c_int32),
                ("col_warps", C.c_int32), ("engine", C.c_int32), ("depth", C.c_int32),
                ("fp32_order", C.c_int32), ("fp32_sum", C.c_int32)]


class View(C.Structure):
    _fields_ = [("m", C.c_int64), ("k", C.c_int64), ("nnz", C.c_int64), ("n_group", C.c_int64),
                ("rows_per_group", C.c_int32), ("group_index", C.c_void_p), ("nnz_per_group", C.c_void_p),
                ("vals", C.c_void_p), ("rows", C.c_void_p), ("cols", C.c_void_p)]


class Problem(C.Structure):
    _fields_ = [("a", C.c_void_p), ("dB", C.c_void_p), ("n", C.c_int64), ("dC", C.c_void_p)]


ALLOC_FN = C.CFUNCTYPE(C.c_void_p, C.c_size_t, C.c_void_p)
FREE_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p)

_lib = None
_lock = threading.Lock()


def build(verbose: bool = False) -> None:
    """Compile the library in-tree for sm_103a (make; incremental)."""
    cmd = ["make", "-j", str(max(2, min(16, os.cpu_count() or 2))), "-C", os.path.join(_HERE, "csrc")]
    if not verbose:
        cmd.insert(1, "-s")
    subprocess.run(cmd, check=True)


def _declare(L) -> None:
    vp, i64, i32 = C.c_void_p, C.c_int64, C.c_int32
    st = C.c_int
    sig = {
        "gcoo_abi_version": (C.c_int, []),
        "gcoo_status_string": (C.c_char_p, [st]),
        "gcoo_last_error": (C.c_char_p, []),
        "gcoo_params_default": (st, [C.POINTER(Params)]),
        "gcoo_set_allocator": (st, [ALLOC_FN, FREE_FN, vp]),
        "gcoo_create": (st, [C.POINTER(vp), vp, i64, i64, C.POINTER(Params)]),
        "gcoo_create_coo": (st, [C.POINTER(vp), i64, i64, vp, vp, vp, i64, C.POINTER(Params)]),
        "gcoo_build": (st, [vp, vp]),
        "gcoo_export": (st, [vp, C.POINTER(View)]),
        "gcoo_spdm": (st, [vp, vp, i64, vp, vp]),
        "gcoo_spdm_ex": (st, [vp, vp, i64, vp, C.c_int, vp]),
        "gcoo_prepare": (st, [vp, i64, C.c_int, vp]),
        "gcoo_multiply_by": (st, [vp, vp, i64, vp, vp]),
        "gcoo_destroy": (st, [vp]),
        "gcoo_spdm_left": (st, [vp, vp, i64, vp, vp]),
        "gcoo_query_engine": (st, [vp, C.c_int, C.POINTER(i32)]),
        "gcoo_kernel_launches": (C.c_uint64, []),
        "gcoo_check_bounded_wait": (st, [C.c_uint64, vp]),
        "gcoo_check_arrays": (st, [vp, vp, C.POINTER(i64)]),
        "gcoo_device_status": (st, [vp, vp, C.POINTER(C.c_uint32)]),
        "gcoo_convert_count": (st, [vp, i64, i64, i32, vp, vp, C.POINTER(i64), vp]),
        "gcoo_convert_count_static": (st, [vp, i64, i64, i32, vp, vp, C.POINTER(i64), vp]),
        "gcoo_convert_scatter": (st, [vp, i64, i64, i32, vp, vp, vp, vp, vp]),
        "gcoo_spdm_view": (st, [C.POINTER(View), vp, i64, vp, vp]),
        "gcoo_error_norm": (st, [vp, vp, i64, vp, C.POINTER(C.c_double), vp]),
        "gcoo_batch_create": (st, [C.POINTER(vp), C.POINTER(Problem), i32, C.c_int, vp]),
        "gcoo_batch_run": (st, [vp, vp]),
        "gcoo_batch_launches": (st, [vp, C.POINTER(i32)]),
        "gcoo_batch_destroy": (st, [vp]),
        "gcoo_session_create": (st, [C.POINTER(vp), C.POINTER(Params), i64]),
        "gcoo_session_multiply": (st, [vp, vp, i64, i64, vp, i64, vp, vp]),
        "gcoo_session_stats": (st, [vp, C.POINTER(i32), C.POINTER(i32)]),
        "gcoo_session_destroy": (st, [vp]),
        "gcoo_autotune": (st, [vp, vp, i64, vp, vp, C.POINTER(Params)]),
        "gcoo_autotune_save": (st, [C.c_char_p]),
        "gcoo_autotune_load": (st, [C.c_char_p]),
        "gcoo_autotune_clear": (st, []),
        "gcoo_read_matrix_market": (st, [C.c_char_p, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64),
                                         C.POINTER(C.POINTER(i32)), C.POINTER(C.POINTER(i32)),
                                         C.POINTER(C.POINTER(C.c_float))]),
        "gcoo_free_host": (None, [vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def lib():
    """The loaded libgcoo.so; raises NativeLibraryError when it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise NativeLibraryError(
                    f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
                    " (there is no CPU fallback)")
            try:
                L = C.CDLL(LIB_PATH, mode=C.RTLD_GLOBAL)
            except OSError as e:  # pragma: no cover - depends on the machine
                raise NativeLibraryError(f"cannot load {LIB_PATH}: {e}") from e
            _declare(L)
            _lib = L
    return _lib


def check(status: int) -> None:
    if status != GCOO_SUCCESS:
        msg = lib().gcoo_last_error()
        raise GcooError(status, msg.decode() if msg else "")
