"""ctypes binding of libssgpu.so (the C ABI in include/ssgpu.h).

The library is built in-tree by ``builder.py``; importing this module never
builds it.  If the shared object is missing the first call raises
``NativeLibraryMissing`` -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libssgpu.so")

SSG_OK = 0
SSG_EINVAL = -1
SSG_ENOMEM = -2
SSG_ECUDA = -3
SSG_ETIMEOUT = -4
SSG_EUNSUPPORTED = -5

METRIC_SQL2, METRIC_L2, METRIC_NORMCOSINE, METRIC_COSINE, METRIC_IP, METRIC_HAMMING = range(6)
ELEM_F32, ELEM_U64, ELEM_F64, ELEM_F16, ELEM_U8, ELEM_I8 = range(6)
PREC_FP32, PREC_BF16, PREC_FP8 = 0, 1, 2
FLAG_ASYNC = 1

# Every symbol include/ssgpu.h declares, with its ctypes signature.
_p, _i64, _i32, _int, _dbl = C.c_void_p, C.c_int64, C.c_int32, C.c_int, C.c_double
SIGNATURES = {
    "ssg_version": ([], _int),
    "ssg_create": ([_int, _int, _i64, _i64, _p, _i64, _int, C.POINTER(_p)], _int),
    "ssg_create_device": ([_int, _int, _i64, _i64, _p, _i64, _int, C.POINTER(_p)], _int),
    "ssg_create_mmap": ([_int, C.c_char_p, _int, C.POINTER(_p)], _int),
    "ssg_search": ([_p, _p, _i64, _i64, _i32, _p, _p, _i32], _int),
    "ssg_search_device": ([_p, _p, _i64, _i32, _p, _p, _i32], _int),
    "ssg_allknn": ([_p, _i32, _i32, _p, _p], _int),
    "ssg_allknn_device": ([_p, _i32, _i32, _p, _p], _int),
    "ssg_append": ([_p, _p, _i64], _int),
    "ssg_rerank": ([_p, _p, _i64, _i32, _p, _p], _int),
    "ssg_set_param": ([_p, C.c_char_p, _dbl], _int),
    "ssg_get_param": ([_p, C.c_char_p, C.POINTER(_dbl)], _int),
    "ssg_set_stream": ([_p, _p], _int),
    "ssg_last_error": ([_p, C.c_char_p, _i64], _int),
    "ssg_destroy": ([_p], None),
    "ssg_knn_noalloc": ([_int, _p, _i64, _i64, _p, _i64, _i32, _p, _p, _p], _int),
    "ssg_closestpairs": ([_p, _p, _i64, _i32, _i32, _i32, _p, _p, _p, C.POINTER(_i64)], _int),
    "ssg_bitsketch": ([_p, _i64, _i64, _p, _i64, _p, _p], _int),
    "ssg_search_batches": ([_p, _i32, _p, _p, _p, _p, _p], _int),
    "ssg_train_mlp": ([_p, _i64, _i64, _i32, _i32, _i32, _i32, _dbl, C.c_uint64], _int),
    "ssg_save_model": ([_p, C.c_char_p], _int),
    "ssg_load_model": ([_p, C.c_char_p], _int),
    "ssg_mlp_grad_check": ([_i64, _i64, _i64, _p, _p, _p, _p, _p, _i32, C.c_float, _p, _p, _p, _p, _p], _int),
}


class NativeLibraryMissing(RuntimeError):
    pass


class ArgumentError(ValueError):
    """Raised where the reference throws ArgumentError (bad shapes, empty inputs)."""


class SSGError(RuntimeError):
    """A device-side failure reported by libssgpu (carries ssg_last_error text)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"libssgpu status {code}: {msg}")
        self.code = code


class UnsupportedError(SSGError):
    pass


_lib = None
_lock = threading.Lock()


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise NativeLibraryMissing(
                    f"{LIB_PATH} is not built; run similaritysearch.jl_gb300/builder.py (or "
                    "__graft_entry__.build()) first")
            L = C.CDLL(LIB_PATH)
            for name, (args, res) in SIGNATURES.items():
                f = getattr(L, name)
                f.argtypes = args
                f.restype = res
            _lib = L
    return _lib


def last_error(handle) -> str:
    buf = C.create_string_buffer(1024)
    lib().ssg_last_error(handle, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, handle=None):
    if rc == SSG_OK:
        return
    msg = last_error(handle)
    if rc == SSG_EINVAL:
        raise ArgumentError(msg)
    if rc == SSG_EUNSUPPORTED:
        raise UnsupportedError(rc, msg)
    raise SSGError(rc, msg)
