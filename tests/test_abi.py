"""The C ABI without a GPU: the library builds, loads, exports every symbol the
header declares, and rejects bad arguments before touching the device."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, load_package

HEADER = os.path.join(ROOT, "include", "ssgpu.h")


def header_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(ssg_[a-z_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def native():
    ss = load_package()
    ss.build()
    return ss._native


def test_header_declares_expected_entry_points():
    syms = header_symbols()
    for name in ("ssg_create", "ssg_search", "ssg_allknn", "ssg_append", "ssg_set_param",
                 "ssg_last_error", "ssg_destroy"):
        assert name in syms


def test_library_exports_every_header_symbol(native):
    L = native.lib()
    for name in header_symbols():
        assert hasattr(L, name), name
        assert name in native.SIGNATURES, f"{name} has no ctypes signature"


def test_version(native):
    assert native.lib().ssg_version() >= 100


@pytest.mark.parametrize("metric,elem,dim,ld,prec,code", [
    (9, 0, 4, 4, 0, -5),     # unknown metric
    (0, 1, 4, 4, 0, -5),     # float metric on UInt64
    (5, 0, 4, 4, 0, -5),     # Hamming on Float32
    (0, 0, 0, 0, 0, -1),     # zero dimension
    (0, 0, 4, 3, 0, -1),     # ld < dim
    (5, 1, 33, 33, 0, -5),   # too many sketch words
    (0, 0, 4, 4, 7, -5),     # unknown precision
])
def test_create_rejects_bad_arguments_on_host(native, metric, elem, dim, ld, prec, code):
    L = native.lib()
    h = C.c_void_p()
    buf = np.zeros(64, dtype=np.float64)
    rc = L.ssg_create(metric, elem, dim, 2, buf.ctypes.data_as(C.c_void_p), ld, prec, C.byref(h))
    assert rc == code
    assert h.value is None
    msg = native.last_error(None)
    assert len(msg) > 0


def test_calls_on_null_index_fail_cleanly(native):
    L = native.lib()
    ids = np.zeros(4, dtype=np.uint32)
    d = np.zeros(4, dtype=np.float32)
    q = np.zeros(4, dtype=np.float32)
    assert L.ssg_search(None, q.ctypes.data_as(C.c_void_p), 4, 1, 4, ids.ctypes.data_as(C.c_void_p),
                        d.ctypes.data_as(C.c_void_p), 0) == -1
    assert L.ssg_allknn(None, 1, 0, ids.ctypes.data_as(C.c_void_p), d.ctypes.data_as(C.c_void_p)) == -1
    assert L.ssg_set_param(None, b"splits", 1.0) == -1
    L.ssg_destroy(None)


def test_python_errors_map_status_codes(native):
    with pytest.raises(native.ArgumentError):
        native.check(-1)
    with pytest.raises(native.UnsupportedError):
        native.check(-5)
    with pytest.raises(native.SSGError):
        native.check(-3)
