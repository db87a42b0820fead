"""MMapMatrixDatabase files (src/db/mmapmatrixdatabase.jl:10-27,151-175):
the writer and reader mirror, and the header checks of ssg_create_mmap, which
run before any device work (so they need no GPU)."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_package


def test_write_and_reopen_round_trip(tmp_path):
    ss = load_package()
    X = np.arange(3 * 5, dtype=np.float32).reshape(3, 5)           # (dim, n)
    p = tmp_path / "db.bin"
    ss.write_mmap_matrix(p, X, capacity=8)
    raw = p.read_bytes()
    assert len(raw) == 4096 + 3 * 8 * 4
    assert int(np.frombuffer(raw[0:8], "<u8")[0]) == 0x4D4D444231000001
    assert (int(np.frombuffer(raw[8:12], "<i4")[0]), int(np.frombuffer(raw[12:20], "<i8")[0]),
            int(np.frombuffer(raw[20:24], "<i4")[0]), int(np.frombuffer(raw[24:32], "<i8")[0])) == (1, 3, 2, 5)
    db = ss.MMapMatrixDatabase(p)
    assert len(db) == 5 and db.dim == 3 and np.array_equal(db[2], X[:, 1])
    assert np.array_equal(db.rows(), X.T)


@pytest.mark.parametrize("case,code", [("magic", -1), ("version", -1), ("type", -5), ("short", -1), ("missing", -1)])
def test_create_mmap_rejects_bad_files(tmp_path, case, code):
    ss = load_package()
    N = ss._native
    p = tmp_path / "db.bin"
    ss.write_mmap_matrix(p, np.ones((4, 10), dtype=np.float32))
    raw = bytearray(p.read_bytes())
    if case == "magic":
        raw[0] ^= 0xFF
    elif case == "version":
        raw[8:12] = np.int32(2).tobytes()
    elif case == "type":
        raw[20:24] = np.int32(6).tobytes()        # Int16: no GPU metric takes it
    elif case == "short":
        raw[24:32] = np.int64(11).tobytes()        # more objects than the data holds
    if case == "missing":
        path = str(tmp_path / "nope.bin").encode()
    else:
        p.write_bytes(bytes(raw))
        path = str(p).encode()
    h = C.c_void_p()
    assert N.lib().ssg_create_mmap(N.METRIC_SQL2, path, 0, C.byref(h)) == code
    assert not h.value
    assert N.last_error(None)
