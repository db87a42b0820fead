"""An index built straight from a MMapMatrixDatabase file (ssg_create_mmap)
answers exactly like one built from the same matrix in memory."""
import numpy as np
import pytest

from conftest import load_package
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ss():
    mod = load_package()
    mod.build()
    return mod


@pytest.mark.parametrize("dtype,dist,name", [(np.float32, "SqL2", "sql2"), (np.float64, "CastF32.SqL2", "sql2"),
                                             (np.uint8, "CastF32.NormCosine", None), (np.uint64, "Bits.Hamming", "hamming")])
def test_index_from_file_equals_in_memory(ss, tmp_path, dtype, dist, name):
    rng = np.random.default_rng(3)
    if dtype == np.uint64:
        X = rng.integers(0, 2**63, size=(4, 2000), dtype=np.uint64)
    elif dtype == np.uint8:
        X = rng.integers(0, 255, size=(24, 2000), dtype=np.uint8)
    else:
        X = rng.standard_normal((24, 2000)).astype(dtype)
    p = tmp_path / "db.bin"
    ss.write_mmap_matrix(p, X, capacity=2100)
    D = ss.Dist
    for part in dist.split("."):
        D = getattr(D, part)
    fdb = ss.MMapMatrixDatabase(p)
    a = ss.GPUExhaustiveSearch(D(), fdb)
    b = ss.GPUExhaustiveSearch(D(), ss.MatrixDatabase(np.asfortranarray(X)))
    assert len(a) == 2000
    Q = ss.MatrixDatabase(np.asfortranarray(X[:, :37]))
    ctx = ss.GenericContext(logger=None)
    ia, da = ss.searchbatch(a, ctx, Q, 7)
    ib, db_ = ss.searchbatch(b, ctx, Q, 7)
    assert np.array_equal(ia, ib) and np.array_equal(da, db_)
    if name:
        ri, rd = O.searchbatch(name, np.ascontiguousarray(X.T).astype(np.float32) if name == "sql2" else
                               np.ascontiguousarray(X.T), np.ascontiguousarray(X[:, :37].T).astype(
                                   np.float32 if name == "sql2" else np.uint64), 7)
        assert np.array_equal(np.ascontiguousarray(ia.T), ri)
