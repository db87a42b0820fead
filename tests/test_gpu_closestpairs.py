"""GPU closest pairs (ssg_closestpairs): closestpair / closestpairs /
bichromatic_kclosestpairs against the oracle's restatement."""
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


def close(a, b):
    assert len(a) == len(b)
    for (i, j, d), (ri, rj, rd) in zip(a, b):
        assert (i, j) == (ri, rj)
        assert d == np.float32(rd)


@pytest.mark.parametrize("name,dist", [("sql2", "SqL2"), ("l2", "L2"), ("ip", "InnerProduct")])
@pytest.mark.parametrize("k", [1, 7, 40])
def test_closestpairs_self(ss, name, dist, k):
    rng = np.random.default_rng(k + len(name))
    X = rng.standard_normal((3000, 24)).astype(np.float32)
    idx = ss.GPUExhaustiveSearch(getattr(ss.Dist, dist)(), ss.MatrixDatabase.from_rows(X))
    ctx = ss.GenericContext(logger=None)
    got = ss.closestpairs(idx, ctx, k=k)
    ref = O.closestpairs(name, X, X, k, max(k, 8), True)
    close(got, ref)
    if k == 1:
        assert ss.closestpair(idx, ctx) == got[0]


def test_bichromatic_pairs(ss):
    rng = np.random.default_rng(4)
    A = rng.standard_normal((5000, 16)).astype(np.float32)
    B = rng.standard_normal((700, 16)).astype(np.float32)
    idx = ss.GPUExhaustiveSearch(ss.Dist.SqL2(), ss.MatrixDatabase.from_rows(A))
    ctx = ss.GenericContext(logger=None)
    got = ss.bichromatic_kclosestpairs(idx, ctx, ss.MatrixDatabase.from_rows(B), k=25, min_k=25)
    close(got, O.closestpairs("sql2", A, B, 25, 25, False))
    # the same data passed as B excludes self-matches only with samedata
    same = ss.bichromatic_kclosestpairs(idx, ctx, ss.MatrixDatabase.from_rows(A[:300]), k=5, samedata=True)
    close(same, O.closestpairs("sql2", A, A[:300], 5, 8, True))
    zero = ss.bichromatic_kclosestpairs(idx, ctx, ss.MatrixDatabase.from_rows(A[:300]), k=5, samedata=False)
    assert all(d == 0.0 for _, _, d in zero)


def test_closestpairs_large_and_edge_cases(ss):
    rng = np.random.default_rng(9)
    X = rng.standard_normal((60000, 8)).astype(np.float32)      # many merge passes (60k sorted segments)
    idx = ss.GPUExhaustiveSearch(ss.Dist.SqL2(), ss.MatrixDatabase.from_rows(X))
    ctx = ss.GenericContext(logger=None)
    got = ss.closestpairs(idx, ctx, k=10)
    close(got, O.closestpairs("sql2", X, X, 10, 10, True))
    one = ss.GPUExhaustiveSearch(ss.Dist.SqL2(), ss.MatrixDatabase.from_rows(X[:1]))
    assert ss.closestpairs(one, ctx, k=3) == []                    # no pair among one object
    assert ss.closestpair(one, ctx) == (0, 0, float("inf"))
    two = ss.GPUExhaustiveSearch(ss.Dist.SqL2(), ss.MatrixDatabase.from_rows(X[:2]))
    p = ss.closestpairs(two, ctx, k=5)
    assert [(i, j) for i, j, _ in p] == [(2, 1), (1, 2)]
    with pytest.raises(ss.ArgumentError):
        ss.closestpairs(idx, ctx, k=9, min_k=3)
