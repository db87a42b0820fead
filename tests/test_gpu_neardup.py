"""neardup on the GPU index against the oracle's restatement of
src/neardup.jl: the same epsilon-net, covering objects and distances."""
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


def data(rng, n, d):
    base = rng.standard_normal((n // 4, d)).astype(np.float32)
    X = np.repeat(base, 4, axis=0)[:n] + rng.standard_normal((n, d)).astype(np.float32) * 0.01
    return X[rng.permutation(n)].astype(np.float32)


@pytest.mark.parametrize("name,dist,eps", [("sql2", "SqL2", 0.05), ("l2", "L2", 0.2)])
@pytest.mark.parametrize("blocksize,filterblocks", [(64, True), (1000, True), (50, False)])
def test_neardup_matches_oracle(ss, name, dist, eps, blocksize, filterblocks):
    rng = np.random.default_rng(blocksize + len(name))
    X = data(rng, 600, 8)
    empty = ss.GPUExhaustiveSearch(getattr(ss.Dist, dist)(), ss.MatrixDatabase(np.zeros((8, 0), np.float32)))
    ctx = ss.GenericContext(logger=None)
    R = ss.neardup(empty, ctx, ss.MatrixDatabase.from_rows(X), eps, blocksize=blocksize, filterblocks=filterblocks)
    L, D, M = O.neardup(name, X, eps, blocksize=blocksize, filterblocks=filterblocks)
    assert np.array_equal(R["nn"], L) and np.array_equal(R["dist"], D) and np.array_equal(R["map"], M)
    assert len(R["idx"]) == len(M) and np.array_equal(R["centers"], np.unique(L))
    if filterblocks:
        assert len(M) < 600                                   # the duplicates were found
        assert np.all(R["dist"] <= np.float32(eps))
