"""GPU bit sketches (ssg_bitsketch): bit-exact against the oracle's sequential
dot products, and the sketch -> Hamming search pipeline of the C3 data."""
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


@pytest.mark.parametrize("indim,outdim,n", [(5, 1, 1), (96, 64, 300), (100, 130, 257), (768, 1024, 1000)])
def test_bitsketch_bit_exact(ss, indim, outdim, n):
    rng = np.random.default_rng(indim + outdim + n)
    R = rng.standard_normal((indim, outdim)).astype(np.float32)      # the reference's (indim, outdim) map
    X = rng.standard_normal((indim, n)).astype(np.float32)           # one object per column
    X[:, 0] = 0.0                                                    # all dots 0: every bit 1
    B = ss.bitsketch(R, X)
    assert B.shape == ((outdim + 63) // 64, n) and B.dtype == np.uint64
    ref = O.bitsketch(np.ascontiguousarray(R.T), np.ascontiguousarray(X.T))
    assert np.array_equal(np.ascontiguousarray(B.T), ref)
    assert B[0, 0] == np.uint64((1 << min(outdim, 64)) - 1) if outdim < 64 else B[0, 0] == np.uint64(2**64 - 1)
    j = min(3, n - 1)
    v = ss.bitsketch(R, X[:, j])
    assert np.array_equal(v, B[:, j])


def test_sketches_feed_the_hamming_scan(ss):
    rng = np.random.default_rng(7)
    R = rng.standard_normal((64, 256)).astype(np.float32)
    X = rng.standard_normal((64, 3000)).astype(np.float32)
    Q = X[:, :40] + 0.1 * rng.standard_normal((64, 40)).astype(np.float32)
    S, SQ = ss.bitsketch(R, X), ss.bitsketch(R, Q)
    idx = ss.GPUExhaustiveSearch(ss.Dist.Bits.Hamming(), ss.MatrixDatabase(S))
    ids, dists = ss.searchbatch(idx, ss.GenericContext(logger=None), ss.MatrixDatabase(SQ), 5)
    ri, rd = O.searchbatch("hamming", np.ascontiguousarray(S.T), np.ascontiguousarray(SQ.T), 5)
    assert np.array_equal(np.ascontiguousarray(ids.T), ri) and np.array_equal(np.ascontiguousarray(dists.T), rd)
    assert np.mean(ids[0] == np.arange(1, 41)) > 0.9                  # the perturbed object is nearest
