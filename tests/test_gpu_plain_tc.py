"""The plain FP32 method on the tensor cores (two-piece BF16 scan, exact FP32
rerank of k + margin candidates, completeness check, exact-scan fallback)
against the oracle's sequential (lanes=1) ExhaustiveSearch restatement
(src/exact/sequential-exhaustive.jl:60-78, src/allknn.jl:66-110): ids and
distances bit-identical, for every metric it serves, across dimensions,
k, allknn, and inputs made to defeat the check (exact ties, duplicates),
where the fallback must take over.  The same searches with "plain_tc" off
(CUDA-core GEMM form) give the same arrays."""
import numpy as np
import pytest

from conftest import load_package
from oracle import oracle as O

pytestmark = pytest.mark.gpu

METRICS = {"sql2": "SqL2", "l2": "L2", "normcosine": "NormCosine", "ip": "InnerProduct", "cosine": "Cosine"}


@pytest.fixture(scope="module")
def ss():
    mod = load_package()
    mod.build()
    return mod


def make(name, n, m, d, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, d), dtype=np.float32)
    Q = rng.standard_normal((m, d), dtype=np.float32)
    if name == "normcosine":
        X /= np.linalg.norm(X, axis=1, keepdims=True)
        Q /= np.linalg.norm(Q, axis=1, keepdims=True)
    return X, Q


def run(ss, name, X, Q, k, plain_tc=1):
    idx = ss.GPUExhaustiveSearch(getattr(ss.Dist, METRICS[name])(), ss.MatrixDatabase.from_rows(X))
    idx.set_param("plain_tc", plain_tc)
    ids, dists = ss.searchbatch(idx, ss.GenericContext(logger=None), ss.MatrixDatabase.from_rows(Q), k)
    return ids.T, dists.T, idx


@pytest.mark.parametrize("name", list(METRICS))
@pytest.mark.parametrize("d,k,on_tc", [(8, 1, 1), (33, 10, 1), (96, 32, 1), (128, 10, 1), (24, 48, 1), (100, 64, 0)])
def test_plain_tc_searchbatch_bitexact(ss, name, d, k, on_tc):
    # (100, 64): 80 candidates per query do not fit the scans' on-chip heaps
    # next to K = 384 tiles, so the plain method stays on the CUDA cores
    X, Q = make(name, 20000, 300, d, seed=d * 7 + k)
    gi, gd, idx = run(ss, name, X, Q, k)
    assert idx.get_param("last_plain_tc") == on_tc
    ri, rd = O.searchbatch(name, X, Q, k, lanes=1, nthreads=O.num_threads())
    assert np.array_equal(gi, ri)
    assert np.array_equal(gd, rd)
    # the margin is rarely too small on Gaussian data
    assert idx.get_param("fallbacks") <= 0.05 * Q.shape[0]
    ci, cd, cidx = run(ss, name, X, Q, k, plain_tc=0)
    assert cidx.get_param("last_plain_tc") == 0.0
    assert np.array_equal(gi, ci) and np.array_equal(gd, cd)


@pytest.mark.parametrize("name", list(METRICS))
@pytest.mark.parametrize("d,k", [(200, 10), (768, 1), (768, 20), (300, 33)])
def test_plain_tc_streaming_wide_vectors_bitexact(ss, name, d, k):
    """dim > 128: the split tiles stream along K = 3 kp through the K-streaming
    scan; same certificate, same exact results."""
    X, Q = make(name, 12000, 200, d, seed=d + k)
    gi, gd, idx = run(ss, name, X, Q, k)
    assert idx.get_param("last_plain_tc") == 1.0
    ri, rd = O.searchbatch(name, X, Q, k, lanes=1, nthreads=O.num_threads())
    assert np.array_equal(gi, ri)
    assert np.array_equal(gd, rd)
    ci, cd, cidx = run(ss, name, X, Q, k, plain_tc=0)
    assert np.array_equal(gi, ci) and np.array_equal(gd, cd)


@pytest.mark.parametrize("name", ["sql2", "normcosine"])
def test_plain_tc_allknn_bitexact(ss, name):
    rng = np.random.default_rng(61)
    C = rng.standard_normal((40, 96), dtype=np.float32)
    X = C[rng.integers(0, 40, 12000)] + 0.3 * rng.standard_normal((12000, 96), dtype=np.float32)
    if name == "normcosine":
        X /= np.linalg.norm(X, axis=1, keepdims=True)
    idx = ss.GPUExhaustiveSearch(getattr(ss.Dist, METRICS[name])(), ss.MatrixDatabase.from_rows(X))
    ids, dists = ss.allknn(idx, ss.GenericContext(logger=None), 32, exclude_self=True)
    assert idx.get_param("last_plain_tc") == 1.0
    rows = np.sort(rng.choice(12000, size=300, replace=False))
    ri, rd = O.allknn_rows(name, X, 33, rows, lanes=1, nthreads=O.num_threads())
    for r, j in enumerate(rows):
        keep = [t for t in range(33) if ri[r, t] != j + 1][:32]
        assert np.array_equal(ids.T[j], ri[r, keep])
        assert np.array_equal(dists.T[j], rd[r, keep])


@pytest.mark.parametrize("name", list(METRICS))
def test_plain_tc_ties_defeat_the_check_and_fall_back(ss, name):
    """Each database row repeated 40 times: every candidate list is a run of
    equal distances, no margin certifies it, and the fallback's exact scan
    answers; ids still follow the (distance, id) order."""
    rng = np.random.default_rng(62)
    base = rng.standard_normal((200, 48), dtype=np.float32)
    if name == "normcosine":
        base /= np.linalg.norm(base, axis=1, keepdims=True)
    X = np.repeat(base, 40, axis=0)
    Q = base[:50] + np.float32(1e-3) * rng.standard_normal((50, 48), dtype=np.float32)
    if name == "normcosine":
        Q /= np.linalg.norm(Q, axis=1, keepdims=True)
    gi, gd, idx = run(ss, name, X, Q, 10)
    assert idx.get_param("last_plain_tc") == 1.0
    assert idx.get_param("fallbacks") == 50
    ri, rd = O.searchbatch(name, X, Q, 10, lanes=1, nthreads=O.num_threads())
    assert np.array_equal(gi, ri) and np.array_equal(gd, rd)


def test_plain_tc_wide_magnitudes_and_appends(ss):
    """Log-normal row norms over several binades, then appended rows: the
    split tiles are rebuilt for the grown database."""
    rng = np.random.default_rng(63)
    X = rng.standard_normal((9000, 64), dtype=np.float32) * rng.lognormal(0, 2.0, (9000, 1)).astype(np.float32)
    Q = rng.standard_normal((200, 64), dtype=np.float32) * rng.lognormal(0, 2.0, (200, 1)).astype(np.float32)
    idx = ss.GPUExhaustiveSearch(ss.Dist.SqL2(), ss.MatrixDatabase.from_rows(X))
    ctx = ss.GenericContext(logger=None)
    ids, dists = ss.searchbatch(idx, ctx, ss.MatrixDatabase.from_rows(Q), 10)
    ri, rd = O.searchbatch("sql2", X, Q, 10, lanes=1, nthreads=O.num_threads())
    assert np.array_equal(ids.T, ri) and np.array_equal(dists.T, rd)
    extra = Q[:30] + np.float32(1e-2)
    for row in extra:
        ss.push_item_b(idx, ctx, row)
    X2 = np.concatenate([X, extra])
    ids, dists = ss.searchbatch(idx, ctx, ss.MatrixDatabase.from_rows(Q), 10)
    assert idx.get_param("last_plain_tc") == 1.0
    ri, rd = O.searchbatch("sql2", X2, Q, 10, lanes=1, nthreads=O.num_threads())
    assert np.array_equal(ids.T, ri) and np.array_equal(dists.T, rd)


@pytest.mark.parametrize("name", ["sql2", "ip"])
def test_plain_tc_allknn_locality_order(ss, name):
    """allknn over 40,000 rows scans the database in its locality order
    (rows grouped by nearest pivot); the arrays equal the id-order scan's and
    the oracle's rows."""
    rng = np.random.default_rng(64)
    C = rng.standard_normal((300, 64), dtype=np.float32)
    X = C[rng.integers(0, 300, 40000)] + 0.4 * rng.standard_normal((40000, 64), dtype=np.float32)
    idx = ss.GPUExhaustiveSearch(getattr(ss.Dist, METRICS[name])(), ss.MatrixDatabase.from_rows(X))
    ctx = ss.GenericContext(logger=None)
    ids, dists = ss.allknn(idx, ctx, 16, exclude_self=True)
    assert idx.get_param("last_plain_tc") == 1.0
    idx.set_param("locality", 0)
    ids0, dists0 = ss.allknn(idx, ctx, 16, exclude_self=True)
    assert np.array_equal(ids, ids0) and np.array_equal(dists, dists0)
    # groups in pivot order, one pivot per 1024 rows: the same arrays
    idx.set_param("locality", 1)
    idx.set_param("locality_chain", 0)
    idx.set_param("locality_rows", 1024)
    ids1, dists1 = ss.allknn(idx, ctx, 16, exclude_self=True)
    assert np.array_equal(ids, ids1) and np.array_equal(dists, dists1)
    rows = np.sort(rng.choice(40000, size=200, replace=False))
    ri, rd = O.allknn_rows(name, X, 17, rows, lanes=1, nthreads=O.num_threads())
    for r, j in enumerate(rows):
        keep = [t for t in range(17) if ri[r, t] != j + 1][:16]
        assert np.array_equal(ids.T[j], ri[r, keep])
        assert np.array_equal(dists.T[j], rd[r, keep])


@pytest.mark.parametrize("name", ["sql2", "normcosine"])
def test_plain_tc_on_cta_pairs_bitexact(ss, name):
    """The split scan on CTA pairs (M = 256 MMAs, the odd CTA's half of each
    K-block counted on the even CTA's barrier) answers the same."""
    X, Q = make(name, 20000, 333, 96, seed=71)
    gi, gd, idx = run(ss, name, X, Q, 32)
    idx2 = ss.GPUExhaustiveSearch(getattr(ss.Dist, METRICS[name])(), ss.MatrixDatabase.from_rows(X))
    idx2.set_param("pair", 1)
    pi, pd = ss.searchbatch(idx2, ss.GenericContext(logger=None), ss.MatrixDatabase.from_rows(Q), 32)
    assert idx2.get_param("last_plain_tc") == 1.0
    assert np.array_equal(pi.T, gi) and np.array_equal(pd.T, gd)
    ri, rd = O.searchbatch(name, X, Q, 32, lanes=1, nthreads=O.num_threads())
    assert np.array_equal(gi, ri) and np.array_equal(gd, rd)


@pytest.mark.parametrize("m", [1, 129])
@pytest.mark.parametrize("d", [17, 160])
def test_plain_tc_edge_shapes(ss, m, d):
    """The smallest database the tensor-core form takes (4,096 rows), a single
    query and a query count one past a tile, dims off the padding grid."""
    X, Q = make("sql2", 4096, m, d, seed=m * 1000 + d)
    gi, gd, idx = run(ss, "sql2", X, Q, 7)
    assert idx.get_param("last_plain_tc") == 1.0
    ri, rd = O.searchbatch("sql2", X, Q, 7, lanes=1, nthreads=O.num_threads())
    assert np.array_equal(gi, ri) and np.array_equal(gd, rd)


def test_plain_tc_allknn_with_duplicate_rows(ss):
    """allknn excluding self over rows that come in identical pairs: the
    twin sits at distance 0 and self is dropped by id, in (distance, id)
    order, as the reference's KnnSorted gives."""
    rng = np.random.default_rng(65)
    base = rng.standard_normal((2100, 40), dtype=np.float32)
    X = np.repeat(base, 2, axis=0)
    idx = ss.GPUExhaustiveSearch(ss.Dist.SqL2(), ss.MatrixDatabase.from_rows(X))
    ids, dists = ss.allknn(idx, ss.GenericContext(logger=None), 5, exclude_self=True)
    assert idx.get_param("last_plain_tc") == 1.0
    ri, rd = O.allknn("sql2", X, 6, lanes=1, nthreads=O.num_threads())
    for j in range(0, X.shape[0], 97):
        keep = [t for t in range(6) if ri[j, t] != j + 1][:5]
        assert np.array_equal(ids.T[j], ri[j, keep])
        assert np.array_equal(dists.T[j], rd[j, keep])
    # every row's nearest neighbour is its twin at distance 0
    twin = np.arange(X.shape[0]) ^ 1
    assert np.array_equal(ids[0], (twin + 1).astype(np.uint32))
    assert np.all(dists[0] == 0)


@pytest.mark.parametrize("name", ["sql2", "normcosine"])
def test_plain_tc_half_heaps_under_shared_bounds(ss, name):
    """Rows stored cluster by cluster and a handful of queries: many database
    splits per query, half-heaps that the shared bound keeps from filling;
    the certificate must still hold (or fall back) -- results exact."""
    rng = np.random.default_rng(66)
    C = rng.standard_normal((40, 96), dtype=np.float32)
    lab = np.sort(rng.integers(0, 40, 20000))
    X = C[lab] + 0.2 * rng.standard_normal((20000, 96), dtype=np.float32)
    if name == "normcosine":
        X /= np.linalg.norm(X, axis=1, keepdims=True)
    Q = X[rng.choice(20000, 37, replace=False)] + np.float32(1e-3)
    if name == "normcosine":
        Q /= np.linalg.norm(Q, axis=1, keepdims=True)
    gi, gd, idx = run(ss, name, X, Q, 32)
    assert idx.get_param("last_plain_tc") == 1.0
    ri, rd = O.searchbatch(name, X, Q, 32, lanes=1, nthreads=O.num_threads())
    assert np.array_equal(gi, ri) and np.array_equal(gd, rd)
