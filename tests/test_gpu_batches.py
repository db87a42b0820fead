"""GPU tests of ssg_search_batches: uneven batches with mixed k answered by
one packed search per distinct k, and the CUDA-graph replay of its device
work."""
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


def data(rng, n, d, m_total):
    C = rng.standard_normal((64, d), dtype=np.float32)
    X = C[rng.integers(0, 64, size=n)] + 0.3 * rng.standard_normal((n, d), dtype=np.float32)
    Q = X[rng.integers(0, n, size=m_total)] + 0.05 * rng.standard_normal((m_total, d), dtype=np.float32)
    return X.astype(np.float32), Q.astype(np.float32)


def split(Q, sizes):
    offs = np.concatenate([[0], np.cumsum(sizes)])
    return [Q[offs[i]:offs[i + 1]] for i in range(len(sizes))]


def dbs(ss, parts):
    return [ss.MatrixDatabase.from_rows(p) for p in parts]


SIZES = [1, 0, 37, 128, 5, 300]
KS = [10, 3, 1, 100, 17, 10]


@pytest.mark.parametrize("name", ["sql2", "ip", "hamming"])
def test_batches_plain_equal_separate_calls(ss, name):
    rng = np.random.default_rng(len(name))
    if name == "hamming":
        X = rng.integers(0, 2**63, size=(4000, 4), dtype=np.uint64)
        Q = X[rng.integers(0, 4000, size=sum(SIZES))] ^ rng.integers(0, 2**8, size=(sum(SIZES), 4), dtype=np.uint64)
        dist = ss.Dist.Bits.Hamming()
    else:
        X, Q = data(rng, 5000, 48, sum(SIZES))
        dist = ss.Dist.SqL2() if name == "sql2" else ss.Dist.InnerProduct()
    idx = ss.GPUExhaustiveSearch(dist, ss.MatrixDatabase.from_rows(X))
    ctx = ss.GenericContext(logger=None)
    res = ss.searchbatches(idx, ctx, dbs(ss, split(Q, SIZES)), KS)
    for (ids, dists), q, k in zip(res, split(Q, SIZES), KS):
        assert ids.shape == (k, q.shape[0])
        if q.shape[0] == 0:
            continue
        ri, rd = ss.searchbatch(idx, ctx, ss.MatrixDatabase.from_rows(q), k)
        assert np.array_equal(ids, ri) and np.array_equal(dists, rd)


# (the BF16 case keeps k small enough for the on-chip heaps: longer lists take
# the threshold filter, which reads flags on the host and is not captured)
@pytest.mark.parametrize("precision,d,name,ks,overfetch", [("fp8", 384, "ip", KS, 4.0),
                                                           ("bf16", 96, "sql2", [10, 3, 1, 20, 17, 10], 2.0)])
def test_batches_graph_replay(ss, precision, d, name, ks, overfetch):
    rng = np.random.default_rng(d)
    X, Q = data(rng, 20000, d, sum(SIZES))
    dist = ss.Dist.SqL2() if name == "sql2" else ss.Dist.InnerProduct()
    idx = ss.GPUExhaustiveSearch(dist, ss.MatrixDatabase.from_rows(X), precision=precision, overfetch=overfetch)
    ctx = ss.GenericContext(logger=None)
    KS = ks
    runs = [ss.searchbatches(idx, ctx, dbs(ss, split(Q, SIZES)), KS) for _ in range(5)]
    assert idx.get_param("graph_replays") >= 2 and idx.get_param("last_graph") == 1
    # replays give the results of the eager runs, bit for bit
    for r in runs[1:]:
        for (a, b), (c, e) in zip(runs[0], r):
            assert np.array_equal(a, c) and np.array_equal(b, e)
    idx.set_param("graphs", 0)
    eager = ss.searchbatches(idx, ctx, dbs(ss, split(Q, SIZES)), KS)
    assert idx.get_param("last_graph") == 0
    for (a, b), (c, e) in zip(runs[0], eager):
        assert np.array_equal(a, c) and np.array_equal(b, e)
    # exact distances, (distance, id) order, recall against the FP64 oracle
    for (ids, dists), q, k in zip(runs[0], split(Q, SIZES), KS):
        if q.shape[0] == 0:
            continue
        gi, gd = np.ascontiguousarray(ids.T), np.ascontiguousarray(dists.T)
        for j in range(min(3, q.shape[0])):
            pairs = [(float(gd[j, t]), int(gi[j, t])) for t in range(k)]
            assert pairs == sorted(pairs)
            assert all(np.float32(O.evaluate(name, X[i - 1], q[j])) == np.float32(dd) for dd, i in pairs)
        fi, _ = O.searchbatch_f64(name, X, q, k)
        assert O.macrorecall(fi, gi) >= 0.99


@pytest.mark.parametrize("precision,d,name,overfetch", [("fp8", 384, "ip", 4.0), ("bf16", 96, "sql2", 2.0)])
def test_batches_reduced_precision_equal_separate_calls(ss, precision, d, name, overfetch):
    # batches of one k share a packed search; a query's kept candidates do not
    # depend on the other queries of its search (padding rows, splits and the
    # shared pruning bounds leave the kept key set unchanged), so every batch
    # gets exactly the rows of a separate call with its own k -- also when its
    # search is replayed from a graph
    rng = np.random.default_rng(d + 1)
    sizes = [3, 64, 0, 17, 200, 1, 40]
    ks = [10, 1, 10, 100, 10, 1, 100]
    X, Q = data(rng, 20000, d, sum(sizes))
    dist = ss.Dist.SqL2() if name == "sql2" else ss.Dist.InnerProduct()
    idx = ss.GPUExhaustiveSearch(dist, ss.MatrixDatabase.from_rows(X), precision=precision, overfetch=overfetch)
    ctx = ss.GenericContext(logger=None)
    runs = [ss.searchbatches(idx, ctx, dbs(ss, split(Q, sizes)), ks) for _ in range(3)]
    for res in runs:
        for (ids, dists), q, k in zip(res, split(Q, sizes), ks):
            assert ids.shape == (k, q.shape[0])
            if q.shape[0] == 0:
                continue
            ri, rd = ss.searchbatch(idx, ctx, ss.MatrixDatabase.from_rows(q), k)
            assert np.array_equal(ids, ri) and np.array_equal(dists, rd)


def test_batches_argument_errors(ss):
    rng = np.random.default_rng(0)
    X, Q = data(rng, 300, 8, 4)
    idx = ss.GPUExhaustiveSearch(ss.Dist.SqL2(), ss.MatrixDatabase.from_rows(X))
    ctx = ss.GenericContext(logger=None)
    with pytest.raises(ss.ArgumentError):
        ss.searchbatches(idx, ctx, dbs(ss, [Q]), [0])
    with pytest.raises(ss.ArgumentError):
        ss.searchbatches(idx, ctx, dbs(ss, [Q, Q]), [1])
    with pytest.raises(ss.ArgumentError):
        ss.searchbatches(idx, ctx, dbs(ss, [Q[:, :4].copy()]), [1])
    assert [r[0].shape for r in ss.searchbatches(idx, ctx, dbs(ss, [Q[:0]]), [5])] == [(5, 0)]
