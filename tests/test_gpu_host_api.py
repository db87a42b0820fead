"""GPU tests of the host-facing forms of the path beyond the matrix
searchbatch: the queue-vector searchbatch! (src/SimilaritySearch.jl:384-398),
VectorDatabase inputs (src/db/vectordatabase.jl:30-104), and the three ways
SearchGraph construction and its tests use ExhaustiveSearch as a gold
standard, with GPUExhaustiveSearch in its place:

* optimize_index! (src/opt.jl:249-255): a SubDatabase sample of the database
  as queries, the queue-vector searchbatch! into KnnSorted queues, the gold
  id sets read from the queues;
* the static index's reference projection
  (src/searchgraph/staticindexing.jl:221-224): an ExhaustiveSearch over a
  SubDatabase of reference objects, searchbatch of the whole database;
* the allknn tests' gold (test/testallknn.jl:12-15): allknn of ExhaustiveSearch.

Every result is compared with the oracle's sequential (lanes=1) restatement:
the plain method's ids and distances are identical to it."""
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


def test_queue_vector_searchbatch_mixed_k_vs_oracle(ss):
    rng = np.random.default_rng(41)
    X = rng.standard_normal((5000, 24), dtype=np.float32)
    Q = rng.standard_normal((7, 24), dtype=np.float32)
    idx = ss.GPUExhaustiveSearch(ss.Dist.SqL2(), ss.MatrixDatabase.from_rows(X))
    ctx = ss.GenericContext(logger=None)
    ks = [1, 5, 10, 30, 3, 12, 7]
    knns = [ss.KnnSorted(k=k) for k in ks]
    # a queue that already holds an item: the search merges into it, as the
    # reference's pushes would (its search does not call reuse!)
    knns[2].push_item(4321, 0.5)
    out = ss.searchbatch_b(idx, ctx, ss.MatrixDatabase.from_rows(Q), knns)
    assert out is not None and len(out) == len(ks)
    for j, (k, res) in enumerate(zip(ks, knns)):
        ri, rd = O.searchbatch("sql2", X, Q[j:j + 1], k, lanes=1)
        ref = list(zip(ri[0].tolist(), rd[0].tolist()))
        if j == 2:
            ref = sorted(ref + [(4321, float(np.float32(0.5)))], key=lambda t: (t[1], t[0]))[:k]
        got = [(it.id, it.dist) for it in res.items()]
        assert [g[0] for g in got] == [r[0] for r in ref]
        assert np.array_equal(np.float32([g[1] for g in got]), np.float32([r[1] for r in ref]))
    assert ss.distance_evaluations(ctx) == 7 * 5000


def test_queue_vector_searchbatch_rejects_radius_queues(ss):
    rng = np.random.default_rng(42)
    X = rng.standard_normal((300, 8), dtype=np.float32)
    idx = ss.GPUExhaustiveSearch(ss.Dist.L2(), ss.MatrixDatabase.from_rows(X))
    Q = ss.MatrixDatabase.from_rows(X[:2])
    with pytest.raises(ss.ArgumentError):
        ss.searchbatch_b(idx, ss.GenericContext(logger=None), Q, [ss.RadiusSorted(0.3), ss.RadiusSorted(0.3)])


@pytest.mark.parametrize("name", ["sql2", "normcosine", "hamming"])
def test_vector_database_input_vs_oracle(ss, name):
    """A VectorDatabase database and query set are packed into contiguous
    rows on upload; results equal the oracle's on the same vectors, and
    push_item! into a VectorDatabase index grows both."""
    rng = np.random.default_rng(43)
    if name == "hamming":
        X = rng.integers(0, 2**64 - 1, size=(3000, 4), dtype=np.uint64, endpoint=True)
        Q = X[:40] ^ np.uint64(0x0F)
        dist = ss.Dist.Bits.Hamming()
    else:
        X = rng.standard_normal((3000, 33), dtype=np.float32)
        Q = rng.standard_normal((40, 33), dtype=np.float32)
        dist = ss.Dist.SqL2() if name == "sql2" else ss.Dist.NormCosine()
        if name == "normcosine":
            X /= np.linalg.norm(X, axis=1, keepdims=True)
            Q /= np.linalg.norm(Q, axis=1, keepdims=True)
    db = ss.VectorDatabase([x for x in X])
    idx = ss.GPUExhaustiveSearch(dist, db)
    ctx = ss.GenericContext(logger=None)
    ids, dists = ss.searchbatch(idx, ctx, ss.VectorDatabase([q for q in Q]), 15)
    ri, rd = O.searchbatch(name, X, Q, 15, lanes=1)
    assert np.array_equal(ids.T, ri) and np.array_equal(dists.T, rd)
    ss.push_item_b(idx, ctx, Q[0])
    assert len(idx) == 3001 and len(db) == 3001
    ids, dists = ss.searchbatch(idx, ctx, ss.VectorDatabase([Q[0]]), 3)
    assert ids[0, 0] == 3001 and dists[0, 0] <= (0.0 if name != "normcosine" else 1e-6)


def test_gold_standard_sample_queries_into_queues(ss):
    """optimize_index!'s gold (src/opt.jl:249-255): knnqueue views of a (k, m)
    matrix filled by the queue-vector searchbatch! over a SubDatabase sample."""
    rng = np.random.default_rng(44)
    X = rng.standard_normal((20000, 16), dtype=np.float32)
    db = ss.MatrixDatabase.from_rows(X)
    idx = ss.GPUExhaustiveSearch(ss.Dist.L2(), db)
    sample = np.unique(rng.integers(1, len(db) + 1, size=64))
    queries = ss.SubDatabase(db, sample)
    ksearch = 10
    knns_ids = np.zeros((ksearch, len(queries)), dtype=np.uint32, order="F")
    knns_dists = np.zeros((ksearch, len(queries)), dtype=np.float32, order="F")
    knns = [ss.knnqueue(ss.KnnSorted, knns_ids[:, i], knns_dists[:, i]) for i in range(len(queries))]
    ss.searchbatch_b(idx, ss.GenericContext(logger=None), queries, knns)
    gold = [set(int(it.id) for it in c.items()) for c in knns]
    ri, rd = O.searchbatch("l2", X, X[sample - 1], ksearch, lanes=1)
    assert gold == [set(r.tolist()) for r in ri]
    # the queues are views of the caller's matrices, filled in place
    assert np.array_equal(knns_ids.T, ri) and np.array_equal(knns_dists.T, rd)
    # each sampled object is its own nearest neighbour at distance 0
    assert np.array_equal(knns_ids[0], sample.astype(np.uint32))


def test_gold_standard_reference_projection(ss):
    """The static index's projection onto references
    (src/searchgraph/staticindexing.jl:221-224): ExhaustiveSearch over a
    SubDatabase of sorted reference ids, searchbatch of the whole database."""
    rng = np.random.default_rng(45)
    X = rng.standard_normal((30000, 12), dtype=np.float32)
    db = ss.MatrixDatabase.from_rows(X)
    ref_ids = np.sort(rng.permutation(len(db))[:512] + 1)
    refs_db = ss.SubDatabase(db, ref_ids)
    seq = ss.GPUExhaustiveSearch(ss.Dist.SqL2(), refs_db)
    knr_ids, knr_dists = ss.searchbatch(seq, ss.GenericContext(logger=None), db, 4)
    assert knr_ids.shape == (4, 30000)
    ri, rd = O.searchbatch("sql2", X[ref_ids - 1], X, 4, lanes=1)
    assert np.array_equal(knr_ids.T, ri) and np.array_equal(knr_dists.T, rd)


def test_gold_standard_allknn(ss):
    """The allknn tests' gold (test/testallknn.jl:12-15): allknn(E, ectx, k)."""
    rng = np.random.default_rng(46)
    X = rng.standard_normal((6000, 20), dtype=np.float32)
    E = ss.GPUExhaustiveSearch(ss.Dist.SqL2(), ss.MatrixDatabase.from_rows(X))
    ids, dists = ss.allknn(E, ss.GenericContext(logger=None), 8)
    ri, rd = O.allknn("sql2", X, 8, lanes=1)
    assert np.array_equal(ids.T, ri) and np.array_equal(dists.T, rd)
