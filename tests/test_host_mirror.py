"""The host mirror of the reference API (the package's own Python code above
the C ABI) pinned to SimilaritySearch.jl's known answers, without a GPU:
KnnSorted's order and frontier rule, knnqueue, macrorecall / recallscore and
the host-side distance evaluation.  The same known answers pin the oracle
(test_oracle.py)."""
import json
import os

import numpy as np
import pytest

from conftest import load_package
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
KA = json.load(open(os.path.join(HERE, "golden", "known_answers.json")))

NAMES = {"sql2": "SqL2", "l2": "L2", "normcosine": "NormCosine", "cosine": "Cosine", "ip": "InnerProduct"}


@pytest.fixture(scope="module")
def ss():
    return load_package()


@pytest.mark.parametrize("k", KA["knnsorted"]["ks"])
def test_knnsorted_mirror_matches_stable_sort(ss, k):
    # test/testresults.jl:57-85: after each push the queue holds the pushed
    # items stably sorted by distance and cut to k (ties keep push order)
    rng = np.random.default_rng(100 + k)
    R = ss.KnnSorted(k=k)
    gold = []
    for i in range(1, KA["knnsorted"]["pushes"] + 1):
        p = float(np.float32(rng.integers(0, 50) / 50.0))
        gold.append((i, p))
        gold.sort(key=lambda x: x[1])
        if len(gold) > k:
            gold.pop()
        R.push_item(i, p)
        got = R.items()
        assert [g[0] for g in gold] == [x.id for x in got]
        assert [np.float32(g[1]) for g in gold] == [np.float32(x.dist) for x in got]
    assert R.nearest() == got[0] and R.frontier() == got[-1]


def test_knnsorted_mirror_rejects_equal_frontier(ss):
    # knnsorted.jl:163: a full queue rejects a distance equal to its frontier
    R = ss.KnnSorted(k=3)
    for i, d in ((1, 0.5), (2, 0.25), (3, 0.75)):
        assert R.push_item(i, d)
    assert R.covradius() == np.float32(0.75)
    assert not R.push_item(4, 0.75)
    assert R.push_item(5, 0.5)
    assert [x.id for x in R.items()] == [2, 1, 5]


def test_knnsorted_mirror_equals_oracle_queue(ss):
    rng = np.random.default_rng(7)
    for k in (1, 5, 32):
        A, B = ss.KnnSorted(k=k), O.KnnSorted(k)
        for i in range(1, 400):
            d = float(np.float32(rng.integers(0, 30) / 7.0))
            A.push_item(i, d)
            B.push(i, d)
        assert [(x.id, np.float32(x.dist)) for x in A.items()] == [(x[0], np.float32(x[1])) for x in B.items()]


def test_knnqueue_wraps_columns(ss):
    ids = np.zeros(4, dtype=np.uint32)
    dists = np.full(4, np.inf, dtype=np.float32)
    q = ss.knnqueue(ss.KnnSorted, ids, dists)
    q.push_item(9, 1.5)
    q.push_item(3, 0.5)
    assert list(ids[:2]) == [3, 9] and list(dists[:2]) == [np.float32(0.5), np.float32(1.5)]
    assert ss.knnqueue(ss.KnnSorted, 6).maxlength() == 6
    with pytest.raises(TypeError):
        ss.knnqueue(dict, 3)


def test_macrorecall_mirror_equals_oracle(ss):
    # perf.jl:31-33,71-79: mean over columns of |gold ∩ res| / |gold|
    rng = np.random.default_rng(3)
    gold = np.stack([rng.permutation(50)[:10] + 1 for _ in range(40)], axis=1).astype(np.uint32)
    res = gold.copy()
    res[rng.integers(0, 10, size=40), np.arange(40)] = 99
    r = ss.macrorecall(gold, res)
    assert r == pytest.approx(0.9)
    assert r == pytest.approx(O.macrorecall(gold.T, res.T))
    assert ss.recallscore([1, 2, 3, 4], [4, 3, 9, 8]) == 0.5


@pytest.mark.parametrize("case", [c for c in KA["distances"] if c["metric"] in NAMES or c["metric"] == "hamming"],
                         ids=lambda c: f"{c['metric']}@{c['cite']}")
def test_host_evaluate_known_values(ss, case):
    # test/testdistances.jl:34-68,183-205 through the package's Dist types
    m = case["metric"]
    if m == "hamming":
        dist = ss.Dist.Bits.Hamming()
        a = np.array(case["a"], dtype=np.uint64)
        b = np.array(case["b"], dtype=np.uint64)
    else:
        dist = getattr(ss.Dist, NAMES[m])()
        a = np.array(case["a"], dtype=np.float32)
        b = np.array(case["b"], dtype=np.float32)
    got = np.float32(ss.evaluate(dist, a, b))
    if "expect_f32_sqrt_of" in case:
        expect = np.sqrt(np.float32(case["expect_f32_sqrt_of"]))
    else:
        expect = np.float32(case["expect"])
    tol = 0.0 if m == "hamming" else max(float(case.get("atol", 0.0)), 1e-5 * max(1.0, abs(float(expect))))
    assert abs(float(got) - float(expect)) <= tol


def test_queue_vector_searchbatch_rejects_radius_queues_before_searching(ss):
    """searchbatch!(index, ctx, Q, knns) with a radius queue raises
    ArgumentError (src/SimilaritySearch.jl:384-398 accepts any
    AbstractMetricQueue; the GPU index answers fixed-k queries only and never
    falls back to another method).  Checked before any search runs, so an
    index object that would fail if touched stands in for the GPU index."""
    import pytest
    from similaritysearch_gb300.index import _searchbatch_queues

    class Untouchable:
        def __getattr__(self, name):
            raise AssertionError("the index must not be used")

    Q = ss.MatrixDatabase.from_rows(np.zeros((3, 4), dtype=np.float32))
    ctx = ss.GenericContext(logger=None)
    queues = [ss.KnnSorted(k=5), ss.RadiusSorted(0.3), ss.KnnSorted(k=2)]
    with pytest.raises(ss.ArgumentError, match="KnnSorted"):
        _searchbatch_queues(Untouchable(), ctx, Q, queues)
    with pytest.raises(ss.ArgumentError, match="number of queries"):
        _searchbatch_queues(Untouchable(), ctx, Q, [ss.KnnSorted(k=5)])
    with pytest.raises(ss.ArgumentError, match="not a result queue"):
        _searchbatch_queues(Untouchable(), ctx, Q, [ss.KnnSorted(k=5), None, ss.KnnSorted(k=1)])


def test_radius_sorted_mirror_keeps_items_within_radius_sorted(ss):
    """RadiusSorted (src/pqueue/radiussorted.jl:28-52): accepts dist <= radius,
    keeps ascending order, later equal distances after earlier ones."""
    r = ss.RadiusSorted(0.5)
    for i, d in [(1, 0.4), (2, 0.6), (3, 0.1), (4, 0.4), (5, 0.5)]:
        r.push_item(i, d)
    assert r.ids == [3, 1, 4, 5]
    assert r.dists == [np.float32(0.1), np.float32(0.4), np.float32(0.4), np.float32(0.5)]
