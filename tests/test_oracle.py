"""Pins the CPU oracle to SimilaritySearch.jl's own known answers and tests.

Each test restates one reference test (cited) against ``oracle/knn_oracle.c``.
These run without a GPU.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
KA = json.load(open(os.path.join(HERE, "golden", "known_answers.json")))


@pytest.mark.parametrize("case", KA["distances"], ids=lambda c: f"{c['metric']}@{c['cite']}")
def test_known_distance_values(case):
    # test/testdistances.jl:34-68,183-205
    m = case["metric"]
    if m == "hamming":
        a = np.array(case["a"], dtype=np.uint64)
        b = np.array(case["b"], dtype=np.uint64)
    else:
        a = np.array(case["a"], dtype=np.float32)
        b = np.array(case["b"], dtype=np.float32)
    got = np.float32(O.evaluate(m, a, b))
    if "expect_f32_sqrt_of" in case:
        expect = np.sqrt(np.float32(case["expect_f32_sqrt_of"]))
    else:
        expect = np.float32(case["expect"])
    if case["exact"]:
        assert got == expect
    else:
        assert abs(float(got) - float(expect)) <= case["atol"]
    # symmetry (testdistances.jl:26-29)
    assert abs(float(np.float32(O.evaluate(m, b, a))) - float(got)) <= 1e-5


@pytest.mark.parametrize("k", KA["knnsorted"]["ks"])
def test_knnsorted_matches_stable_sort(k):
    # test/testresults.jl:57-85: after each push, the queue equals the pushed
    # items stably sorted by distance, cut to k (ties keep insertion order).
    rng = np.random.default_rng(k)
    R = O.KnnSorted(k)
    gold = []
    for i in range(1, KA["knnsorted"]["pushes"] + 1):
        # quantised distances force many ties, exercising insert-after-equal
        p = float(np.float32(rng.integers(0, 50) / 50.0))
        gold.append((i, p))
        gold.sort(key=lambda x: x[1])  # Python's sort is stable
        if len(gold) > k:
            gold.pop()
        R.push(i, p)
        got = R.items()
        assert [g[0] for g in gold] == [x[0] for x in got]
        assert [np.float32(g[1]) for g in gold] == [np.float32(x[1]) for x in got]


def test_knnsorted_rejects_equal_frontier():
    # knnsorted.jl:163: a full queue rejects d == frontier
    R = O.KnnSorted(2)
    assert R.push(1, 1.0) and R.push(2, 2.0)
    assert not R.push(3, 2.0)
    assert R.push(4, 1.0)
    assert R.items() == [(1, 1.0), (4, 1.0)]


def _rand_db(rng, n, dim, metric):
    if metric == "hamming":
        return rng.integers(0, 2**63, size=(n, dim), dtype=np.uint64) * 2 + rng.integers(
            0, 2, size=(n, dim), dtype=np.uint64)
    return rng.random((n, dim), dtype=np.float32)


@pytest.mark.parametrize("k", KA["parallel"]["ks"])
def test_parallel_equals_sequential(k):
    # test/testparallelexhaustive.jl:21-37 (k in {1,4,n,n+5}, clamped to n)
    c = KA["parallel"]
    rng = np.random.default_rng(0)
    db = rng.random((c["n"], c["dim"]), dtype=np.float32)
    Q = rng.random((c["m"], c["dim"]), dtype=np.float32)
    kk = min(k, c["n"])
    for j in range(c["m"]):
        gi, gd = O.search("sql2", db, Q[j], kk)
        for minbatch in (1, 7, 64, c["n"]):
            pi, pd = O.parallel_search("sql2", db, Q[j], kk, minbatch)
            assert np.array_equal(gi, pi) and np.array_equal(gd, pd)


def test_searchbatch_and_allknn_parallel_forms():
    # test/testparallelexhaustive.jl:39-64: macrorecall == 1 and dists match
    c = KA["parallel"]
    rng = np.random.default_rng(0)
    db = rng.random((c["n"], c["dim"]), dtype=np.float32)
    Q = rng.random((c["m"], c["dim"]), dtype=np.float32)
    gi, gd = O.searchbatch("sql2", db, Q, c["batch_k"])
    pi, pd = O.searchbatch("sql2", db, Q, c["batch_k"], parallel_index=True, minbatch=37)
    assert O.macrorecall(gi, pi) == 1.0
    assert np.array_equal(gd, pd)
    ai, ad = O.allknn("sql2", db, c["allknn_k"])
    assert ai.shape == (c["n"], c["allknn_k"])
    # self is kept (allknn.jl:9-10): each object is its own nearest neighbour
    assert np.array_equal(ai[:, 0], np.arange(1, c["n"] + 1, dtype=np.uint32))


@pytest.mark.parametrize("case", KA["selfquery"]["cases"], ids=lambda c: c["metric"])
def test_selfquery_nearest(case):
    # test/testexactseq.jl:15-31,64-78
    rng = np.random.default_rng(1)
    db = _rand_db(rng, case["n"], case["dim"], case["metric"])
    if case["metric"] == "normcosine":
        db = db / np.linalg.norm(db, axis=1, keepdims=True)
    sel = rng.integers(0, case["n"], size=case["m"])
    ids, dists = O.searchbatch(case["metric"], db, db[sel], case["k"])
    assert np.all(dists[:, 0] < KA["selfquery"]["valid_lower"])


def test_unfilled_slots_are_zero_inf():
    # SimilaritySearch.jl:309-313: fewer than k items -> id 0, Inf32
    rng = np.random.default_rng(2)
    db = rng.random((3, 4), dtype=np.float32)
    ids, dists = O.searchbatch("sql2", db, db[:2], 5)
    assert np.all(ids[:, 3:] == 0) and np.all(np.isinf(dists[:, 3:]))
    assert np.all(ids[:, :3] > 0)


@pytest.mark.parametrize("metric", ["sql2", "l2", "normcosine", "cosine", "ip"])
def test_lane_reassociation_within_tolerance(metric):
    # @fastmath @simd (vecs.jl:96) may reassociate the sum; every lane count is
    # a valid execution and must agree within |dd| <= 1e-5 * max(|d|, 1).
    rng = np.random.default_rng(3)
    db = rng.standard_normal((500, 97), dtype=np.float32)
    q = rng.standard_normal((97,), dtype=np.float32)
    for i in range(0, 500, 7):
        d1 = O.evaluate(metric, db[i], q, lanes=1)
        for L in (4, 8, 16, 32):
            dl = O.evaluate(metric, db[i], q, lanes=L)
            assert abs(dl - d1) <= 1e-5 * max(abs(d1), 1.0)
        d64 = O.evaluate_f64(metric, db[i], q)
        assert abs(d64 - d1) <= 1e-5 * max(abs(d64), 1.0)


def test_hamming_ties_broken_by_id():
    # (dist, id) order: equal distances keep ascending ids; smallest ids win at k
    db = np.zeros((10, 2), dtype=np.uint64)
    db[3, 0] = 1
    q = np.zeros((1, 2), dtype=np.uint64)
    ids, dists = O.searchbatch("hamming", db, q, 4)
    assert ids[0].tolist() == [1, 2, 3, 5]
    assert dists[0].tolist() == [0.0, 0.0, 0.0, 0.0]


def test_rerank_sorts_by_exact_distance():
    # rerank.jl:22-41: re-score the non-zero prefix and sort it
    rng = np.random.default_rng(4)
    db = rng.random((50, 8), dtype=np.float32)
    q = rng.random((8,), dtype=np.float32)
    ids = np.array([5, 9, 1, 30, 0, 0], dtype=np.uint32)
    dists = np.zeros(6, dtype=np.float32)
    ri, rd = O.rerank("sql2", db, q, ids, dists)
    exact = {i: O.evaluate("sql2", db[i - 1], q) for i in (5, 9, 1, 30)}
    order = sorted(exact, key=lambda i: (exact[i], i))
    assert ri[:4].tolist() == order and ri[4:].tolist() == [0, 0]
    assert np.all(np.diff(rd[:4]) >= 0)


def test_macrorecall_definition():
    # perf.jl:31-33,71-79: set intersection over the first k, divided by k
    gold = np.array([[1, 2, 3], [4, 5, 6]], dtype=np.uint32)
    res = np.array([[3, 2, 9], [4, 5, 6]], dtype=np.uint32)
    assert O.macrorecall(gold, res) == pytest.approx((2 / 3 + 1) / 2)
    assert O.macrorecall(gold, res, 1) == pytest.approx((0 + 1) / 2)


def test_f64_gold_matches_f32_on_separated_data():
    rng = np.random.default_rng(5)
    db = rng.standard_normal((400, 16), dtype=np.float32)
    Q = rng.standard_normal((25, 16), dtype=np.float32)
    gi, _ = O.searchbatch_f64("sql2", db, Q, 10)
    fi, _ = O.searchbatch("sql2", db, Q, 10)
    assert O.macrorecall(gi, fi) == 1.0


def test_oracle_bitsketch_semantics():
    # packsigns (src/proj/bitsketches.jl:19-32): >= 0 -> bit 1 (zero included),
    # coordinate c in bit c % 64 of word c / 64, unused high bits 0;
    # cld(outdim, 64) words per sketch (test/testprojections.jl:67-75)
    R = np.zeros((70, 4), dtype=np.float32)        # outdim = 70 projection rows of indim = 4
    R[1] = [1, 0, 0, 0]
    R[2] = [-1, 0, 0, 0]
    R[65] = [0, 0, 0, -2]
    X = np.array([[1, 2, 3, 4], [-1, 0, 0, 1]], dtype=np.float32)
    B = O.bitsketch(R, X)
    assert B.shape == (2, 2) and B.dtype == np.uint64
    for r in range(2):
        bits = [(int(B[r, c // 64]) >> (c % 64)) & 1 for c in range(70)]
        for c in range(70):
            assert bits[c] == (1 if float(np.dot(R[c], X[r])) >= 0 else 0)
        assert int(B[r, 1]) >> 6 == 0               # coordinates 70..127 do not exist
    assert (int(B[0, 0]) >> 2) & 1 == 0 and (int(B[1, 0]) >> 2) & 1 == 1
