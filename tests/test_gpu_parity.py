"""GPU parity: libssgpu through the C ABI against the oracle and the golden fixtures.

The plain FP32 path sums every distance in index order with one FMA per
element, exactly like the oracle's ``lanes=1`` chain, so ids AND distances
must be identical.  Against other (SIMD-style) summation orders the
tolerance is the one the path promises: |d_gpu - d_ref| <= 1e-5 * max(|d_ref|, 1),
with ids equal outside near-tie bands of that width.  Hamming is bit-exact.
"""
import os

import numpy as np
import pytest

from conftest import ROOT, load_package
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RTOL = 1e-5
GOLD = np.load(os.path.join(ROOT, "tests", "golden", "knn_golden.npz"))


@pytest.fixture(scope="module")
def ss():
    mod = load_package()
    mod.build()
    return mod


def gpu_search(ss, dist, X, Q, k, **params):
    idx = ss.GPUExhaustiveSearch(dist, ss.MatrixDatabase.from_rows(X), **params)
    ctx = ss.GenericContext()
    ids, dists = ss.searchbatch(idx, ctx, ss.MatrixDatabase.from_rows(Q), k)
    # (k, m) -> (m, k) rows, the oracle's layout
    return np.ascontiguousarray(ids.T), np.ascontiguousarray(dists.T), idx, ctx


DISTS = {"sql2": "SqL2", "l2": "L2", "normcosine": "NormCosine", "cosine": "Cosine", "ip": "InnerProduct"}


def dist_of(ss, name):
    if name == "hamming":
        return ss.Dist.Bits.Hamming()
    return getattr(ss.Dist, DISTS[name])()


def assert_within_tolerance(gi, gd, ri, rd):
    """Distances within RTOL; ids equal except inside near-tie bands."""
    assert gi.shape == ri.shape
    tol = RTOL * np.maximum(np.abs(rd), 1.0)
    assert np.all(np.abs(gd - rd) <= tol)
    mism = gi != ri
    if np.any(mism):
        # a differing id must sit at a distance tied (within tolerance) with another slot
        for j, t in zip(*np.nonzero(mism)):
            row = rd[j]
            near = np.abs(row - row[t]) <= 2 * tol[j, t]
            assert near.sum() >= 2 or t == row.size - 1


@pytest.mark.parametrize("name", ["sql2", "l2", "normcosine", "cosine", "ip"])
def test_golden_float(ss, name):
    X, Q = GOLD[f"{name}_X"], GOLD[f"{name}_Q"]
    k = GOLD[f"{name}_ids"].shape[1]
    gi, gd, _, _ = gpu_search(ss, dist_of(ss, name), X, Q, k)
    assert np.array_equal(gi, GOLD[f"{name}_ids"])
    assert np.array_equal(gd, GOLD[f"{name}_dists"])


def test_golden_hamming_ties(ss):
    X, Q = GOLD["hamming_X"], GOLD["hamming_Q"]
    gi, gd, _, _ = gpu_search(ss, ss.Dist.Bits.Hamming(), X, Q, 16)
    assert np.array_equal(gi, GOLD["hamming_ids"])
    assert np.array_equal(gd, GOLD["hamming_dists"])


def test_golden_allknn(ss):
    X = GOLD["allknn_X"]
    idx = ss.GPUExhaustiveSearch(ss.Dist.SqL2(), ss.MatrixDatabase.from_rows(X))
    ids, dists = ss.allknn(idx, ss.GenericContext(), 4)
    assert np.array_equal(ids.T, GOLD["allknn_ids"])
    assert np.array_equal(dists.T, GOLD["allknn_dists"])


@pytest.mark.parametrize("name", ["sql2", "l2", "normcosine", "cosine", "ip"])
@pytest.mark.parametrize("k", [1, 10, 100])
def test_float_metrics_bitexact_vs_oracle(ss, name, k):
    rng = np.random.default_rng(k * 7 + len(name))
    n, d, m = 3000, 37, 150
    X = rng.standard_normal((n, d), dtype=np.float32)
    Q = rng.standard_normal((m, d), dtype=np.float32)
    if name == "normcosine":
        X /= np.linalg.norm(X, axis=1, keepdims=True)
        Q /= np.linalg.norm(Q, axis=1, keepdims=True)
    gi, gd, _, _ = gpu_search(ss, dist_of(ss, name), X, Q, k)
    ri, rd = O.searchbatch(name, X, Q, k, lanes=1)
    assert np.array_equal(gi, ri)
    assert np.array_equal(gd, rd)
    # and within the stated tolerance of a SIMD-reassociated reference sum
    si, sd = O.searchbatch(name, X, Q, k, lanes=16)
    assert_within_tolerance(gi, gd, si, sd)


@pytest.mark.parametrize("splits", [1, 2, 3, 7, 33])
def test_splits_do_not_change_results(ss, splits):
    rng = np.random.default_rng(11)
    X = rng.standard_normal((5000, 24), dtype=np.float32)
    Q = rng.standard_normal((70, 24), dtype=np.float32)
    gi, gd, _, _ = gpu_search(ss, ss.Dist.SqL2(), X, Q, 25, splits=splits)
    ri, rd = O.searchbatch("sql2", X, Q, 25)
    assert np.array_equal(gi, ri) and np.array_equal(gd, rd)


@pytest.mark.parametrize("splits,k", [(64, 200), (148, 130), (40, 500)])
def test_many_splits_need_merge_passes(ss, splits, k):
    # splits x k candidates beyond one merge block go through reduction passes
    rng = np.random.default_rng(splits + k)
    X = rng.standard_normal((30000, 20), dtype=np.float32)
    Q = rng.standard_normal((50, 20), dtype=np.float32)
    for name in ("sql2", "normcosine"):
        gi, gd, _, _ = gpu_search(ss, dist_of(ss, name), X, Q, k, splits=splits)
        ri, rd = O.searchbatch(name, X, Q, k)
        assert np.array_equal(gi, ri) and np.array_equal(gd, rd)
    gi, gd, _, _ = gpu_search(ss, ss.Dist.SqL2(), X, Q, k, splits=splits, exact_scan=1)
    ri, rd = O.searchbatch("sql2", X, Q, k)
    assert np.array_equal(gi, ri) and np.array_equal(gd, rd)


@pytest.mark.parametrize("k", [1, 4, 300, 305])
def test_parallel_exhaustive_k_cases(ss, k):
    # test/testparallelexhaustive.jl:21-37: k in {1, 4, n, n+5} on n=300, dim=6
    rng = np.random.default_rng(0)
    X = rng.random((300, 6), dtype=np.float32)
    Q = rng.random((40, 6), dtype=np.float32)
    gi, gd, _, _ = gpu_search(ss, ss.Dist.SqL2(), X, Q, k)
    kk = min(k, 300)
    ri, rd = O.searchbatch("sql2", X, Q, kk)
    assert np.array_equal(gi[:, :kk], ri) and np.array_equal(gd[:, :kk], rd)
    if k > 300:
        assert np.all(gi[:, 300:] == 0) and np.all(np.isinf(gd[:, 300:]))


def test_large_k_uses_global_heaps(ss):
    rng = np.random.default_rng(12)
    X = rng.standard_normal((4000, 16), dtype=np.float32)
    Q = rng.standard_normal((9, 16), dtype=np.float32)
    gi, gd, _, _ = gpu_search(ss, ss.Dist.L2(), X, Q, 1024)
    ri, rd = O.searchbatch("l2", X, Q, 1024)
    assert np.array_equal(gi, ri) and np.array_equal(gd, rd)


@pytest.mark.parametrize("name", ["sql2", "l2", "normcosine"])
def test_duplicates_break_ties_by_id(ss, name):
    # 40 copies of every vector: ties at the k-th boundary everywhere.  For
    # SqL2 / L2 the GEMM-form margin cannot be proven sufficient, so those
    # queries must go through the exact fallback scan -- and still match.
    rng = np.random.default_rng(13)
    base = rng.standard_normal((50, 8), dtype=np.float32)
    if name == "normcosine":
        base /= np.linalg.norm(base, axis=1, keepdims=True)
    X = np.repeat(base, 40, axis=0)
    rng.shuffle(X)
    Q = base[:10].copy()
    for k in (24, 64):  # 24: GEMM-form scan + fallback; 64: heaps exceed it -> exact scan
        gi, gd, idx, _ = gpu_search(ss, dist_of(ss, name), X, Q, k)
        ri, rd = O.searchbatch(name, X, Q, k)
        assert np.array_equal(gi, ri) and np.array_equal(gd, rd)
        if name != "normcosine" and k == 24:
            assert idx.get_param("fallbacks") > 0


@pytest.mark.parametrize("name", ["sql2", "l2", "normcosine", "cosine", "ip"])
def test_exact_direct_scan_forced(ss, name):
    # the exact direct scan (the fallback) on its own, every metric
    rng = np.random.default_rng(21)
    X = rng.standard_normal((2000, 45), dtype=np.float32)
    Q = rng.standard_normal((70, 45), dtype=np.float32)
    gi, gd, idx, _ = gpu_search(ss, dist_of(ss, name), X, Q, 12, exact_scan=1)
    ri, rd = O.searchbatch(name, X, Q, 12)
    assert np.array_equal(gi, ri) and np.array_equal(gd, rd)


@pytest.mark.parametrize("margin", [1, 4, 64])
def test_gemm_margin_is_self_checking(ss, margin):
    # a tiny margin may fail the completeness check; results stay exact
    rng = np.random.default_rng(22)
    X = rng.standard_normal((3000, 33), dtype=np.float32)
    Q = X[rng.integers(0, 3000, size=90)] + rng.standard_normal((90, 33), dtype=np.float32) * 1e-3
    gi, gd, _, _ = gpu_search(ss, ss.Dist.SqL2(), X, Q, 10, margin=margin)
    ri, rd = O.searchbatch("sql2", X, Q, 10)
    assert np.array_equal(gi, ri) and np.array_equal(gd, rd)


@pytest.mark.parametrize("W", [1, 3, 8, 16, 32])
def test_hamming_bitexact(ss, W):
    rng = np.random.default_rng(W)
    n, m, k = 20000, 300, 100
    X = rng.integers(0, 2**64 - 1, size=(n, W), dtype=np.uint64, endpoint=True)
    src = rng.integers(0, n, size=m)
    flips = rng.random((m, W * 64)) < 0.1
    mask = np.ascontiguousarray(np.packbits(flips, axis=1)).view(np.uint64)
    Q = X[src] ^ mask
    gi, gd, _, _ = gpu_search(ss, ss.Dist.Bits.Hamming(), X, Q, k)
    ri, rd = O.searchbatch("hamming", X, Q, k)
    assert np.array_equal(gi, ri)
    assert np.array_equal(gd, rd)


def test_selfquery_nearest(ss):
    # test/testexactseq.jl:15-31: the nearest distance of a self-query is < 1e-3
    rng = np.random.default_rng(1)
    X = rng.random((200, 4), dtype=np.float32)
    Q = X[rng.integers(0, 200, size=20)]
    _, gd, _, _ = gpu_search(ss, ss.Dist.SqL2(), X, Q, 4)
    assert np.all(gd[:, 0] < 1e-3)


@pytest.mark.parametrize("exclude_self", [False, True])
def test_allknn_vs_oracle(ss, exclude_self):
    rng = np.random.default_rng(14)
    X = rng.standard_normal((2500, 20), dtype=np.float32)
    X /= np.linalg.norm(X, axis=1, keepdims=True)
    idx = ss.GPUExhaustiveSearch(ss.Dist.NormCosine(), ss.MatrixDatabase.from_rows(X))
    ids, dists = ss.allknn(idx, ss.GenericContext(), 10, exclude_self=exclude_self)
    gi, gd = ids.T, dists.T
    ri, rd = O.allknn("normcosine", X, 11 if exclude_self else 10)
    if exclude_self:
        ei = np.zeros((2500, 10), dtype=np.uint32)
        ed = np.zeros((2500, 10), dtype=np.float32)
        for j in range(2500):
            keep = [t for t in range(11) if ri[j, t] != j + 1][:10]
            ei[j], ed[j] = ri[j, keep], rd[j, keep]
        ri, rd = ei, ed
    assert np.array_equal(gi, ri) and np.array_equal(gd, rd)


@pytest.mark.parametrize("dtype", [np.float64, np.float16, np.uint8, np.int8])
def test_castf32_twins(ss, dtype):
    rng = np.random.default_rng(15)
    lo, hi = (0, 255) if dtype == np.uint8 else (-100, 100)
    X = rng.uniform(lo, hi, size=(800, 12)).astype(dtype)
    Q = rng.uniform(lo, hi, size=(30, 12)).astype(dtype)
    gi, gd, _, _ = gpu_search(ss, ss.Dist.CastF32.SqL2(), X, Q, 9)
    ri, rd = O.searchbatch("sql2", X.astype(np.float32), Q.astype(np.float32), 9)
    assert np.array_equal(gi, ri) and np.array_equal(gd, rd)


def test_plain_metric_rejects_non_float32(ss):
    X = np.zeros((10, 3), dtype=np.float64)
    with pytest.raises(ss.ArgumentError):
        ss.GPUExhaustiveSearch(ss.Dist.SqL2(), ss.MatrixDatabase.from_rows(X))


def test_rerank_vs_oracle(ss):
    rng = np.random.default_rng(16)
    X = rng.standard_normal((700, 10), dtype=np.float32)
    Q = rng.standard_normal((25, 10), dtype=np.float32)
    idx = ss.GPUExhaustiveSearch(ss.Dist.L2(), ss.MatrixDatabase.from_rows(X))
    cand = rng.integers(1, 701, size=(12, 25)).astype(np.uint32)
    cand[9:, ::3] = 0  # some lists end early
    dists = np.zeros((12, 25), dtype=np.float32)
    ids = np.asfortranarray(cand.copy())
    dists = np.asfortranarray(dists)
    ss.rerank_b(idx, ss.MatrixDatabase.from_rows(Q), ids, dists)
    for j in range(25):
        ri, rd = O.rerank("l2", X, Q[j], cand[:, j], np.zeros(12, np.float32))
        assert np.array_equal(ids[:, j], ri)
        valid = ri != 0
        assert np.array_equal(dists[valid, j], rd[valid])


def test_append_and_log_events(ss):
    # test/testlog.jl:72-100: one :add! per append with the exact range, :info for index!
    rng = np.random.default_rng(17)
    X = rng.standard_normal((100, 6), dtype=np.float32)
    rec = ss.RecorderLog()
    ctx = ss.GenericContext(logger=rec)
    idx = ss.GPUExhaustiveSearch(ss.Dist.L2(), ss.MatrixDatabase.from_rows(X))
    extra = rng.standard_normal((5, 6), dtype=np.float32)
    ss.append_items_b(idx, ctx, ss.MatrixDatabase.from_rows(extra))
    assert rec.events == [("add!", 101, 105)]
    rec.events.clear()
    ss.index_b(idx, ctx)
    assert len(rec.events) == 1 and rec.events[0][0] == "info"
    ss.push_item_b(idx, ctx, extra[0] + 1)
    assert rec.events[-1] == ("add!", 106, 106)
    assert len(idx) == 106
    full = np.concatenate([X, extra, extra[:1] + 1])
    Q = rng.standard_normal((20, 6), dtype=np.float32)
    ids, dists = ss.searchbatch(idx, ctx, ss.MatrixDatabase.from_rows(Q), 8)
    ri, rd = O.searchbatch("l2", full, Q, 8)
    assert np.array_equal(ids.T, ri) and np.array_equal(dists.T, rd)
    assert ss.distance_evaluations(ctx) == 106 * 20


def test_search_single_query_fills_knnsorted(ss):
    rng = np.random.default_rng(18)
    X = rng.standard_normal((400, 5), dtype=np.float32)
    q = rng.standard_normal(5, dtype=np.float32)
    idx = ss.GPUExhaustiveSearch(ss.Dist.SqL2(), ss.MatrixDatabase.from_rows(X))
    res = ss.knnqueue(ss.KnnSorted, 7)
    ss.search(idx, ss.GenericContext(), q, res)
    ri, rd = O.search("sql2", X, q, 7)
    assert [it.id for it in res.items()] == ri.tolist()
    assert [np.float32(it.dist) for it in res.items()] == rd.tolist()


def test_errors_leave_index_usable(ss):
    rng = np.random.default_rng(19)
    X = rng.standard_normal((100, 4), dtype=np.float32)
    idx = ss.GPUExhaustiveSearch(ss.Dist.SqL2(), ss.MatrixDatabase.from_rows(X))
    ctx = ss.GenericContext()
    with pytest.raises(ss.ArgumentError):
        ss.searchbatch(idx, ctx, ss.MatrixDatabase(np.zeros((4, 0), np.float32)), 3)
    with pytest.raises(ss.ArgumentError):
        ss.searchbatch(idx, ctx, ss.MatrixDatabase.from_rows(np.zeros((2, 5), np.float32)), 3)
    with pytest.raises(ss.ArgumentError):
        ss.allknn(idx, ctx, 101)
    with pytest.raises(ss.ArgumentError):
        idx.set_param("nonsense", 1)
    Q = rng.standard_normal((3, 4), dtype=np.float32)
    ids, dists = ss.searchbatch(idx, ctx, ss.MatrixDatabase.from_rows(Q), 3)
    ri, rd = O.searchbatch("sql2", X, Q, 3)
    assert np.array_equal(ids.T, ri) and np.array_equal(dists.T, rd)


def test_sorted_output_and_counters(ss):
    rng = np.random.default_rng(20)
    X = rng.standard_normal((1000, 8), dtype=np.float32)
    Q = rng.standard_normal((64, 8), dtype=np.float32)
    gi, gd, idx, ctx = gpu_search(ss, ss.Dist.SqL2(), X, Q, 20)
    for j in range(64):  # (dist, id) lexicographic order per row
        pairs = list(zip(gd[j].tolist(), gi[j].tolist()))
        assert pairs == sorted(pairs)
    assert ss.distance_evaluations(ctx) == 1000 * 64
    assert idx.get_param("kernel_launches") >= 2
