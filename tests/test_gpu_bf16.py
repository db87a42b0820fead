"""GPU tests of the BF16 tensor-core method (tcgen05 scan + exact FP32 rerank).

The method is approximate in which candidates survive the BF16 scan, exact in
what it reports: every returned distance is the plain FP32 distance of the
returned id (bit-identical to the oracle's sequential sum), rows are sorted
by (distance, id), and recall@k against the FP64 oracle is stated per case.
When the over-fetch keeps every database row, the result equals the plain
method exactly.
"""
import numpy as np
import pytest

from conftest import load_package
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NAMES = {"sql2": "SqL2", "l2": "L2", "normcosine": "NormCosine", "cosine": "Cosine", "ip": "InnerProduct"}


@pytest.fixture(scope="module")
def ss():
    mod = load_package()
    mod.build()
    return mod


def mixture(rng, n, d, centres=50, lo=0.1, hi=0.5, normalise=True):
    C = rng.standard_normal((centres, d), dtype=np.float32)
    sig = rng.uniform(lo, hi, size=centres).astype(np.float32)
    lab = rng.integers(0, centres, size=n)
    X = C[lab] + rng.standard_normal((n, d), dtype=np.float32) * sig[lab, None]
    if normalise:
        X /= np.linalg.norm(X, axis=1, keepdims=True)
    return X.astype(np.float32)


def run(ss, name, X, Q, k, **params):
    idx = ss.GPUExhaustiveSearch(getattr(ss.Dist, NAMES[name])(), ss.MatrixDatabase.from_rows(X),
                                 precision="bf16", **params)
    ids, dists = ss.searchbatch(idx, ss.GenericContext(), ss.MatrixDatabase.from_rows(Q), k)
    return np.ascontiguousarray(ids.T), np.ascontiguousarray(dists.T)


def check_reported_distances_exact(name, X, Q, gi, gd):
    for j in range(gi.shape[0]):
        pairs = []
        for t in range(gi.shape[1]):
            i = int(gi[j, t])
            assert i >= 1
            d = np.float32(O.evaluate(name, X[i - 1], Q[j]))
            assert gd[j, t] == d
            pairs.append((float(d), i))
        assert pairs == sorted(pairs)


@pytest.mark.parametrize("name", ["sql2", "l2", "normcosine", "cosine", "ip"])
@pytest.mark.parametrize("d", [32, 96, 100])
def test_bf16_recall_and_exact_distances(ss, name, d):
    rng = np.random.default_rng(d + len(name))
    X = mixture(rng, 6000, d, normalise=(name != "ip" and name != "sql2" and name != "l2"))
    Q = X[rng.integers(0, 6000, size=300)] + rng.standard_normal((300, d), dtype=np.float32) * 0.05
    if name in ("normcosine",):
        Q /= np.linalg.norm(Q, axis=1, keepdims=True)
    k = 10
    gi, gd = run(ss, name, X, Q, k, overfetch=2.0)
    check_reported_distances_exact(name, X, Q, gi[:40], gd[:40])
    fi, _ = O.searchbatch_f64(name, X, Q, k)
    assert O.macrorecall(fi, gi) >= 0.99


def test_bf16_full_overfetch_equals_plain(ss):
    # kk = n: every row is a candidate, the exact rerank decides everything
    rng = np.random.default_rng(3)
    X = rng.standard_normal((100, 96), dtype=np.float32)
    Q = rng.standard_normal((200, 96), dtype=np.float32)
    gi, gd = run(ss, "sql2", X, Q, 10, overfetch=64.0)
    ri, rd = O.searchbatch("sql2", X, Q, 10)
    assert np.array_equal(gi, ri) and np.array_equal(gd, rd)


@pytest.mark.parametrize("splits", [1, 3, 8])
def test_bf16_splits(ss, splits):
    rng = np.random.default_rng(4)
    X = mixture(rng, 9000, 64)
    Q = X[:130] + rng.standard_normal((130, 64), dtype=np.float32) * 0.02
    Q /= np.linalg.norm(Q, axis=1, keepdims=True)
    gi, gd = run(ss, "normcosine", X, Q, 16, overfetch=2.0, splits=splits)
    fi, _ = O.searchbatch_f64("normcosine", X, Q, 16)
    assert O.macrorecall(fi, gi) >= 0.99
    check_reported_distances_exact("normcosine", X, Q, gi[:20], gd[:20])


@pytest.mark.parametrize("m", [1, 127, 128, 129, 257, 600])
def test_bf16_query_counts(ss, m):
    rng = np.random.default_rng(m)
    X = mixture(rng, 3000, 96)
    Q = X[rng.integers(0, 3000, size=m)]
    gi, gd = run(ss, "normcosine", X, Q, 5, overfetch=2.0)
    fi, _ = O.searchbatch_f64("normcosine", X, Q, 5)
    assert O.macrorecall(fi, gi) >= 0.99


def test_bf16_allknn_exclude_self(ss):
    rng = np.random.default_rng(5)
    X = mixture(rng, 5000, 96, centres=20)
    idx = ss.GPUExhaustiveSearch(ss.Dist.NormCosine(), ss.MatrixDatabase.from_rows(X), precision="bf16",
                                 overfetch=1.5)
    ids, dists = ss.allknn(idx, ss.GenericContext(), 32, exclude_self=True)
    gi = np.ascontiguousarray(ids.T)
    assert not np.any(gi == np.arange(1, 5001, dtype=np.uint32)[:, None])
    rows = rng.choice(5000, size=300, replace=False)
    fi, _ = O.searchbatch_f64("normcosine", X, X[rows], 33)
    gold = np.zeros((300, 32), dtype=np.uint32)
    for r, j in enumerate(rows):
        keep = [t for t in range(33) if fi[r, t] != j + 1][:32]
        gold[r] = fi[r, keep]
    assert O.macrorecall(gold, gi[rows]) >= 0.99


@pytest.mark.parametrize("name", ["normcosine", "sql2", "cosine"])
def test_bf16_allknn_locality_order_identical(ss, name):
    # allknn scans a database of >= 32768 rows in its locality order (rows
    # grouped by nearest pivot, each query tile starting at its own group);
    # the kept (distance, id) keys do not depend on the order, so the result
    # equals the id-order scan exactly -- ties between duplicated rows, the
    # partial last tile and the scan's wrap-around included
    rng = np.random.default_rng(11 + len(name))
    n, d = 35007, 96
    X = mixture(rng, n, d, centres=300, normalise=(name != "sql2"))
    X[500:700] = X[:200]
    X[n - 50:] = X[1000:1050]
    dist = getattr(ss.Dist, NAMES[name])()
    idx = ss.GPUExhaustiveSearch(dist, ss.MatrixDatabase.from_rows(X), precision="bf16", overfetch=1.25)
    ids_l, dists_l = ss.allknn(idx, ss.GenericContext(), 16, exclude_self=True)
    idx.set_param("locality", 0)
    ids_p, dists_p = ss.allknn(idx, ss.GenericContext(), 16, exclude_self=True)
    assert np.array_equal(ids_l, ids_p)
    assert np.array_equal(dists_l, dists_p)
    idx.set_param("locality", 1)
    ids_2, _ = ss.allknn(idx, ss.GenericContext(), 16, exclude_self=True)
    assert np.array_equal(ids_l, ids_2)
    rows = rng.choice(n, size=200, replace=False)
    fi, _ = O.searchbatch_f64(name, X, X[rows], 17)
    gi = np.ascontiguousarray(ids_l.T)[rows]
    gold = np.zeros((200, 16), dtype=np.uint32)
    for r, j in enumerate(rows):
        keep = [t for t in range(17) if fi[r, t] != j + 1][:16]
        gold[r] = fi[r, keep]
    assert O.macrorecall(gold, gi) >= 0.98


@pytest.mark.parametrize("rows,chain,name", [(64, 1, "normcosine"), (1024, 0, "normcosine"), (1024, 1, "sql2"),
                                            (128, 1, "cosine")])
def test_bf16_allknn_locality_chain_variants(ss, rows, chain, name):
    # the pivots' chain order and the group size (rows per pivot) only
    # reorder the scan: the results equal the id-order scan's exactly, with
    # duplicated rows in different groups and a partial last tile
    rng = np.random.default_rng(rows + chain)
    n, d = 33001, 64
    X = mixture(rng, n, d, centres=200, normalise=(name != "sql2"))
    X[100:300] = X[20000:20200]
    dist = getattr(ss.Dist, NAMES[name])()
    idx = ss.GPUExhaustiveSearch(dist, ss.MatrixDatabase.from_rows(X), precision="bf16", overfetch=1.5)
    idx.set_param("locality", 0)
    ids_p, dists_p = ss.allknn(idx, ss.GenericContext(), 12, exclude_self=True)
    idx.set_param("locality", 1)
    idx.set_param("locality_rows", rows)
    idx.set_param("locality_chain", chain)
    assert idx.get_param("locality_rows") == rows and idx.get_param("locality_chain") == chain
    ids_l, dists_l = ss.allknn(idx, ss.GenericContext(), 12, exclude_self=True)
    assert np.array_equal(ids_l, ids_p)
    assert np.array_equal(dists_l, dists_p)


@pytest.mark.parametrize("d,k,name", [(96, 50, "normcosine"), (256, 10, "sql2"), (32, 1, "ip"), (200, 20, "cosine")])
def test_bf16_wide_equals_narrow(ss, d, k, name):
    # the wide scan (128 x 256 MMAs, K-block ring; at d = 96, k = 50 its
    # heaps leave room for three stages only, at d = 256 eight K-blocks per
    # tile) keeps exactly the candidates of the 128 x 128 scan; at d >= 200
    # the 128 x 128 scan's ring does not fit beside the heaps and the
    # threshold filter answers instead, with the same candidates unless it
    # falls back to the exact scan
    rng = np.random.default_rng(d + k)
    X = mixture(rng, 9000, d, normalise=(name != "sql2" and name != "ip"))
    Q = X[rng.integers(0, 9000, size=260)] + rng.standard_normal((260, d), dtype=np.float32) * 0.02
    if name == "normcosine":
        Q /= np.linalg.norm(Q, axis=1, keepdims=True)
    gi, gd = run(ss, name, X, Q, k, overfetch=1.25, wide=1)
    ni, nd = run(ss, name, X, Q, k, overfetch=1.25, wide=0)
    if d < 200:
        assert np.array_equal(gi, ni) and np.array_equal(gd, nd)
    check_reported_distances_exact(name, X, Q, gi[:10], gd[:10])
    fi, _ = O.searchbatch_f64(name, X, Q, k)
    assert O.macrorecall(fi, gi) >= 0.97


@pytest.mark.parametrize("name,d,k,m,splits", [("normcosine", 96, 32, 300, 0), ("sql2", 64, 10, 129, 3),
                                                ("cosine", 128, 20, 1000, 0), ("ip", 32, 5, 1, 0),
                                                ("sql2", 256, 8, 385, 2)])
def test_bf16_pair_scan_equals_single_cta_scan(ss, name, d, k, m, splits):
    # the pair scan (CTA pairs, M = 256 MMAs, each CTA loading half of every
    # database K-block) keeps exactly the candidates of the one-CTA wide
    # scan: odd query-tile counts (the last pair's second tile is padding),
    # forced database splits, one query
    rng = np.random.default_rng(d + k + m)
    X = mixture(rng, 12000, d, normalise=(name in ("normcosine", "cosine")))
    Q = X[rng.integers(0, 12000, size=m)] + rng.standard_normal((m, d), dtype=np.float32) * 0.02
    if name == "normcosine":
        Q /= np.linalg.norm(Q, axis=1, keepdims=True)
    pi, pd = run(ss, name, X, Q, k, overfetch=1.5, pair=1, splits=splits)
    wi, wd = run(ss, name, X, Q, k, overfetch=1.5, pair=0, splits=splits)
    assert np.array_equal(pi, wi) and np.array_equal(pd, wd)
    check_reported_distances_exact(name, X, Q, pi[:8], pd[:8])


@pytest.mark.parametrize("name", ["normcosine", "sql2"])
def test_bf16_pair_scan_allknn_locality_identical(ss, name):
    # allknn over 313 query tiles (odd) in the locality order on CTA pairs
    # equals the one-CTA scan, self excluded
    rng = np.random.default_rng(17 + len(name))
    n, d = 40000, 96
    X = mixture(rng, n, d, centres=300, normalise=(name != "sql2"))
    X[700:800] = X[:100]
    dist = getattr(ss.Dist, NAMES[name])()
    idx = ss.GPUExhaustiveSearch(dist, ss.MatrixDatabase.from_rows(X), precision="bf16", overfetch=1.5)
    ids_p, dists_p = ss.allknn(idx, ss.GenericContext(), 32, exclude_self=True)
    idx.set_param("pair", 0)
    ids_w, dists_w = ss.allknn(idx, ss.GenericContext(), 32, exclude_self=True)
    assert np.array_equal(ids_p, ids_w) and np.array_equal(dists_p, dists_w)


def test_bf16_autotune_scan_keeps_results(ss):
    # the autotuner times scan shapes (tile width, database splits); every
    # shape keeps the same candidates, so the tuned index answers exactly as
    # the default one
    rng = np.random.default_rng(21)
    X = mixture(rng, 20000, 96)
    Q = X[rng.integers(0, 20000, size=300)] + rng.standard_normal((300, 96), dtype=np.float32) * 0.02
    Q /= np.linalg.norm(Q, axis=1, keepdims=True)
    idx = ss.GPUExhaustiveSearch(ss.Dist.NormCosine(), ss.MatrixDatabase.from_rows(X), precision="bf16",
                                 overfetch=2.0)
    ctx = ss.GenericContext()
    qdb = ss.MatrixDatabase.from_rows(Q)
    ids0, d0 = ss.searchbatch(idx, ctx, qdb, 10)
    tuned = idx.autotune_scan(qdb, 10, repeats=1, splits=(0, 1, 4, 16))
    assert tuned["wide"] in (0, 1) and tuned["splits"] in (0, 1, 4, 16)
    assert len(tuned["timings"]) == 8
    assert idx.get_param("wide") == tuned["wide"] and idx.get_param("splits") == tuned["splits"]
    ids1, d1 = ss.searchbatch(idx, ctx, qdb, 10)
    assert np.array_equal(ids0, ids1) and np.array_equal(d0, d1)
    for w, sp in ((0, 1), (1, 16), (0, 16)):
        idx.set_param("wide", w)
        idx.set_param("splits", sp)
        ids2, d2 = ss.searchbatch(idx, ctx, qdb, 10)
        assert np.array_equal(ids0, ids2) and np.array_equal(d0, d2)


def test_bf16_rejects_hamming(ss):
    # Hamming distances are integers: only the exact method exists for them
    B = np.zeros((10, 2), dtype=np.uint64)
    with pytest.raises(ss._native.UnsupportedError):
        ss.GPUExhaustiveSearch(ss.Dist.Bits.Hamming(), ss.MatrixDatabase.from_rows(B), precision="bf16")


@pytest.mark.parametrize("name", ["sql2", "cosine", "ip"])
@pytest.mark.parametrize("n,k,d", [(30000, 200, 64), (6000, 300, 64), (20000, 150, 256)])
def test_bf16_large_k_threshold_filter(ss, name, n, k, d):
    # k beyond the on-chip heaps: the sampled-bound filter path (n > 8192) or
    # the every-row path (n <= 8192), then the exact rerank; at d = 256 the
    # filter scan runs with two ring stages and the sample scan wide
    rng = np.random.default_rng(n + k + len(name))
    X = mixture(rng, n, d, normalise=False)
    Q = X[rng.integers(0, n, size=150)] + rng.standard_normal((150, d), dtype=np.float32) * 0.05
    gi, gd = run(ss, name, X, Q, k, overfetch=1.5)
    check_reported_distances_exact(name, X, Q[:10], gi[:10], gd[:10])
    fi, _ = O.searchbatch_f64(name, X, Q, k)
    assert O.macrorecall(fi, gi) >= 0.99


def test_bf16_filter_overflow_falls_back_to_exact_scan(ss):
    # all rows equal: every distance ties, every row passes the bound, the
    # filtered lists overflow and each query is recomputed by the exact scan
    rng = np.random.default_rng(3)
    X = np.tile(rng.standard_normal((1, 48), dtype=np.float32), (20000, 1))
    Q = rng.standard_normal((9, 48), dtype=np.float32)
    idx = ss.GPUExhaustiveSearch(ss.Dist.SqL2(), ss.MatrixDatabase.from_rows(X), precision="bf16", overfetch=1.0,
                                 long_lists=0)
    ids, dists = ss.searchbatch(idx, ss.GenericContext(), ss.MatrixDatabase.from_rows(Q), 100)
    assert idx.get_param("fallbacks") == 9
    ri, rd = O.searchbatch("sql2", X, Q, 100)
    assert np.array_equal(np.ascontiguousarray(ids.T), ri) and np.array_equal(np.ascontiguousarray(dists.T), rd)


def test_bf16_allknn_large_k(ss):
    rng = np.random.default_rng(17)
    X = mixture(rng, 12000, 32)
    idx = ss.GPUExhaustiveSearch(ss.Dist.NormCosine(), ss.MatrixDatabase.from_rows(X), precision="bf16",
                                 overfetch=1.5)
    ids, _ = ss.allknn(idx, ss.GenericContext(), 120, exclude_self=True)
    gi = np.ascontiguousarray(ids.T)
    assert not np.any(gi == np.arange(1, 12001, dtype=np.uint32)[:, None])
    rows = rng.choice(12000, size=60, replace=False)
    fi, _ = O.searchbatch_f64("normcosine", X, X[rows], 121)
    gold = np.array([[i for i in fi[r] if i != j + 1][:120] for r, j in enumerate(rows)], dtype=np.uint32)
    assert O.macrorecall(gold, gi[rows]) >= 0.99


@pytest.mark.parametrize("name,d,k,of", [("normcosine", 96, 32, 4.0), ("sql2", 64, 100, 1.0), ("ip", 128, 48, 2.0)])
def test_bf16_long_lists_equal_threshold_filter(ss, name, d, k, of):
    # lists too long for two heaps per query (C2 as written: 4 (k + 1) = 132
    # candidates): CTA pairs with one heap per query keep exactly the kk
    # best approximate keys, as the threshold filter does
    rng = np.random.default_rng(d + k + 5)
    X = mixture(rng, 20000, d, normalise=(name == "normcosine"))
    Q = X[rng.integers(0, 20000, size=257)] + rng.standard_normal((257, d), dtype=np.float32) * 0.02
    if name == "normcosine":
        Q /= np.linalg.norm(Q, axis=1, keepdims=True)
    li, ld = run(ss, name, X, Q, k, overfetch=of, long_lists=1)
    fi, fd = run(ss, name, X, Q, k, overfetch=of, long_lists=0)
    assert np.array_equal(li, fi) and np.array_equal(ld, fd)
    check_reported_distances_exact(name, X, Q[:10], li[:10], ld[:10])


def test_bf16_long_lists_allknn_locality(ss):
    rng = np.random.default_rng(91)
    X = mixture(rng, 40000, 96)
    idx = ss.GPUExhaustiveSearch(ss.Dist.NormCosine(), ss.MatrixDatabase.from_rows(X), precision="bf16",
                                 overfetch=4.0)
    ctx = ss.GenericContext(logger=None)
    ids, dists = ss.allknn(idx, ctx, 32, exclude_self=True)
    idx.set_param("long_lists", 0)
    fi, fd = ss.allknn(idx, ctx, 32, exclude_self=True)
    assert np.array_equal(ids, fi) and np.array_equal(dists, fd)
