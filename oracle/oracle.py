"""ctypes front end of ``knn_oracle.c`` -- TEST INFRASTRUCTURE ONLY.

The C file restates SimilaritySearch.jl's ``ExhaustiveSearch`` /
``ParallelExhaustiveSearch`` / ``KnnSorted`` / ``allknn`` / ``rerank!`` /
``macrorecall`` (file:line citations are in its header).  This module builds it
on demand with the committed Makefile and exposes numpy-friendly wrappers.

Layout convention (same as the GPU library): a Julia ``Matrix{Float32}(d, n)``
is column-major, which is a C-contiguous numpy array of shape ``(n, d)``;
result matrices ``(k, m)`` are numpy arrays of shape ``(m, k)``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

SQL2, L2, NORMCOSINE, COSINE, IP, HAMMING = 0, 1, 2, 3, 4, 5
METRIC_NAMES = {"sql2": SQL2, "l2": L2, "normcosine": NORMCOSINE, "cosine": COSINE,
                "ip": IP, "hamming": HAMMING}

_lib = None
_lock = threading.Lock()

_p = C.c_void_p
_i64 = C.c_int64
_i32 = C.c_int32
_int = C.c_int


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, no CUDA)."""
    if force or not os.path.exists(LIB_PATH) or (
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "knn_oracle.c"))):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(LIB_PATH)
            L.oracle_knnsorted_push.argtypes = [_p, _p, _i32, _p, _p, _i32, C.c_uint32, C.c_float]
            L.oracle_knnsorted_push.restype = _int
            L.oracle_evaluate.argtypes = [_int, _p, _p, _i64, _int]
            L.oracle_evaluate.restype = C.c_float
            L.oracle_evaluate_f64.argtypes = [_int, _p, _p, _i64]
            L.oracle_evaluate_f64.restype = C.c_double
            L.oracle_search.argtypes = [_int, _p, _i64, _i64, _p, _i32, _p, _p, _int]
            L.oracle_parallel_search.argtypes = [_int, _p, _i64, _i64, _p, _i32, _p, _p, _int, _i64]
            L.oracle_searchbatch.argtypes = [_int, _p, _i64, _i64, _p, _i64, _i32, _p, _p, _int,
                                             _int, _int, _i64]
            L.oracle_allknn.argtypes = [_int, _p, _i64, _i64, _i32, _p, _p, _int, _int]
            L.oracle_allknn_rows.argtypes = [_int, _p, _i64, _i64, _i32, _p, _i64, _p, _p, _int, _int]
            L.oracle_searchbatch_f64.argtypes = [_int, _p, _i64, _i64, _p, _i64, _i32, _p, _p, _int]
            L.oracle_rerank.argtypes = [_int, _p, _i64, _p, _p, _p, _i32, _int]
            L.oracle_macrorecall.argtypes = [_p, _i64, _p, _i64, _i64, _i64]
            L.oracle_bitsketch.argtypes = [_p, _i64, _i64, _p, _i64, _p, _int]
            L.oracle_bitsketch.restype = None
            L.oracle_macrorecall.restype = C.c_double
            L.oracle_num_threads.restype = _int
            _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _metric(metric) -> int:
    return METRIC_NAMES[metric] if isinstance(metric, str) else int(metric)


def _prep(metric, X):
    m = _metric(metric)
    if m == HAMMING:
        X = np.ascontiguousarray(X, dtype=np.uint64)
    else:
        X = np.ascontiguousarray(X, dtype=np.float32)
    if X.ndim == 1:
        X = X.reshape(1, -1)
    return m, X


class KnnSorted:
    """Host restatement of ``KnnSorted`` (knnsorted.jl:31-168) over the C push."""

    def __init__(self, k: int, cap: int | None = None):
        cap = k if cap is None else cap
        self.ids = np.zeros(cap, dtype=np.uint32)
        self.dists = np.zeros(cap, dtype=np.float32)
        self.k = k
        self._sp = C.c_int32(1)
        self._ep = C.c_int32(0)

    def push(self, i: int, d: float) -> bool:
        return bool(lib().oracle_knnsorted_push(_ptr(self.ids), _ptr(self.dists), len(self.ids),
                                                C.byref(self._sp), C.byref(self._ep), self.k,
                                                int(i), float(d)))

    def __len__(self):
        return self._ep.value - self._sp.value + 1

    def items(self):
        s, e = self._sp.value - 1, self._ep.value
        return list(zip(self.ids[s:e].tolist(), self.dists[s:e].tolist()))


def bitsketch(R, X, lanes: int = 1) -> np.ndarray:
    """Sign sketches of the rows of X (n x indim) against the projection R
    given as outdim rows of indim: n rows of ceil(outdim / 64) UInt64 words
    (oracle_bitsketch; src/proj/bitsketches.jl:19-32,56-57,101-104)."""
    R = np.ascontiguousarray(R, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.float32)
    assert R.shape[1] == X.shape[1]
    out = np.zeros((X.shape[0], (R.shape[0] + 63) // 64), dtype=np.uint64)
    lib().oracle_bitsketch(_ptr(R), R.shape[1], R.shape[0], _ptr(X), X.shape[0], _ptr(out), lanes)
    return out


def evaluate(metric, a, b, lanes: int = 1) -> float:
    m, A = _prep(metric, a)
    _, B = _prep(metric, b)
    return float(lib().oracle_evaluate(m, _ptr(A), _ptr(B), A.shape[1], lanes))


def evaluate_f64(metric, a, b) -> float:
    m, A = _prep(metric, a)
    _, B = _prep(metric, b)
    return float(lib().oracle_evaluate_f64(m, _ptr(A), _ptr(B), A.shape[1]))


def search(metric, db, q, k: int, lanes: int = 1):
    """One query through ExhaustiveSearch; returns (ids[k], dists[k])."""
    m, X = _prep(metric, db)
    _, Q = _prep(metric, q)
    ids = np.zeros(k, dtype=np.uint32)
    dists = np.full(k, np.inf, dtype=np.float32)
    lib().oracle_search(m, _ptr(X), X.shape[1], X.shape[0], _ptr(Q), k, _ptr(ids), _ptr(dists), lanes)
    return ids, dists


def parallel_search(metric, db, q, k: int, minbatch: int, lanes: int = 1):
    """One query through the ParallelExhaustiveSearch restatement."""
    m, X = _prep(metric, db)
    _, Q = _prep(metric, q)
    ids = np.zeros(k, dtype=np.uint32)
    dists = np.full(k, np.inf, dtype=np.float32)
    lib().oracle_parallel_search(m, _ptr(X), X.shape[1], X.shape[0], _ptr(Q), k, _ptr(ids),
                                 _ptr(dists), lanes, int(minbatch))
    return ids, dists


def searchbatch(metric, db, Q, k: int, lanes: int = 1, nthreads: int = 0,
                parallel_index: bool = False, minbatch: int = 1):
    """searchbatch(ExhaustiveSearch or ParallelExhaustiveSearch, ctx, Q, k).

    Returns ``(ids, dists)`` of shape ``(m, k)`` (row j = Julia column j)."""
    m_, X = _prep(metric, db)
    _, Qa = _prep(metric, Q)
    mq = Qa.shape[0]
    ids = np.zeros((mq, k), dtype=np.uint32)
    dists = np.empty((mq, k), dtype=np.float32)
    lib().oracle_searchbatch(m_, _ptr(X), X.shape[1], X.shape[0], _ptr(Qa), mq, k, _ptr(ids),
                             _ptr(dists), lanes, nthreads, 1 if parallel_index else 0, int(minbatch))
    return ids, dists


def allknn(metric, db, k: int, lanes: int = 1, nthreads: int = 0):
    m_, X = _prep(metric, db)
    n = X.shape[0]
    ids = np.zeros((n, k), dtype=np.uint32)
    dists = np.empty((n, k), dtype=np.float32)
    lib().oracle_allknn(m_, _ptr(X), X.shape[1], n, k, _ptr(ids), _ptr(dists), lanes, nthreads)
    return ids, dists


def allknn_rows(metric, db, k: int, rows, lanes: int = 1, nthreads: int = 0):
    """allknn for the listed objects only (0-based rows) -- sampled baselines."""
    m_, X = _prep(metric, db)
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    ids = np.zeros((rows.size, k), dtype=np.uint32)
    dists = np.empty((rows.size, k), dtype=np.float32)
    lib().oracle_allknn_rows(m_, _ptr(X), X.shape[1], X.shape[0], k, _ptr(rows), rows.size,
                             _ptr(ids), _ptr(dists), lanes, nthreads)
    return ids, dists


def searchbatch_f64(metric, db, Q, k: int, nthreads: int = 0):
    """Gold standard ranked by (FP64 distance, id)."""
    m_, X = _prep(metric, db)
    _, Qa = _prep(metric, Q)
    mq = Qa.shape[0]
    ids = np.zeros((mq, k), dtype=np.uint32)
    dists = np.empty((mq, k), dtype=np.float64)
    lib().oracle_searchbatch_f64(m_, _ptr(X), X.shape[1], X.shape[0], _ptr(Qa), mq, k, _ptr(ids),
                                 _ptr(dists), nthreads)
    return ids, dists


def rerank(metric, db, q, ids, dists, lanes: int = 1):
    m_, X = _prep(metric, db)
    _, Qa = _prep(metric, q)
    ids = np.ascontiguousarray(ids, dtype=np.uint32).copy()
    dists = np.ascontiguousarray(dists, dtype=np.float32).copy()
    lib().oracle_rerank(m_, _ptr(X), X.shape[1], _ptr(Qa), _ptr(ids), _ptr(dists), ids.size, lanes)
    return ids, dists


def macrorecall(gold, res, k: int | None = None) -> float:
    """macrorecall(goldI, resI, k) with (m, k)-shaped numpy id matrices."""
    g = np.ascontiguousarray(gold, dtype=np.uint32)
    r = np.ascontiguousarray(res, dtype=np.uint32)
    if k is None:
        k = g.shape[1]
    return float(lib().oracle_macrorecall(_ptr(g), g.shape[1], _ptr(r), r.shape[1], g.shape[0], k))


def num_threads() -> int:
    return int(lib().oracle_num_threads())


def closestpairs(metric, A, B, k: int, min_k: int, samedata: bool, lanes: int = 1):
    """The k closest pairs (i in A, j in B, dist), 1-based, restating
    bichromatic_kclosestpairs (src/bichromatic/bichromaticclosestpairs.jl):
    each object j of B is searched for its min_k nearest objects of A
    (KnnSorted order; with samedata the object itself is excluded, as
    bichromatic_search! does), its candidates are offered in ascending order
    to a bounded top-k (insert_topk!), and the buffers are merged.  Ties are
    ordered by (distance, j, rank), the order the GPU's merge produces; the
    reference's order among equal distances depends on its batching."""
    A = np.ascontiguousarray(A)
    B = np.ascontiguousarray(B)
    take = min_k + (1 if samedata else 0)
    take = min(take, A.shape[0])
    ids, dists = searchbatch(metric, A, B, take, lanes=lanes)
    cand = []
    for j in range(B.shape[0]):
        row = [(float(dists[j, t]), int(ids[j, t])) for t in range(take) if ids[j, t] != 0]
        if samedata:
            if any(i == j + 1 for _, i in row):
                row = [p for p in row if p[1] != j + 1]
            else:
                row = row[:-1]
        for r, (d, i) in enumerate(row[:min_k]):
            cand.append((d, j + 1, r, i))
    cand.sort()
    return [(i, j, d) for d, j, r, i in cand[:k]]


def neardup(metric, X, eps: float, blocksize: int = 256, filterblocks: bool = True, lanes: int = 1):
    """Restates neardup_ / neardup_block! (src/neardup.jl:101-244) with an
    exact index: returns (nn, dist, map) with 1-based ids.  The search of a
    block against the net takes the nearest net object (KnnSorted order);
    inside a block an object joins the net unless the nearest already
    accepted object of the block (smallest distance, earliest first) is
    within eps."""
    X = np.ascontiguousarray(X)
    n = X.shape[0]
    eps = np.float32(eps)
    L = np.zeros(n, dtype=np.int32)
    D = np.zeros(n, dtype=np.float32)
    M = []

    def block(imap):
        keep = [imap[0]] if filterblocks else list(imap)
        if filterblocks:
            for i in imap[1:]:
                best_d, best_j = None, None
                for j in keep:
                    d = np.float32(evaluate(metric, X[i], X[j], lanes))
                    if best_d is None or d < best_d:
                        best_d, best_j = d, j
                if best_d > eps:
                    keep.append(i)
                else:
                    L[i], D[i] = best_j + 1, best_d
        for i in keep:
            M.append(i + 1)
            L[i], D[i] = i + 1, 0.0

    blocksize = max(1, min(blocksize, n))
    for start in range(0, n, blocksize):
        rng = list(range(start, min(n, start + blocksize)))
        if not M:
            block(rng)
            continue
        net = X[np.array(M) - 1]
        ids, dists = searchbatch(metric, net, X[rng], 1, lanes=lanes)
        imap = []
        for t, j in enumerate(rng):
            if dists[t, 0] > eps:
                imap.append(j)
            else:
                L[j], D[j] = M[int(ids[t, 0]) - 1], dists[t, 0]
        if imap:
            block(imap)
    return L, D, np.array(M, dtype=np.uint32)
