"""GPUExhaustiveSearch: the drop-in index for the searchbatch / allknn path.

Mirrors the reference's ``AbstractSearchIndex`` surface for
``ExhaustiveSearch`` / ``ParallelExhaustiveSearch``
(src/exact/sequential-exhaustive.jl:18-80, src/exact/parallel-exhaustive.jl:26-123):
``search``, ``searchbatch``, ``searchbatch_b`` (``searchbatch!``), ``allknn``,
``allknn_b``, ``push_item_b``, ``append_items_b``, ``index_b``, ``distance``,
``database``, ``len``.  Julia's ``f!`` is spelled ``f_b`` here.

Result matrices keep Julia's shapes: ``ids`` is a ``(k, m)`` UInt32 array and
``dists`` a ``(k, m)`` Float32 array, both Fortran-ordered so that column ``j``
(query ``j``) is contiguous -- the bytes of a Julia ``Matrix``.  Ids are
1-based; unfilled slots hold 0 / Inf32.

Every call goes through libssgpu.so.  There is no CPU path: without the
built library or a GPU, calls raise.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .db import AbstractDatabase, MatrixDatabase, MMapMatrixDatabase, VectorDatabase, as_database
from .dist import PreMetric
from .log import LOG, InformativeLog
from .pqueue import AbstractKnnQueue, AbstractMetricQueue, KnnSorted

ArgumentError = N.ArgumentError

_ELEM = {
    np.dtype(np.float32): N.ELEM_F32,
    np.dtype(np.uint64): N.ELEM_U64,
    np.dtype(np.float64): N.ELEM_F64,
    np.dtype(np.float16): N.ELEM_F16,
    np.dtype(np.uint8): N.ELEM_U8,
    np.dtype(np.int8): N.ELEM_I8,
}
_PREC = {"fp32": N.PREC_FP32, "bf16": N.PREC_BF16, "fp8": N.PREC_FP8}


class GenericContext:
    """Mirror of GenericContext (src/SimilaritySearch.jl:192-224): logger and
    the distance-evaluation counters (``costdists``)."""

    def __init__(self, verbose: bool = True, logger=None, maxbatches: int = 64):
        self.verbose = verbose
        self.logger = InformativeLog() if logger is None else logger
        self.maxbatches = maxbatches
        self.costdists = [0] * maxbatches
        self.costblocks = [0] * maxbatches
        self.batchid = 0


def add_distance_evaluations(ctx, v: int):
    # add_distance_evaluations!(ctx, v) (SimilaritySearch.jl:224)
    ctx.costdists[ctx.batchid] += int(v)


def distance_evaluations(ctx) -> int:
    return int(sum(ctx.costdists))


def _element_type(dist: PreMetric, dtype) -> int:
    dt = np.dtype(dtype)
    if dist.code == N.METRIC_HAMMING:
        if dt != np.uint64:
            raise ArgumentError("Bits.Hamming needs UInt64 sketches")
        return N.ELEM_U64
    if dt == np.float32:
        return N.ELEM_F32
    if not dist.cast_f32:
        raise ArgumentError(f"{dist!r} on {dt} data: use the Dist.CastF32 twin to cast to Float32")
    if dt not in _ELEM:
        raise ArgumentError(f"element type {dt} is not supported")
    return _ELEM[dt]


class GPUExhaustiveSearch:
    """Exact brute-force index on one GPU.  ``precision`` selects the plain
    FP32 method ("fp32") or the reduced-precision ones with FP32 rerank."""

    def __init__(self, dist: PreMetric, db, precision: str = "fp32", **params):
        self.dist = dist
        self.db = as_database(db)
        self.precision = precision
        if precision not in _PREC:
            raise ArgumentError(f"unknown precision {precision!r}")
        rows = self.db.rows()
        if rows.ndim != 2 or rows.shape[1] == 0:
            raise ArgumentError("GPUExhaustiveSearch needs the database's dimension (a (dim, n) matrix)")
        self._elem = _element_type(dist, rows.dtype)
        self._dtype = rows.dtype
        self.dim = rows.shape[1]
        h = C.c_void_p()
        lib = N.lib()
        if isinstance(self.db, MMapMatrixDatabase):
            # straight from the file into device memory
            N.check(lib.ssg_create_mmap(dist.code, self.db.path.encode(), _PREC[precision], C.byref(h)))
        else:
            N.check(lib.ssg_create(dist.code, self._elem, self.dim, rows.shape[0], rows.ctypes.data_as(C.c_void_p),
                                   self.dim, _PREC[precision], C.byref(h)))
        self._h = h
        for k, v in params.items():
            self.set_param(k, v)

    # -- plumbing --------------------------------------------------------
    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            N.lib().ssg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_param(self, key: str, value: float):
        N.check(N.lib().ssg_set_param(self._h, key.encode(), float(value)), self._h)

    def get_param(self, key: str) -> float:
        v = C.c_double()
        N.check(N.lib().ssg_get_param(self._h, key.encode(), C.byref(v)), self._h)
        return v.value

    def __len__(self):
        return int(self.get_param("n"))

    def autotune_overfetch(self, Q, k: int, target_recall: float = 0.99,
                           candidates=(1.0, 1.25, 1.5, 2.0, 3.0, 4.0, 6.0, 8.0, 12.0, 16.0)) -> float:
        """Picks the smallest over-fetch whose recall@k on the calibration
        queries ``Q`` reaches ``target_recall`` against the plain FP32 method
        on the same index (which matches ExhaustiveSearch), sets it and
        returns it.  A no-op returning 1.0 for the plain method."""
        if self.precision == "fp32":
            return 1.0
        ctx = GenericContext(logger=None)
        self.set_param("plain", 1)
        try:
            gold, _ = searchbatch(self, ctx, Q, k)
        finally:
            self.set_param("plain", 0)
        from .perf import macrorecall
        chosen = candidates[-1]
        for c in candidates:
            self.set_param("overfetch", c)
            ids, _ = searchbatch(self, ctx, Q, k)
            if macrorecall(gold, ids) >= target_recall:
                chosen = c
                break
        self.set_param("overfetch", chosen)
        return chosen

    def autotune_scan(self, Q, k: int, repeats: int = 3,
                      splits=(0, 1, 2, 4, 8, 16, 32, 64), widths=(1, 0)) -> dict:
        """Picks the scan shape for searches like ``searchbatch(self, ctx, Q,
        k)`` by timing them: the database tile width of the BF16 scan
        ("wide": 128 x 256 or 128 x 128 MMA tiles) and the database splits
        per query tile ("splits", 0 = the wave model).  Every shape keeps the
        same candidates, so only the time changes; the fastest (median of
        ``repeats`` calls after a warm-up) is set and returned with the
        timings.  A no-op for the plain method."""
        import time
        if self.precision == "fp32":
            return {}
        ctx = GenericContext(logger=None)
        widths = widths if self.precision == "bf16" else (int(self.get_param("wide")),)
        before = (int(self.get_param("wide")), int(self.get_param("splits")))
        timings = {}
        try:
            for w in widths:
                self.set_param("wide", w)
                for s in splits:
                    self.set_param("splits", s)
                    searchbatch(self, ctx, Q, k)
                    ts = []
                    for _ in range(max(1, repeats)):
                        t0 = time.perf_counter()
                        searchbatch(self, ctx, Q, k)
                        ts.append(time.perf_counter() - t0)
                    timings[(w, s)] = sorted(ts)[len(ts) // 2]
        except BaseException:
            # a failed trial leaves the index as it was
            self.set_param("wide", before[0])
            self.set_param("splits", before[1])
            raise
        best = min(timings, key=timings.get)
        self.set_param("wide", best[0])
        self.set_param("splits", best[1])
        return {"wide": best[0], "splits": best[1], "seconds": timings[best],
                "timings": {f"wide={w},splits={s}": t for (w, s), t in timings.items()}}

    def train_mlp(self, sample: int = 50_000, triplets: int = 200_000, epochs: int = 4, hidden: int = 256,
                  out_dim: int = 64, batch: int = 1024, lr: float = 1e-3, seed: int = 1,
                  target_recall: float | None = None) -> dict:
        """Trains the learned shortlist (``ssg_train_mlp``): a d -> hidden ->
        out_dim network under a triplet loss whose positives are exact
        neighbours found by this index, then indexes the embedded database.
        ``hidden=0`` builds the untrained random-projection baseline instead.
        Searches take the learned path while the estimated recall@10 against
        the plain method reaches ``target_recall`` (default 0.99), the plain
        method otherwise.  Returns the training statistics."""
        if target_recall is not None:
            self.set_param("learned_target", target_recall)
        N.check(N.lib().ssg_train_mlp(self._h, int(sample), int(triplets), int(epochs), int(hidden), int(out_dim),
                                      int(batch), float(lr), int(seed)), self._h)
        return self.learned_stats()

    def learned_stats(self) -> dict:
        keys = ("learned_ready", "learned_recall", "learned_target", "train_loss", "train_seconds", "train_steps",
                "shortlist")
        return {k: self.get_param(k) for k in keys}

    def save_model(self, path: str):
        N.check(N.lib().ssg_save_model(self._h, str(path).encode()), self._h)

    def load_model(self, path: str) -> dict:
        N.check(N.lib().ssg_load_model(self._h, str(path).encode()), self._h)
        return self.learned_stats()

    def _queries(self, Q) -> np.ndarray:
        Qdb = as_database(Q)
        rows = Qdb.rows()
        if rows.ndim != 2 or (rows.shape[0] > 0 and rows.shape[1] != self.dim):
            raise ArgumentError(f"queries have dimension {rows.shape[-1]}, the index has {self.dim}")
        if rows.dtype != self._dtype:
            rows = rows.astype(self._dtype)
        return np.ascontiguousarray(rows)


def distance(idx: GPUExhaustiveSearch):
    return idx.dist


def database(idx: GPUExhaustiveSearch, i: int | None = None):
    return idx.db if i is None else idx.db[i]


def _check_out(ids, dists, m):
    if ids.dtype != np.uint32 or dists.dtype != np.float32:
        raise ArgumentError("ids must be UInt32 and dists Float32")
    if ids.ndim != 2 or ids.shape != dists.shape:
        raise ArgumentError("ids and dists must be (k, m) matrices of the same shape")
    if ids.shape[1] != m:
        raise ArgumentError("the number of queries is different from the given output containers")


def _col_major_view(a: np.ndarray):
    """(k, m) matrix -> (pointer, needs_copy_back) with column-contiguous bytes."""
    if a.flags.f_contiguous:
        return a, False
    return np.asfortranarray(a), True


def searchbatch_b(idx: GPUExhaustiveSearch, ctx: GenericContext, Q, ids, dists: np.ndarray | None = None,
                  sorted: bool = False):
    """searchbatch!(index, ctx, Q, ids, dists; sorted) -- src/SimilaritySearch.jl:331-348.
    Columns come back sorted by (distance, id) whether or not ``sorted``.

    searchbatch!(index, ctx, Q, knns) -- src/SimilaritySearch.jl:384-398:
    with a sequence of per-query queues in place of ``ids`` (and no
    ``dists``), query j's results are pushed into ``knns[j]``."""
    if dists is None and not isinstance(ids, np.ndarray):
        return _searchbatch_queues(idx, ctx, Q, ids)
    rows = idx._queries(Q)
    m = rows.shape[0]
    if m <= 0:
        raise ArgumentError("empty set of queries")
    _check_out(ids, dists, m)
    k = ids.shape[0]
    oi, ci = _col_major_view(ids)
    od, cd = _col_major_view(dists)
    N.check(N.lib().ssg_search(idx.handle, rows.ctypes.data_as(C.c_void_p), idx.dim, m, k,
                               oi.ctypes.data_as(C.c_void_p), od.ctypes.data_as(C.c_void_p), 0), idx.handle)
    if ci:
        ids[...] = oi
    if cd:
        dists[...] = od
    add_distance_evaluations(ctx, len(idx) * m)
    return ids, dists


def _searchbatch_queues(idx: GPUExhaustiveSearch, ctx: GenericContext, Q, knns):
    """The queue-vector searchbatch!: one GPU search with the largest k of the
    queues, then each KnnSorted queue receives its query's first maxlength()
    results in (distance, id) order -- the state the reference's pushes of
    every object would leave, since a queue of k keeps exactly the first k of
    that order (also when it already held items).  Radius queues and other
    containers raise ArgumentError: the GPU index answers fixed-k queries
    only, and does not fall back to another method."""
    knns = list(knns)
    m = len(as_database(Q))
    if m <= 0:
        raise ArgumentError("empty set of queries")
    if m != len(knns):
        raise ArgumentError("the number of queries is different from the given output containers")
    for res in knns:
        if not isinstance(res, AbstractMetricQueue):
            raise ArgumentError(f"{type(res).__name__} is not a result queue")
        if not isinstance(res, KnnSorted):
            raise ArgumentError(f"the GPU index fills KnnSorted queues only, not {type(res).__name__}")
    k = max(res.maxlength() for res in knns)
    ids, dists = searchbatch(idx, ctx, Q, k)
    for j, res in enumerate(knns):
        for i in range(res.maxlength()):
            if ids[i, j] == 0:
                break
            res.push_item(int(ids[i, j]), float(dists[i, j]))
    return knns


def searchbatch(idx: GPUExhaustiveSearch, ctx: GenericContext, Q, k: int, sorted: bool = True):
    """searchbatch(index, ctx, Q, k) -> (ids (k, m), dists (k, m))  -- SimilaritySearch.jl:309-313"""
    m = len(as_database(Q))
    ids = np.zeros((k, m), dtype=np.uint32, order="F")
    dists = np.full((k, m), np.inf, dtype=np.float32, order="F")
    return searchbatch_b(idx, ctx, Q, ids, dists, sorted=sorted)


def searchbatches(idx: GPUExhaustiveSearch, ctx: GenericContext, Qs, ks):
    """Several query batches of different sizes and k answered by one search
    (``ssg_search_batches``): the request-stream form of calling
    ``searchbatch`` once per request.  Returns one ``(ids (k, m), dists (k, m))``
    pair per batch.  Device staging goes through torch tensors."""
    import torch
    if len(Qs) != len(ks) or not Qs:
        raise ArgumentError("need one k per batch and at least one batch")
    qs = [idx._queries(Q) for Q in Qs]
    host = [q.view(np.int64) if q.dtype == np.uint64 else q for q in qs]   # torch has no uint64 tensors
    dev_q = [torch.from_numpy(h).cuda() if h.shape[0] else None for h in host]
    outs_i = [torch.empty((q.shape[0], int(k)), dtype=torch.int32, device="cuda") for q, k in zip(qs, ks)]
    outs_d = [torch.empty((q.shape[0], int(k)), dtype=torch.float32, device="cuda") for q, k in zip(qs, ks)]
    nb = len(qs)
    P = C.c_void_p * nb
    ptr = lambda t: t.data_ptr() if t is not None and t.numel() else None
    N.check(N.lib().ssg_search_batches(
        idx._h, nb, P(*[ptr(t) for t in dev_q]), (C.c_int64 * nb)(*[q.shape[0] for q in qs]),
        (C.c_int32 * nb)(*[int(k) for k in ks]), P(*[ptr(t) for t in outs_i]), P(*[ptr(t) for t in outs_d])),
        idx._h)
    res = []
    for q, ti, td in zip(qs, outs_i, outs_d):
        add_distance_evaluations(ctx, q.shape[0] * len(idx))
        res.append((np.asfortranarray(ti.cpu().numpy().view(np.uint32).T),
                    np.asfortranarray(td.cpu().numpy().T)))
    return res


def search(idx: GPUExhaustiveSearch, ctx: GenericContext, q, res: AbstractKnnQueue):
    """search(index, ctx, q, res): one query as a batch of one; the results are
    pushed into ``res`` in (distance, id) order (sequential-exhaustive.jl:68-80)."""
    if not isinstance(res, KnnSorted):
        raise ArgumentError("the GPU index fills KnnSorted queues only")
    k = res.maxlength()
    q = np.asarray(q)
    Qm = MatrixDatabase(q.reshape(-1, 1))
    ids, dists = searchbatch(idx, ctx, Qm, k)
    for i in range(k):
        if ids[i, 0] == 0:
            break
        res.push_item(int(ids[i, 0]), float(dists[i, 0]))
    return res


def allknn_b(idx: GPUExhaustiveSearch, ctx: GenericContext, ids: np.ndarray, dists: np.ndarray,
             sort: bool = True, progress=None, exclude_self: bool = False):
    """allknn!(index, ctx, ids, dists) -- src/allknn.jl:66-91.  The object
    itself is kept unless ``exclude_self`` (an extension of this index)."""
    n = len(idx)
    if ids.ndim != 2 or ids.shape != dists.shape:
        raise ArgumentError("ids and dists must be (k, n) matrices")
    k, nn = ids.shape
    if not n > 0:
        raise ArgumentError("invalid assertion n > 0")
    if nn != n:
        raise ArgumentError("invalid assertion n == m")
    if not 0 < k <= n:
        raise ArgumentError("invalid assertion 0 < k <= n")
    oi, ci = _col_major_view(ids)
    od, cd = _col_major_view(dists)
    N.check(N.lib().ssg_allknn(idx.handle, k, 1 if exclude_self else 0, oi.ctypes.data_as(C.c_void_p),
                               od.ctypes.data_as(C.c_void_p)), idx.handle)
    if ci:
        ids[...] = oi
    if cd:
        dists[...] = od
    add_distance_evaluations(ctx, n * n)
    return ids, dists


def allknn(idx: GPUExhaustiveSearch, ctx: GenericContext, k: int, sort: bool = True, progress=None,
           exclude_self: bool = False):
    """allknn(index, ctx, k) -> (ids (k, n), dists (k, n)) -- src/allknn.jl:39-47"""
    n = len(idx)
    ids = np.zeros((k, n), dtype=np.uint32, order="F")
    dists = np.full((k, n), np.inf, dtype=np.float32, order="F")
    return allknn_b(idx, ctx, ids, dists, sort=sort, progress=progress, exclude_self=exclude_self)


def push_item_b(idx: GPUExhaustiveSearch, ctx: GenericContext, u):
    """push_item!(index, ctx, u) -- sequential-exhaustive.jl:33-38"""
    row = np.ascontiguousarray(np.asarray(u, dtype=idx._dtype).reshape(1, -1))
    if row.shape[1] != idx.dim:
        raise ArgumentError("object dimension does not match the index")
    N.check(N.lib().ssg_append(idx.handle, row.ctypes.data_as(C.c_void_p), 1), idx.handle)
    if isinstance(idx.db, VectorDatabase):
        idx.db.push_item(row[0])
    else:
        idx.db = MatrixDatabase(np.concatenate([idx.db.matrix, row.T], axis=1))
    n = len(idx)
    LOG(ctx.logger, "add!", idx, ctx, n, n)
    return idx


def append_items_b(idx: GPUExhaustiveSearch, ctx: GenericContext, u: AbstractDatabase):
    """append_items!(index, ctx, db) -- sequential-exhaustive.jl:40-46: one
    ``add!`` event for the appended range (none for an empty batch)."""
    rows = idx._queries(u)
    sp = len(idx) + 1
    if rows.shape[0] > 0:
        N.check(N.lib().ssg_append(idx.handle, rows.ctypes.data_as(C.c_void_p), rows.shape[0]), idx.handle)
        if isinstance(idx.db, VectorDatabase):
            idx.db.append_items(list(rows))
        else:
            idx.db = MatrixDatabase(np.concatenate([idx.db.matrix, rows.T], axis=1))
    ep = len(idx)
    if ep >= sp:
        LOG(ctx.logger, "add!", idx, ctx, sp, ep)
    return idx


def index_b(idx: GPUExhaustiveSearch, ctx: GenericContext):
    """index!(index, ctx): a no-op for a brute-force index; logs ``info``
    (sequential-exhaustive.jl:48-53)."""
    n = len(idx)
    LOG(ctx.logger, "info", idx, ctx, n, n)
    return idx


def rerank_b(idx: GPUExhaustiveSearch, queries, knns_ids: np.ndarray, knns_dists: np.ndarray):
    """rerank!(dist, db, queries, ids, dists) -- src/rerank.jl:77-86, on the
    GPU against the index's database and distance.  Each column is re-scored
    exactly (the first 0 id ends it) and sorted by (distance, id)."""
    rows = idx._queries(queries)
    m = rows.shape[0]
    if knns_ids.ndim != 2 or knns_ids.shape != knns_dists.shape or knns_ids.shape[1] != m:
        raise ArgumentError("ids and dists must be (len, m) matrices with one column per query")
    oi, ci = _col_major_view(np.ascontiguousarray(knns_ids, dtype=np.uint32) if knns_ids.dtype != np.uint32 else knns_ids)
    od, cd = _col_major_view(knns_dists)
    N.check(N.lib().ssg_rerank(idx.handle, rows.ctypes.data_as(C.c_void_p), m, knns_ids.shape[0],
                               oi.ctypes.data_as(C.c_void_p), od.ctypes.data_as(C.c_void_p)), idx.handle)
    if oi is not knns_ids:
        knns_ids[...] = oi
    if od is not knns_dists:
        knns_dists[...] = od
    return knns_ids, knns_dists


def bichromatic_kclosestpairs(idx: GPUExhaustiveSearch, ctx: GenericContext, B, k: int = 1, min_k: int | None = None,
                              samedata: bool | None = None):
    """The k closest pairs (i in the index, j in B, dist), ascending by
    distance (src/bichromatic/bichromaticclosestpairs.jl): every object of B
    takes its min_k nearest indexed objects (itself excluded when
    ``samedata``, by default when B is the index's own database) and the k
    best candidates overall are kept.  Ids are 1-based."""
    min_k = max(k, 8) if min_k is None else min_k
    if min_k < k:
        raise ArgumentError("min_k must be >= k")
    own = B is None or B is idx.db
    if samedata is None:
        samedata = own
    oi = np.zeros(k, dtype=np.int32)
    oj = np.zeros(k, dtype=np.int32)
    od = np.zeros(k, dtype=np.float32)
    cnt = C.c_int64(0)
    if own:
        m = len(idx)
        N.check(N.lib().ssg_closestpairs(idx._h, None, 0, k, min_k, 1, oi.ctypes.data_as(C.c_void_p),
                                         oj.ctypes.data_as(C.c_void_p), od.ctypes.data_as(C.c_void_p),
                                         C.byref(cnt)), idx._h)
    else:
        rows = idx._queries(B)
        m = rows.shape[0]
        N.check(N.lib().ssg_closestpairs(idx._h, rows.ctypes.data_as(C.c_void_p), m, k, min_k, int(bool(samedata)),
                                         oi.ctypes.data_as(C.c_void_p), oj.ctypes.data_as(C.c_void_p),
                                         od.ctypes.data_as(C.c_void_p), C.byref(cnt)), idx._h)
    add_distance_evaluations(ctx, m * len(idx))
    c = int(cnt.value)
    return [(int(oi[r]), int(oj[r]), float(od[r])) for r in range(c)]


def bichromatic_closestpair(idx: GPUExhaustiveSearch, ctx: GenericContext, B, min_k: int = 8,
                            samedata: bool | None = None):
    """The closest pair (i, j, dist) (bichromatic_closestpair); (0, 0, inf)
    when there is none."""
    p = bichromatic_kclosestpairs(idx, ctx, B, k=1, min_k=max(1, min_k), samedata=samedata)
    return p[0] if p else (0, 0, float("inf"))


def closestpairs(idx: GPUExhaustiveSearch, ctx: GenericContext, k: int = 1, min_k: int | None = None):
    """closestpairs(idx, ctx; k, min_k): the k closest pairs among the indexed
    objects (src/bichromatic/closestpairs.jl)."""
    return bichromatic_kclosestpairs(idx, ctx, None, k=k, min_k=min_k, samedata=True)


def closestpair(idx: GPUExhaustiveSearch, ctx: GenericContext, min_k: int = 8):
    """closestpair(idx, ctx; min_k): (i, j, dist) of the closest pair among
    the indexed objects (src/bichromatic/closestpair.jl)."""
    p = closestpairs(idx, ctx, k=1, min_k=max(2, min_k))
    return p[0] if p else (0, 0, float("inf"))
