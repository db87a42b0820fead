"""The no-allocation entry point, ssg_knn_noalloc, through the C ABI.

It serves callers that cannot call cudaMalloc (their own allocator owns the
GPU's memory, or their request path must not allocate because cudaMalloc can
synchronise the device): they pass device buffers they own and the search
uses a fixed scratch array compiled into the library.  Its results must equal
those of the existing device entry point (ssg_search_device on an index over
the same data) exactly -- the tolerance every plain-method test here uses --
on two calls in a row, since the second call reuses the array the first one
left filled.  This file is collected last so that, if it fails, a run that
stops at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_package
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    ss = load_package()
    ss.build()
    return ss, torch


def reference_search(ss, torch, metric, elem, X, Q, k):
    """Results of the existing entry point: ssg_create + ssg_search_device."""
    N = ss._native
    L = N.lib()
    h = C.c_void_p()
    N.check(L.ssg_create(metric, elem, X.shape[1], X.shape[0], X.ctypes.data_as(C.c_void_p), X.shape[1], 0,
                         C.byref(h)))
    try:
        dq = torch.from_numpy(Q).cuda()
        ids = torch.empty((Q.shape[0], k), dtype=torch.int32, device="cuda")
        dists = torch.empty((Q.shape[0], k), dtype=torch.float32, device="cuda")
        N.check(L.ssg_search_device(h, C.c_void_p(dq.data_ptr()), Q.shape[0], k, C.c_void_p(ids.data_ptr()),
                                    C.c_void_p(dists.data_ptr()), 0), h)
        torch.cuda.synchronize()
        return ids.cpu().numpy().view(np.uint32), dists.cpu().numpy()
    finally:
        L.ssg_destroy(h)


def noalloc_search(ss, torch, metric, dX, dQ, dim, n, m, k):
    N = ss._native
    ids = torch.full((m, k), -1, dtype=torch.int32, device="cuda")
    dists = torch.full((m, k), -1.0, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    rc = N.lib().ssg_knn_noalloc(metric, C.c_void_p(dX.data_ptr()), dim, n, C.c_void_p(dQ.data_ptr()), m, k,
                                 C.c_void_p(ids.data_ptr()), C.c_void_p(dists.data_ptr()),
                                 C.c_void_p(stream.cuda_stream))
    N.check(rc)
    torch.cuda.synchronize()
    return ids.cpu().numpy().view(np.uint32), dists.cpu().numpy()


@pytest.mark.parametrize("metric_name", ["SQL2", "L2", "NORMCOSINE", "IP"])
def test_noalloc_equals_search_device_twice(env, metric_name):
    ss, torch = env
    N = ss._native
    metric = getattr(N, "METRIC_" + metric_name)
    rng = np.random.default_rng(31)
    X = rng.standard_normal((6000, 40), dtype=np.float32)
    Q1 = rng.standard_normal((300, 40), dtype=np.float32)
    Q2 = rng.standard_normal((77, 40), dtype=np.float32)
    dX = torch.from_numpy(X).cuda()
    # two calls in a row: different batch sizes and k, the second reuses the
    # scratch array the first left behind
    for Q, k in ((Q1, 10), (Q2, 25)):
        ri, rd = reference_search(ss, torch, metric, N.ELEM_F32, X, Q, k)
        dQ = torch.from_numpy(Q).cuda()
        gi, gd = noalloc_search(ss, torch, metric, dX, dQ, 40, X.shape[0], Q.shape[0], k)
        assert np.array_equal(gi, ri)
        assert np.array_equal(gd, rd)
        # and directly against the oracle's sequential (lanes=1) restatement
        oi, od = O.searchbatch(metric_name.lower(), X, Q, k, lanes=1)
        assert np.array_equal(gi, oi)
        assert np.array_equal(gd, od)


def test_noalloc_hamming_twice(env):
    ss, torch = env
    N = ss._native
    rng = np.random.default_rng(32)
    X = rng.integers(0, 2**64 - 1, size=(20000, 16), dtype=np.uint64, endpoint=True)
    dX = torch.from_numpy(X.view(np.int64)).cuda()
    for m, k in ((200, 100), (33, 7)):
        Q = X[rng.integers(0, 20000, size=m)] ^ np.uint64(0x00FF00FF)
        ri, rd = reference_search(ss, torch, N.METRIC_HAMMING, N.ELEM_U64, X, Q, k)
        dQ = torch.from_numpy(Q.view(np.int64)).cuda()
        gi, gd = noalloc_search(ss, torch, N.METRIC_HAMMING, dX, dQ, 16, X.shape[0], m, k)
        assert np.array_equal(gi, ri)
        assert np.array_equal(gd, rd)


def test_noalloc_rejects_requests_beyond_the_fixed_scratch(env):
    ss, torch = env
    N = ss._native
    dX = torch.zeros((3000, 8), dtype=torch.float32, device="cuda")
    dQ = torch.zeros((30000, 8), dtype=torch.float32, device="cuda")
    ids = torch.empty((30000, 100), dtype=torch.int32, device="cuda")
    dists = torch.empty((30000, 100), dtype=torch.float32, device="cuda")
    rc = N.lib().ssg_knn_noalloc(N.METRIC_SQL2, C.c_void_p(dX.data_ptr()), 8, 3000, C.c_void_p(dQ.data_ptr()),
                                 30000, 100, C.c_void_p(ids.data_ptr()), C.c_void_p(dists.data_ptr()), None)
    assert rc == N.SSG_EINVAL
    assert "scratch" in N.last_error(None)
    rc = N.lib().ssg_knn_noalloc(N.METRIC_COSINE, C.c_void_p(dX.data_ptr()), 8, 3000, C.c_void_p(dQ.data_ptr()),
                                 10, 5, C.c_void_p(ids.data_ptr()), C.c_void_p(dists.data_ptr()), None)
    assert rc == N.SSG_EUNSUPPORTED


def test_noalloc_scratch_caps_the_splits(env):
    """m * min(k, n) just below the 2,097,152-key scratch: the database would
    be split four ways to fill the GPU, but only one split's keys fit, so the
    scan runs unsplit; results still equal ssg_search_device's, twice."""
    ss, torch = env
    N = ss._native
    rng = np.random.default_rng(33)
    n, m, k, d = 200_000, 20_000, 100, 16
    X = rng.standard_normal((n, d), dtype=np.float32)
    Q = rng.standard_normal((m, d), dtype=np.float32)
    assert m * k <= 2_097_152 < 2 * m * k
    ri, rd = reference_search(ss, torch, N.METRIC_SQL2, N.ELEM_F32, X, Q, k)
    dX = torch.from_numpy(X).cuda()
    dQ = torch.from_numpy(Q).cuda()
    for _ in range(2):
        gi, gd = noalloc_search(ss, torch, N.METRIC_SQL2, dX, dQ, d, n, m, k)
        assert np.array_equal(gi, ri)
        assert np.array_equal(gd, rd)


def test_noalloc_refuses_misaligned_buffers(env):
    """Buffers not aligned to their element are refused on the host (no
    kernel runs), instead of faulting on the GPU."""
    ss, torch = env
    N = ss._native
    L = N.lib()
    dX = torch.zeros((1024, 8), dtype=torch.int64, device="cuda")
    dQ = torch.zeros((4, 8), dtype=torch.int64, device="cuda")
    ids = torch.empty((4, 5), dtype=torch.int32, device="cuda")
    dists = torch.empty((4, 5), dtype=torch.float32, device="cuda")
    p = lambda t, off=0: C.c_void_p(t.data_ptr() + off)
    rc = L.ssg_knn_noalloc(N.METRIC_HAMMING, p(dX, 4), 8, 1000, p(dQ), 4, 5, p(ids), p(dists), None)
    assert rc == N.SSG_EINVAL and "aligned" in N.last_error(None)
    rc = L.ssg_knn_noalloc(N.METRIC_SQL2, p(dX), 8, 1000, p(dQ, 2), 4, 5, p(ids), p(dists), None)
    assert rc == N.SSG_EINVAL and "aligned" in N.last_error(None)
    rc = L.ssg_knn_noalloc(N.METRIC_SQL2, p(dX), 8, 1000, p(dQ), 4, 5, p(ids, 1), p(dists), None)
    assert rc == N.SSG_EINVAL and "aligned" in N.last_error(None)
