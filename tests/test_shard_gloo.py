"""World-size-2 tests of the sharded path's host logic on CPU (gloo): the
shard partition, the (distance, id) merge of per-shard lists, the all-gather
exchange, and the max-over-ranks timing reduction.  The per-shard search is
the oracle (no GPU), so the merged result must equal the oracle's search over
the whole database -- ties across the shard boundary included."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from conftest import load_package


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, X, Q, k, name, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import sys
        sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
        from oracle import oracle as O
        S = load_package().shard
        lo, hi = S.shard_bounds(X.shape[0], world, rank)
        ids, dists = S.sharded_searchbatch(lambda q, kk: O.searchbatch(name, X[lo:hi], q, kk), Q, k, X.shape[0])
        slowest = S.max_over_ranks(10.0 + rank)
        out[rank] = (ids, dists, slowest)
    finally:
        dist.destroy_process_group()


def _run(world, X, Q, k, name):
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, world, port, X, Q, k, name, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
        assert all(p.exitcode == 0 for p in procs)
        return [out[r] for r in range(world)]


def test_shard_bounds_partition():
    S = load_package().shard
    for n in (0, 1, 7, 100, 101):
        for world in (1, 2, 3, 8):
            spans = [S.shard_bounds(n, world, r) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [h - l for l, h in spans]
            assert max(sizes) - min(sizes) <= 1 and sizes == sorted(sizes, reverse=True)
    with pytest.raises(ValueError):
        S.shard_bounds(10, 2, 2)


def test_merge_topk_orders_by_distance_then_id():
    S = load_package().shard
    a_i = np.array([[3, 1, 0]], np.uint32); a_d = np.array([[0.5, 0.5, np.inf]], np.float32)
    b_i = np.array([[7, 2]], np.uint32);    b_d = np.array([[0.25, 0.5]], np.float32)
    ids, d = S.merge_topk([a_i, b_i], [a_d, b_d], 4)
    assert ids.tolist() == [[7, 1, 2, 3]] and d.tolist() == [[0.25, 0.5, 0.5, 0.5]]
    ids, d = S.merge_topk([a_i[:, 2:]], [a_d[:, 2:]], 2)        # only empty slots
    assert ids.tolist() == [[0, 0]] and np.all(np.isinf(d))


@pytest.mark.parametrize("name", ["sql2", "normcosine"])
def test_sharded_search_world2_equals_whole_database(name):
    from oracle import oracle as O
    rng = np.random.default_rng(5)
    X = rng.standard_normal((301, 12)).astype(np.float32)
    X[150:160] = X[140]                 # equal rows straddling the shard boundary
    if name == "normcosine":
        X /= np.linalg.norm(X, axis=1, keepdims=True)
    Q = np.concatenate([X[[140, 3]], rng.standard_normal((6, 12)).astype(np.float32)])
    res = _run(2, X, Q, 15, name)
    ri, rd = O.searchbatch(name, X, Q, 15)
    for ids, dists, slowest in res:
        assert np.array_equal(ids, ri) and np.array_equal(dists, rd)
        assert slowest == 11.0
