"""neardup on the GPU index (mirror of src/neardup.jl).

The reference builds an epsilon-net of X block by block (neardup_, :101-172):
each block of `blocksize` objects is searched against the net built so far;
an object within epsilon of its nearest net member is a near duplicate of it,
the others are filtered against each other in arrival order (neardup_block!,
:174-244: an object joins the net unless an already accepted object of the
block is within epsilon) and appended to the net.  Here the searches run on a
GPUExhaustiveSearch and the block's pairwise distances come from one GPU
search of the block against itself; the host only compares and bookkeeps.
"""
from __future__ import annotations

import numpy as np

from .db import MatrixDatabase, as_database
from .index import GenericContext, GPUExhaustiveSearch, append_items_b, searchbatch
from . import _native as N


def _block(idx, ctx, rows, imap, L, D, M, eps, filterblocks):
    if not filterblocks:
        keep = list(imap)
    else:
        # pairwise distances of the block's objects (GPU), then the reference's
        # arrival-order filter: object i joins unless its nearest accepted
        # object (smallest distance, then id) is within eps
        B = rows[imap]
        sub = GPUExhaustiveSearch(idx.dist, MatrixDatabase.from_rows(B))
        ids, dists = searchbatch(sub, GenericContext(logger=None), MatrixDatabase.from_rows(B), len(imap))
        pos = np.empty((len(imap), len(imap)), dtype=np.float32)
        for q in range(len(imap)):
            pos[q, ids[:, q].astype(np.int64) - 1] = dists[:, q]
        sub.close()
        keep = [imap[0]]
        kept_pos = [0]
        for ii in range(1, len(imap)):
            d = pos[ii, kept_pos]
            best = int(np.argmin(d))          # first minimum: the earliest accepted object
            if d[best] > eps:
                keep.append(imap[ii])
                kept_pos.append(ii)
            else:
                L[imap[ii]] = imap[kept_pos[best]] + 1
                D[imap[ii]] = d[best]
    for i in keep:
        M.append(i + 1)
        L[i] = i + 1
        D[i] = 0.0
    append_items_b(idx, ctx, MatrixDatabase.from_rows(rows[keep]))


def neardup(idx: GPUExhaustiveSearch, ctx: GenericContext, X, eps: float, k: int = 8, blocksize: int = 256,
            filterblocks: bool = True, verbose: bool = False):
    """neardup(idx, ctx, X, eps; k, blocksize, filterblocks) with an empty
    GPU index: returns a dict with ``idx``, ``map`` (net position -> 1-based id
    of X), ``nn`` (each object's covering object, 1-based), ``dist``,
    ``centers`` (sorted ids of the net) and ``costdists``."""
    if len(idx) != 0:
        raise N.ArgumentError("neardup needs an empty index")
    rows = as_database(X).rows()
    n = rows.shape[0]
    eps = np.float32(eps)
    L = np.zeros(n, dtype=np.int32)
    D = np.zeros(n, dtype=np.float32)
    M: list[int] = []
    before = sum(ctx.costdists)
    blocksize = max(1, min(blocksize, n))
    for start in range(0, n, blocksize):
        rng = list(range(start, min(n, start + blocksize)))
        if len(idx) == 0:
            _block(idx, ctx, rows, rng, L, D, M, eps, filterblocks)
            continue
        ids, dists = searchbatch(idx, ctx, MatrixDatabase.from_rows(rows[rng]), min(k, len(idx)))
        imap = []
        for i, j in enumerate(rng):
            pid, pd = int(ids[0, i]), dists[0, i]
            if pd > eps:
                imap.append(j)
            else:
                D[j] = pd
                L[j] = M[pid - 1]
        if imap:
            _block(idx, ctx, rows, imap, L, D, M, eps, filterblocks)
    return {"idx": idx, "map": np.array(M, dtype=np.uint32), "nn": L, "dist": D,
            "centers": np.array(sorted(set(L.tolist())), dtype=np.int32),
            "costdists": sum(ctx.costdists) - before}
