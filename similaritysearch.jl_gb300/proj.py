"""Bit sketches on the GPU: the producer of the sketches the Hamming scan
searches (mirror of ``bitsketch(R, X)``, src/proj/bitsketches.jl:101-104).

``R`` has the reference's shape ``(indim, outdim)`` (column c is projection
vector c, ``transform`` computes ``R' * x``, src/proj/Projections.jl:137-143);
``X`` is a vector of ``indim`` or a ``(indim, n)`` matrix / database (one
object per column).  Bit c of a sketch is 1 iff coordinate c is >= 0
(``packsigns``, bitsketches.jl:19-32); 64 coordinates per UInt64 word.
Everything runs in libssgpu.so (``ssg_bitsketch``); device staging goes
through torch tensors.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .db import as_database


def bitsketch(R, X):
    """Vector -> ``(ceil(outdim/64),)`` UInt64; matrix -> ``(ceil(outdim/64), n)``."""
    import torch
    R = np.asarray(R)
    if R.ndim != 2 or R.shape[0] == 0 or R.shape[1] == 0:
        raise N.ArgumentError("R must be an (indim, outdim) matrix")
    indim, outdim = R.shape
    vector = isinstance(X, np.ndarray) and X.ndim == 1
    rows = np.asarray(X, dtype=np.float32)[None, :] if vector else as_database(X).rows()
    if rows.ndim != 2 or (rows.shape[0] and rows.shape[1] != indim):
        raise N.ArgumentError(f"objects have dimension {rows.shape[-1]}, R has {indim}")
    n = rows.shape[0]
    words = (outdim + 63) // 64
    out = np.zeros((n, words), dtype=np.uint64)
    if n:
        dR = torch.from_numpy(np.ascontiguousarray(R.T, dtype=np.float32)).cuda()
        dX = torch.from_numpy(np.ascontiguousarray(rows, dtype=np.float32)).cuda()
        dO = torch.empty((n, words), dtype=torch.int64, device="cuda")
        N.check(N.lib().ssg_bitsketch(C.c_void_p(dR.data_ptr()), indim, outdim, C.c_void_p(dX.data_ptr()), n,
                                      C.c_void_p(dO.data_ptr()), None))
        out = dO.cpu().numpy().view(np.uint64)
    return out[0] if vector else np.asfortranarray(out.T)
