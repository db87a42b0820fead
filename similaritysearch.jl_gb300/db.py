"""Database containers (mirror of src/db/matrixdatabase.jl and vectordatabase.jl).

Shapes follow Julia: ``MatrixDatabase(X)`` takes a ``(dim, n)`` matrix whose
column ``i`` is object ``i``; indexing is 1-based like the reference
(``db[1]`` is the first object).  A Fortran-ordered ``(dim, n)`` numpy array
has exactly the bytes of the Julia matrix (n rows of dim elements), so it is
handed to the GPU without a copy; other layouts are packed once.
"""
from __future__ import annotations

import numpy as np


class AbstractDatabase:
    def rows(self) -> np.ndarray:
        """C-contiguous ``(n, dim)`` view/copy: the bytes the C ABI expects."""
        raise NotImplementedError

    def __iter__(self):
        for i in range(1, len(self) + 1):
            yield self[i]


class MatrixDatabase(AbstractDatabase):
    """Fixed-size database over a ``(dim, n)`` matrix (matrixdatabase.jl:27-59)."""

    def __init__(self, matrix):
        m = np.asarray(matrix)
        if m.ndim != 2:
            raise ValueError("MatrixDatabase needs a (dim, n) matrix")
        self.matrix = m

    @classmethod
    def from_rows(cls, rows):
        """Builds the database from an ``(n, dim)`` row-major array (no copy)."""
        r = np.ascontiguousarray(rows)
        return cls(r.T)

    def __len__(self):
        return self.matrix.shape[1]

    @property
    def dim(self):
        return self.matrix.shape[0]

    @property
    def dtype(self):
        return self.matrix.dtype

    def __getitem__(self, i: int):
        # db[i] = view(matrix, :, i)  (matrixdatabase.jl:40-41), 1-based
        if not 1 <= i <= len(self):
            raise IndexError(i)
        return self.matrix[:, i - 1]

    def rows(self) -> np.ndarray:
        return np.ascontiguousarray(self.matrix.T)

    def push_item(self, v):
        raise TypeError("push! is not supported for MatrixDatabase (matrixdatabase.jl:49)")

    def append_items(self, other):
        raise TypeError("append! is not supported for MatrixDatabase (matrixdatabase.jl:57)")


class VectorDatabase(AbstractDatabase):
    """Growable database of equal-length vectors (vectordatabase.jl:30-104).
    It is packed into a contiguous staging matrix when uploaded."""

    def __init__(self, vectors=None):
        self.vecs = [np.asarray(v) for v in (vectors or [])]

    def __len__(self):
        return len(self.vecs)

    @property
    def dim(self):
        return int(self.vecs[0].shape[0]) if self.vecs else 0

    @property
    def dtype(self):
        return self.vecs[0].dtype if self.vecs else np.dtype(np.float32)

    def __getitem__(self, i: int):
        if not 1 <= i <= len(self):
            raise IndexError(i)
        return self.vecs[i - 1]

    def rows(self) -> np.ndarray:
        if not self.vecs:
            return np.zeros((0, 0), dtype=np.float32)
        return np.ascontiguousarray(np.stack(self.vecs, axis=0))

    def push_item(self, v):
        self.vecs.append(np.asarray(v))

    def append_items(self, other):
        for v in other:
            self.push_item(v)


def as_database(x) -> AbstractDatabase:
    if isinstance(x, AbstractDatabase):
        return x
    a = np.asarray(x)
    if a.ndim == 1:
        return MatrixDatabase(a.reshape(-1, 1))
    return MatrixDatabase(a)
