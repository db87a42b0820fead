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


class SubDatabase(AbstractDatabase):
    """Read-only view of ``parent`` objects ``map[1], map[2], ...`` (1-based
    ids), src/db/subdatabase.jl: what SearchGraph construction hands to
    ExhaustiveSearch for its gold standards (query samples, reference sets).
    Uploaded to the GPU as the gathered rows."""

    def __init__(self, parent, ids):
        self.parent = parent
        self.map = np.asarray(ids, dtype=np.int64).reshape(-1)
        if self.map.size and (self.map.min() < 1 or self.map.max() > len(parent)):
            raise IndexError("SubDatabase ids out of range")

    def __len__(self):
        return int(self.map.size)

    @property
    def dim(self):
        return self.parent.dim

    @property
    def dtype(self):
        return self.parent.dtype

    def __getitem__(self, i: int):
        if not 1 <= i <= len(self):
            raise IndexError(i)
        return self.parent[int(self.map[i - 1])]

    def rows(self) -> np.ndarray:
        return np.ascontiguousarray(self.parent.rows()[self.map - 1])


# MMapMatrixDatabase files (src/db/mmapmatrixdatabase.jl:10-27): a 4096-byte
# header -- magic UInt64 @0, version Int32 @8, dim Int64 @12, element type
# code Int32 @20, length n Int64 @24 -- then the column-major (dim, capacity)
# data, little-endian.
MMAP_MAGIC = 0x4D4D444231000001
MMAP_HEADER = 4096
_MMAP_CODES = {np.dtype(np.float16): 1, np.dtype(np.float32): 2, np.dtype(np.float64): 3, np.dtype(np.int8): 4,
               np.dtype(np.uint8): 5, np.dtype(np.int16): 6, np.dtype(np.uint16): 7, np.dtype(np.int32): 8,
               np.dtype(np.uint32): 9, np.dtype(np.int64): 10, np.dtype(np.uint64): 11}
_MMAP_TYPES = {v: k for k, v in _MMAP_CODES.items()}


def write_mmap_matrix(path, X, capacity: int | None = None):
    """Writes the ``(dim, n)`` matrix X as a MMapMatrixDatabase file (spare
    capacity columns are zero, as the reference preallocates)."""
    X = np.asarray(X)
    dim, n = X.shape
    cap = max(n, capacity or n)
    hdr = bytearray(MMAP_HEADER)
    hdr[0:8] = np.uint64(MMAP_MAGIC).tobytes()
    hdr[8:12] = np.int32(1).tobytes()
    hdr[12:20] = np.int64(dim).tobytes()
    hdr[20:24] = np.int32(_MMAP_CODES[X.dtype]).tobytes()
    hdr[24:32] = np.int64(n).tobytes()
    with open(path, "wb") as f:
        f.write(bytes(hdr))
        f.write(np.asfortranarray(X).tobytes(order="F"))
        f.write(bytes((cap - n) * dim * X.dtype.itemsize))


class MMapMatrixDatabase(MatrixDatabase):
    """Read-only view of a MMapMatrixDatabase file (the reference's reopen
    constructor, mmapmatrixdatabase.jl:151-175).  GPUExhaustiveSearch builds
    its device copy straight from the file (``ssg_create_mmap``)."""

    def __init__(self, path):
        self.path = str(path)
        with open(self.path, "rb") as f:
            hdr = f.read(32)
        if len(hdr) < 32 or int(np.frombuffer(hdr[0:8], "<u8")[0]) != MMAP_MAGIC:
            raise ValueError(f"{path} is not a MMapMatrixDatabase file (bad magic)")
        if int(np.frombuffer(hdr[8:12], "<i4")[0]) != 1:
            raise ValueError("unsupported MMapMatrixDatabase version")
        dim = int(np.frombuffer(hdr[12:20], "<i8")[0])
        code = int(np.frombuffer(hdr[20:24], "<i4")[0])
        n = int(np.frombuffer(hdr[24:32], "<i8")[0])
        if code not in _MMAP_TYPES:
            raise ValueError(f"unknown element type code {code}")
        dt = _MMAP_TYPES[code]
        mat = np.memmap(self.path, dtype=dt, mode="r", offset=MMAP_HEADER, shape=(dim, n), order="F") if n \
            else np.zeros((dim, 0), dtype=dt)
        super().__init__(mat)


def as_database(x) -> AbstractDatabase:
    if isinstance(x, AbstractDatabase):
        return x
    a = np.asarray(x)
    if a.ndim == 1:
        return MatrixDatabase(a.reshape(-1, 1))
    return MatrixDatabase(a)
